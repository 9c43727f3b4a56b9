"""CPU restatement of the warm-start network's forward and backward passes.

TEST INFRASTRUCTURE ONLY: the checker of the tensor-core kernels of
numericalearth.jl_gb300/csrc/nesf_mlp.cu (tests/ call it; the product never does).
The network is the one the library defines (6 -> 64 -> 64 -> 3, GELU in its tanh
form, features and targets normalised by stored means and deviations, mean over
the samples of the squared error of the normalised targets that the mask keeps).
With `emulate_bf16` the operands of every product are rounded to BF16 as the
tensor cores receive them (FP64 accumulation stands in for the kernels' FP32);
without it everything is FP64, which the finite-difference check uses.
"""
import numpy as np

IN, IN_PAD, HID, OUT, OUT_PAD = 6, 16, 64, 3, 16
K_GELU = np.sqrt(2.0 / np.pi)


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(K_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(K_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * K_GELU * (1.0 + 3.0 * 0.044715 * x * x)


def forward_backward(p, features, targets=None, emulate_bf16=True):
    """p: dict w1 (64x16), b1, w2 (64x64), b2, w3 (16x64), b3, in_mu, in_sig, out_mu, out_sig.
    Returns (outputs (n, 3) de-normalised, loss sum, gradients dict or None)."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    n = features.shape[0]
    X = np.zeros((n, IN_PAD))
    xn = (features[:, :IN].astype(np.float32) - np.float32(1) * p["in_mu"][:IN].astype(np.float32)) \
        / p["in_sig"][:IN].astype(np.float32)
    X[:, :IN] = xn
    Xb, W1, W2, W3 = r(X), r(p["w1"]), r(p["w2"]), r(p["w3"])
    Z1 = Xb @ W1.T + p["b1"]
    H1 = r(gelu(Z1))
    Z2 = H1 @ W2.T + p["b2"]
    H2 = r(gelu(Z2))
    Y = H2 @ W3.T + p["b3"]
    out = Y[:, :OUT] * p["out_sig"][:OUT] + p["out_mu"][:OUT]
    if targets is None:
        return out, None, None
    mask = targets[:, 3].astype(np.int64)
    m = np.stack([(mask >> k) & 1 for k in range(OUT)], axis=1).astype(np.float64)
    tn = (targets[:, :OUT] - p["out_mu"][:OUT]) / p["out_sig"][:OUT]
    E = m * (Y[:, :OUT] - tn)
    loss = float((E * E).sum())
    dY = np.zeros((n, OUT_PAD))
    dY[:, :OUT] = 2.0 * E / n
    dYb = r(dY)
    dZ2 = (dYb @ W3) * gelu_grad(Z2)
    dZ2b = r(dZ2)
    dZ1 = (dZ2b @ W2) * gelu_grad(Z1)
    dZ1b = r(dZ1)
    g = {"w3": dYb.T @ H2, "w2": dZ2b.T @ H1, "w1": dZ1b.T @ Xb, "b3": dY.sum(0), "b2": dZ2.sum(0),
         "b1": dZ1.sum(0)}
    return out, loss, g


def mean_loss(p, features, targets):
    _, loss, _ = forward_backward(p, features, targets, emulate_bf16=False)
    return loss / features.shape[0]
