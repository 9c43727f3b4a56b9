"""The learned warm start's tensor-core kernels (tcgen05, BF16 in / FP32 accumulate).

First the GEMM building blocks in the three operand arrangements the network uses
(forward: both operands K-major; activation gradient: MN-major weights; weight
gradient: both MN-major), against float64 products of the same BF16 values."""
import ctypes as C

import numpy as np
import pytest

from nesf import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2])
def test_tcgen05_gemm_layouts(which):
    import torch
    lib = _lib.load()
    g = torch.Generator(device="cpu").manual_seed(11 + which)
    shapes = {0: ((128, 64), (64, 64)), 1: ((128, 64), (64, 64)), 2: ((128, 128), (128, 16))}
    sa, sb = shapes[which]
    a = torch.randn(sa, generator=g).to(torch.bfloat16)
    b = torch.randn(sb, generator=g).to(torch.bfloat16)
    A, B = a.double(), b.double()
    ref = {0: lambda: A @ B.T, 1: lambda: A @ B, 2: lambda: A.T @ B}[which]()
    d = torch.zeros(ref.shape, dtype=torch.float32, device="cuda")
    da, db = a.cuda(), b.cuda()            # held: the kernel reads them
    code = lib.nesf_mlp_selftest(C.c_void_p(da.data_ptr()), C.c_void_p(db.data_ptr()), C.c_void_p(d.data_ptr()),
                                 which, None)
    assert code == 0, lib.nesf_last_error()
    got = d.cpu().double()
    err = (got - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, (which, err)


def test_tcgen05_wait_timeout_is_reported_and_the_context_survives():
    """The failure path of the tensor-core kernels' bounded mbarrier waits, without a
    fault: in self-test mode 3 no MMA is issued and nothing arrives on the barrier, so
    the wait gives up after a short limit; the kernel records the error, frees its TMEM
    and returns, the call reports NESF_ERR_TIMEOUT, and a GEMM afterwards on the same
    context is still correct."""
    import torch
    from nesf import _abi as A
    lib = _lib.load()
    a = torch.zeros((128, 64), dtype=torch.bfloat16, device="cuda")
    b = torch.zeros((64, 64), dtype=torch.bfloat16, device="cuda")
    d = torch.full((128, 64), 7.0, dtype=torch.float32, device="cuda")
    code = lib.nesf_mlp_selftest(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), C.c_void_p(d.data_ptr()), 3,
                                 None)
    assert code == A.NESF_ERR_TIMEOUT, (code, lib.nesf_last_error())
    assert b"did not complete" in lib.nesf_last_error()
    assert torch.all(d == 7.0)          # no result was read out of TMEM
    torch.cuda.synchronize()            # the context is intact
    test_tcgen05_gemm_layouts(0)


def _samples(rng, n):
    """Features in the ranges the solver produces and targets with masks."""
    x = np.zeros((n, 8), np.float32)
    x[:, 0] = rng.uniform(-3, 3, n)            # bulk Richardson number
    x[:, 1] = rng.uniform(0.5, 30, n)          # dU
    x[:, 2] = rng.normal(0, 4, n)              # dtheta_0
    x[:, 3] = rng.normal(-2, 2, n)             # dq_0 (g/kg)
    x[:, 4] = np.log(10.0)
    x[:, 5] = rng.uniform(-11, -6, n)          # ln z0
    x[:, 6] = x[:, 1]
    t = np.zeros((n, 4), np.float32)
    t[:, 0] = 0.035 + 0.01 * np.tanh(x[:, 0]) + 1e-4 * x[:, 1]
    t[:, 1] = 0.03 + 0.01 * np.tanh(-x[:, 0])
    t[:, 2] = 0.031 + 0.01 * np.tanh(-x[:, 0]) + 0.001 * x[:, 5] / 10
    t[:, 3] = rng.choice([1, 3, 7, 5], n)
    return x, t


def test_network_gradient_matches_cpu_checker():
    """Forward + backward on the tensor cores (BF16 operands, FP32 accumulation) against the
    CPU restatement with the same BF16 roundings: gradients of every weight and bias, the loss
    and the outputs, on 300 samples (two full tiles and a ragged one)."""
    import torch
    from nesf.warm import WarmStartNetwork
    from oracle import mlp_reference as R
    rng = np.random.default_rng(5)
    x, t = _samples(rng, 300)
    net = WarmStartNetwork(seed=3)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    net.fit_normalization(dx, dt)
    p = net.parameters()
    assert abs(p["in_mu"][1] - x[:, 1].mean()) < 1e-3 * abs(x[:, 1].mean())
    net.gradient(dx, dt)
    g = net.gradients()
    assert g["error"] == 0
    ref_out, ref_loss, ref = R.forward_backward(p, x.astype(np.float64), t.astype(np.float64))
    assert abs(g["loss"][0] - ref_loss) <= 1e-4 * ref_loss, (g["loss"], ref_loss)
    assert g["loss"][1] == 300
    blocks = {"w1": (slice(None), slice(0, R.IN)), "b1": (slice(None),), "w2": (slice(None), slice(None)),
              "b2": (slice(None),), "w3": (slice(0, R.OUT), slice(None)), "b3": (slice(0, R.OUT),)}
    for k, sl in blocks.items():
        a, b = g[k][sl], ref[k][sl]
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err < 2e-3, (k, err)
    out = net.infer(dx).cpu().numpy()
    assert np.all(out[:, 3] == 1.0)
    err = np.abs(out[:, :3] - ref_out).max() / np.abs(ref_out).max()
    assert err < 2e-3, err


def test_network_training_fits_a_smooth_target():
    import torch
    from nesf.warm import WarmStartNetwork
    rng = np.random.default_rng(6)
    x, t = _samples(rng, 32768)
    net = WarmStartNetwork(seed=1)
    dx, dt = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    net.fit_normalization(dx, dt)
    losses = net.train(dx, dt, epochs=12, batch=1024, lr=3e-3)
    assert losses[-1] < 0.05 * losses[0], losses
    out = net.infer(dx).cpu().numpy()
    rel = np.abs(out[:, 0] - t[:, 0]) / t[:, 0]
    assert np.median(rel) < 0.01, np.median(rel)
