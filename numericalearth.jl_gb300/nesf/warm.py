"""The learned warm start: a 6 -> 64 -> 64 -> 3 GELU network that predicts a cell's
transfer coefficients c_u = u*/dU, c_theta = theta*/dtheta_0, c_q = q*/dq_0 from its
state before the iteration, trained and evaluated by the library's tcgen05 kernels
(include/nesf.h, nesf_mlp_*). The solvers start their FP32 iteration from the
network's guess and run to the same tolerance; a guess whose first residual exceeds
`fallback_ratio` times the cold start's is dropped for the reference's start.

Training data are solver-generated: synthetic surface states drawn over the range
the network must cover, solved by the plain FP64 solver, turned into (features,
targets) by nesf_mlp_ao_samples.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from . import fields as F
from ._lib import check, load


def _torch():
    import torch
    return torch


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class WarmStartNetwork:
    """The network's device blob (FP32 parameters, BF16 copies, gradient, Adam moments)."""

    def __init__(self, seed=0, device="cuda"):
        torch = _torch()
        self.lib = load()
        n = self.lib.nesf_mlp_bytes()
        assert n == C.sizeof(A.MlpBlob), (n, C.sizeof(A.MlpBlob))
        self.blob = torch.zeros(n, dtype=torch.uint8, device=device)
        check(self.lib.nesf_mlp_init(self.ptr, int(seed), _stream(None)))

    @property
    def ptr(self):
        return C.c_void_p(self.blob.data_ptr())

    def fit_normalization(self, features, targets, stream=None):
        check(self.lib.nesf_mlp_fit_normalization(self.ptr, C.c_void_p(features.data_ptr()),
                                                  C.c_void_p(targets.data_ptr()), features.shape[0],
                                                  _stream(stream)))

    def gradient(self, features, targets, stream=None):
        """Add the gradient of the mean loss over the samples to the blob's gradient."""
        check(self.lib.nesf_mlp_gradient(self.ptr, C.c_void_p(features.data_ptr()), C.c_void_p(targets.data_ptr()),
                                         features.shape[0], _stream(stream)))

    def train(self, features, targets, epochs=10, batch=4096, lr=2e-3, betas=(0.9, 0.999), eps=1e-8,
              stream=None):
        """Mini-batch Adam; returns the mean loss of each epoch."""
        o = A.MlpTrainOptions(int(epochs), int(batch), float(lr), float(betas[0]), float(betas[1]), float(eps))
        loss = (C.c_float * int(epochs))()
        check(self.lib.nesf_mlp_train(self.ptr, C.c_void_p(features.data_ptr()), C.c_void_p(targets.data_ptr()),
                                      features.shape[0], C.byref(o), loss, _stream(stream)))
        return list(loss)

    def infer(self, features, stream=None):
        """(n, 4) outputs: c_u, c_theta, c_q, 1."""
        torch = _torch()
        out = torch.zeros((features.shape[0], 4), dtype=torch.float32, device=features.device)
        check(self.lib.nesf_mlp_infer(self.ptr, C.c_void_p(features.data_ptr()), features.shape[0],
                                      C.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def host(self):
        """A host copy of the blob (ctypes MlpBlob)."""
        _torch().cuda.synchronize()
        return A.MlpBlob.from_buffer_copy(self.blob.cpu().numpy().tobytes())

    def parameters(self):
        b = self.host()
        p = np.array(b.p, dtype=np.float64)
        return {"w1": p[A.MLP_W1:A.MLP_B1].reshape(A.MLP_HID, A.MLP_IN_PAD), "b1": p[A.MLP_B1:A.MLP_W2],
                "w2": p[A.MLP_W2:A.MLP_B2].reshape(A.MLP_HID, A.MLP_HID), "b2": p[A.MLP_B2:A.MLP_W3],
                "w3": p[A.MLP_W3:A.MLP_B3].reshape(A.MLP_OUT_PAD, A.MLP_HID), "b3": p[A.MLP_B3:],
                "in_mu": np.array(b.in_mu), "in_sig": np.array(b.in_sig), "out_mu": np.array(b.out_mu),
                "out_sig": np.array(b.out_sig)}

    def gradients(self):
        b = self.host()
        g = np.array(b.g, dtype=np.float64)
        return {"w1": g[A.MLP_W1:A.MLP_B1].reshape(A.MLP_HID, A.MLP_IN_PAD), "b1": g[A.MLP_B1:A.MLP_W2],
                "w2": g[A.MLP_W2:A.MLP_B2].reshape(A.MLP_HID, A.MLP_HID), "b2": g[A.MLP_B2:A.MLP_W3],
                "w3": g[A.MLP_W3:A.MLP_B3].reshape(A.MLP_OUT_PAD, A.MLP_HID), "b3": g[A.MLP_B3:],
                "loss": np.array(b.loss[:2], dtype=np.float64), "error": b.error}


def ao_samples(spec, layout, state, solved, stream=None):
    """(features, targets) of every halo-ring cell of an atmosphere-ocean state whose solved
    u*, theta*, q* are in `solved` (device tensors in the state's layout)."""
    torch = _torch()
    lib = load()
    arrays = {k: state.get(k) for k in F.AO_INPUTS}
    arrays.update({k: solved.get(k) for k in F.AO_OUTPUTS})
    f = F.pack(A.AOFields, F.make_grid(layout), arrays)
    p = spec.to_c() if hasattr(spec, "to_c") else spec
    ring = (layout.nx + 2) * (layout.ny + 2)
    dev = state["u_atm"].device
    feat = torch.zeros((ring, 8), dtype=torch.float32, device=dev)
    targ = torch.zeros((ring, 4), dtype=torch.float32, device=dev)
    check(lib.nesf_mlp_ao_samples(C.byref(p), C.byref(f), C.c_void_p(feat.data_ptr()), C.c_void_p(targ.data_ptr()),
                                  _stream(stream)))
    return feat, targ


def training_set(spec, states, stream=None, shuffle_seed=None):
    """Solver-generated samples: each synthetic state solved by the plain FP64 solver, then
    its (features, targets) pairs with a valid u* target, concatenated. `states` may be a
    generator (each state's host arrays are dropped once its samples are on the device).
    With `shuffle_seed` the samples are put in a seeded random order, so that contiguous
    mini-batches mix cells of every state."""
    torch = _torch()
    from . import api
    feats, targs = [], []
    for st in states:
        dev = api.to_device({k: st.fields.get(k) for k in F.AO_INPUTS if k in st.fields})
        fdt = dev["u_atm"].dtype
        out = {k: torch.zeros(st.layout.shape, dtype=fdt, device="cuda") for k in F.AO_OUTPUTS}
        api.compute_atmosphere_ocean_fluxes(spec, st.layout, dev, out, precision="f64", stream=stream)
        f, t = ao_samples(spec, st.layout, dev, out, stream=stream)
        keep = (t[:, 3].to(torch.int32) & 1) != 0
        feats.append(f[keep])
        targs.append(t[keep])
        del dev, out, f, t
    x, t = torch.cat(feats), torch.cat(targs)
    if shuffle_seed is not None:
        g = torch.Generator(device=x.device)
        g.manual_seed(int(shuffle_seed))
        order = torch.randperm(x.shape[0], generator=g, device=x.device)
        x, t = x[order], t[order]
    return x.contiguous(), t.contiguous()
