"""The double-float arithmetic of the adaptive solver's replays (nesf_double_float_check)
against FP64 on the host: the arguments rounded to double-float (48 significant bits),
each operation's result within a few units of 2^-48 for + - * / sqrt and within 1e-13
relative for cbrt, exp, log, pow and atan, over the ranges the interface solves produce
and beyond (wind speeds, temperatures and their differences, the scales u*, theta*, q*,
roughness lengths, Obukhov-length ratios), within FP32's exponent range: a low part
below ~1.2e-38 is flushed to zero, so values are kept above ~1e-30."""
import ctypes as C

import numpy as np
import pytest

from nesf import _abi as A
from nesf import _lib

pytestmark = pytest.mark.gpu

OPS = {"add": 0, "sub": 1, "mul": 2, "div": 3, "sqrt": 4, "cbrt": 5, "exp": 6, "log": 7, "pow": 8, "atan": 9}


def df_round(x):
    """x rounded to double-float: hi = fl32(x), lo = fl32(x - hi)."""
    hi = x.astype(np.float32).astype(np.float64)
    return hi + (x - hi).astype(np.float32).astype(np.float64)


def run(op, x, y=None):
    import torch
    lib = _lib.load()
    dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    dy = torch.from_numpy(np.ascontiguousarray(y)).cuda() if y is not None else None
    out = torch.zeros_like(dx)
    code = lib.nesf_double_float_check(C.c_void_p(dx.data_ptr()), C.c_void_p(dy.data_ptr()) if dy is not None else None,
                                       C.c_void_p(out.data_ptr()), x.size, OPS[op], None)
    assert code == A.NESF_OK, _lib.load().nesf_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def rel(got, ref):
    return np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)


def signed_logspace(rng, lo, hi, n):
    return rng.choice([-1.0, 1.0], n) * np.exp(rng.uniform(np.log(lo), np.log(hi), n))


@pytest.fixture(scope="module")
def rng():
    return np.random.default_rng(2024)


def test_arithmetic(rng):
    n = 200_000
    x = df_round(signed_logspace(rng, 1e-12, 1e12, n))
    y = df_round(signed_logspace(rng, 1e-12, 1e12, n))
    for op, ref in (("mul", x * y), ("div", x / y)):
        assert rel(run(op, x, y), ref).max() < 4 * 2.0 ** -48, op
    # sums: relative to the larger operand (cancellation leaves the exact difference of
    # the rounded arguments, which the double-float sum reproduces to its own rounding)
    for op, ref in (("add", x + y), ("sub", x - y)):
        err = np.abs(run(op, x, y) - ref) / np.maximum(np.abs(x), np.abs(y))
        assert err.max() < 4 * 2.0 ** -48, op
    # near-cancelling differences, as q_a - q_s and theta_a - T_s are
    a = df_round(rng.uniform(250.0, 310.0, n))
    b = df_round(a * (1.0 + signed_logspace(rng, 1e-9, 1e-3, n)))
    d = run("sub", a, b)
    assert rel(d, a - b).max() < 1e-13


def test_sqrt_and_cbrt(rng):
    n = 200_000
    x = df_round(np.exp(rng.uniform(np.log(1e-20), np.log(1e20), n)))
    assert rel(run("sqrt", x), np.sqrt(x)).max() < 4 * 2.0 ** -48
    s = df_round(signed_logspace(rng, 1e-20, 1e20, n))
    assert rel(run("cbrt", s), np.cbrt(s)).max() < 1e-13
    assert run("sqrt", np.array([0.0]))[0] == 0.0 and run("cbrt", np.array([0.0]))[0] == 0.0


def test_exp_log_pow(rng):
    n = 200_000
    # (results above ~1e-26 keep their low part above FP32's normal range)
    x = df_round(rng.uniform(-60.0, 80.0, n))
    assert rel(run("exp", x), np.exp(x)).max() < 1e-13
    small = df_round(signed_logspace(rng, 1e-12, 1.0, n))
    assert rel(run("exp", small), np.exp(small)).max() < 1e-13
    p = df_round(np.exp(rng.uniform(np.log(1e-25), np.log(1e30), n)))
    assert np.abs(run("log", p) - np.log(p)).max() / np.abs(np.log(p)).max() < 2e-14
    assert rel(run("log", p), np.log(p)).max() < 1e-12
    near1 = df_round(1.0 + signed_logspace(rng, 1e-10, 0.3, n))
    assert rel(run("log", near1), np.log(near1)).max() < 1e-12
    # the saturation vapour pressure's (T / T_tr)^A and the roughness's Re^-b
    base = df_round(rng.uniform(0.8, 1.2, n))
    expo = df_round(rng.uniform(-10.0, 10.0, n))
    assert rel(run("pow", base, expo), base ** expo).max() < 1e-13
    re = df_round(np.exp(rng.uniform(np.log(1e-3), np.log(1e6), n)))
    assert rel(run("pow", re, df_round(np.full(n, -0.6))), re ** df_round(np.full(n, -0.6))).max() < 1e-13
    assert run("exp", np.array([-200.0]))[0] == 0.0 and np.isinf(run("exp", np.array([200.0]))[0])
    assert np.isneginf(run("log", np.array([0.0]))[0]) and np.isnan(run("log", np.array([-1.0]))[0])


def test_atan(rng):
    n = 200_000
    x = df_round(signed_logspace(rng, 1e-10, 1e10, n))
    assert rel(run("atan", x), np.arctan(x)).max() < 1e-13
    grid = df_round(np.linspace(-3.0, 3.0, 100_001))
    err = np.abs(run("atan", grid) - np.arctan(grid))
    assert err.max() < 3e-14
    assert run("atan", np.array([0.0]))[0] == 0.0


def test_arguments_are_checked():
    lib = _lib.load()
    assert lib.nesf_double_float_check(None, None, None, 4, 0, None) == A.NESF_ERR_ARG
    assert lib.nesf_double_float_check(None, None, None, 0, 42, None) == A.NESF_ERR_ARG
    assert lib.nesf_double_float_check(None, None, None, 0, 4, None) == A.NESF_OK
