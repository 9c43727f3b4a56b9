"""Shared helpers of the parity tests."""
import numpy as np


def rel_err(gpu, ref, floor_frac=0.0):
    """Per-cell |gpu - ref| / max(|ref|, floor), floor = floor_frac * max|ref| (0: pure relative,
    with exact zeros compared absolutely)."""
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.abs(ref)
    finite = scale[np.isfinite(scale)]
    floor = floor_frac * np.max(finite) if finite.size else 0.0
    den = np.maximum(scale, floor)
    err = np.abs(gpu - ref)
    out = np.where(den > 0, err / np.where(den > 0, den, 1.0), err)
    both_nan = np.isnan(gpu) & np.isnan(ref)
    one_nan = np.isnan(gpu) ^ np.isnan(ref)
    out = np.where(both_nan, 0.0, out)
    return np.where(one_nan, np.inf, out)


def to_numpy(t):
    return t.detach().cpu().numpy()


def widen(arrays):
    """FP32 inputs as the FP64 values the oracle sees."""
    out = {}
    for k, v in arrays.items():
        if v is None:
            out[k] = None
        elif v.dtype in (np.float32, np.float64):
            out[k] = v.astype(np.float64)
        else:
            out[k] = v
    return out


def assert_conditioned(gpu, ref, keys, response, label="", units=4.0):
    """The plain FP64 parity bar, per cell: relative error (floor 1e-6 of the field's largest
    magnitude) <= 1e-12, or `units` times the oracle's own response to one unit in the last
    place of its interface humidity, of theta_a or of T_s where that is larger (oracle
    conditioning_response). Where q_a - q_s or theta_a - T_s nearly cancels, a last-place
    difference of a libm result or of a contracted multiply-add between the CPU and the GPU
    moves the reference's own answer by that much; elsewhere the bar is 1e-12."""
    for k in keys:
        e = rel_err(gpu[k], ref[k], floor_frac=1e-6)
        bar = np.maximum(1e-12, units * np.asarray(response[k]))
        ok = e <= bar
        if not np.all(ok):
            worst = int(np.argmax(np.where(ok, 0.0, e / bar)))
            raise AssertionError((label, k, "cells over the bar:", int((~ok).sum()), "of", e.size,
                                  "worst error / bar:", float((e / bar).ravel()[worst]),
                                  "error:", float(e.ravel()[worst]), "cells > 1e-12:", int((e > 1e-12).sum())))
