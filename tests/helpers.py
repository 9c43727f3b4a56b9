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
