"""The on-disk tuning cache (nesf_tuning_cache_find / nesf_tuning_cache_store).

Host-only file I/O, so it runs here without a GPU: records round-trip, a key's
record is replaced rather than duplicated, the bytes follow the little-endian
layout include/nesf.h states, a file of another format version is read as empty
and rewritten, and a file that is not a cache (or is cut short) is refused and
left as it was.
"""
import ctypes as C
import struct

import pytest

from nesf import _abi as A
from nesf import _lib, api

TUNING = dict(solve_block=96, deferred_per_sm=8, infer_per_sm=2, two_lanes=1, io_overlap=0, pass1_fetch=3,
              refill_lanes=8, early_ocean_classify=1, ice_deferred_per_sm=2, cells_per_thread=2, step_ms=7.125)


def key(**kw):
    k = A.TuningKey(device=b"NVIDIA GB300", sm_count=152, compute_capability=103, nx=2880, ny=1280, hx=3, hy=3,
                    dtype=1, precision=2, warm_start=1, parts=31, flux_formulation=0)
    for f, v in kw.items():
        setattr(k, f, v)
    return k


def test_round_trip_and_replacement(tmp_path):
    path = tmp_path / "tune.bin"
    assert api.tuning_cache_find(path, key()) is None          # no file yet
    api.tuning_cache_store(path, key(), TUNING)
    assert api.tuning_cache_find(path, key()) == TUNING
    assert api.tuning_cache_find(path, key(nx=1440)) is None
    assert api.tuning_cache_find(path, key(device=b"NVIDIA B200")) is None
    other = dict(TUNING, solve_block=64, step_ms=9.5)
    api.tuning_cache_store(path, key(nx=1440), other)
    replaced = dict(TUNING, pass1_fetch=4, refill_lanes=16, step_ms=6.9)
    api.tuning_cache_store(path, key(), replaced)
    assert api.tuning_cache_find(path, key()) == replaced
    assert api.tuning_cache_find(path, key(nx=1440)) == other
    assert struct.unpack_from("<I", path.read_bytes(), 20)[0] == 2


def test_byte_layout(tmp_path):
    path = tmp_path / "tune.bin"
    api.tuning_cache_store(path, key(), TUNING)
    b = path.read_bytes()
    assert b[:8] == b"NESFTUNE"
    version, key_bytes, fields, count = struct.unpack_from("<4I", b, 8)
    assert (version, key_bytes, fields, count) == (A.TUNING_VERSION, 108, 10, 1)
    assert len(b) == 24 + 108 + 10 * 4 + 8
    rec = b[24:]
    assert rec[:64] == b"NVIDIA GB300".ljust(64, b"\0")
    assert struct.unpack_from("<11i", rec, 64) == (152, 103, 2880, 1280, 3, 3, 1, 2, 1, 31, 0)
    assert struct.unpack_from("<10i", rec, 108) == tuple(TUNING[k] for k in A.TUNING_FIELDS)
    assert struct.unpack_from("<d", rec, 148)[0] == TUNING["step_ms"]


def test_stale_version_reads_empty_and_is_rewritten(tmp_path):
    path = tmp_path / "tune.bin"
    api.tuning_cache_store(path, key(), TUNING)
    api.tuning_cache_store(path, key(ny=600), TUNING)
    b = bytearray(path.read_bytes())
    struct.pack_into("<I", b, 8, A.TUNING_VERSION + 1)
    path.write_bytes(bytes(b))
    assert api.tuning_cache_find(path, key()) is None
    api.tuning_cache_store(path, key(nx=720), TUNING)
    b = path.read_bytes()
    assert struct.unpack_from("<2I", b, 8)[0] == A.TUNING_VERSION and struct.unpack_from("<I", b, 20)[0] == 1
    assert api.tuning_cache_find(path, key(nx=720)) == TUNING


@pytest.mark.parametrize("content", [b"not a tuning cache", b"NESFTUNE\x01\x00", None])
def test_foreign_or_cut_files_are_refused_and_kept(tmp_path, content):
    path = tmp_path / "tune.bin"
    if content is None:                         # a cache cut inside its record
        api.tuning_cache_store(path, key(), TUNING)
        content = path.read_bytes()[:-5]
    path.write_bytes(content)
    lib = _lib.load()
    t, found = A.Tuning(), C.c_int32(7)
    assert lib.nesf_tuning_cache_find(str(path).encode(), C.byref(key()), C.byref(t), C.byref(found)) == A.NESF_ERR_ARG
    t = A.Tuning(**{k: TUNING[k] for k in A.TUNING_FIELDS})
    assert lib.nesf_tuning_cache_store(str(path).encode(), C.byref(key()), C.byref(t)) == A.NESF_ERR_ARG
    assert path.read_bytes() == content


def test_invalid_tuning_and_key_are_refused(tmp_path):
    path = tmp_path / "tune.bin"
    lib = _lib.load()
    bad = A.Tuning(**dict({k: TUNING[k] for k in A.TUNING_FIELDS}, pass1_fetch=9))
    assert lib.nesf_tuning_cache_store(str(path).encode(), C.byref(key()), C.byref(bad)) == A.NESF_ERR_ARG
    k = key()
    C.memmove(C.addressof(k), b"x" * 64, 64)     # device name without its NUL
    good = A.Tuning(**{f: TUNING[f] for f in A.TUNING_FIELDS})
    assert lib.nesf_tuning_cache_store(str(path).encode(), C.byref(k), C.byref(good)) == A.NESF_ERR_ARG
    assert not path.exists()
