"""Prescribed-atmosphere forcing streamed from host storage into a device window of
snapshots: the FieldTimeSeries of a PrescribedAtmosphere with an InMemory(K) backend
(JRA55_prescribed_atmosphere.jl:17,37-42: `time_indices_in_memory = 10`,
`time_indexing = Cyclical()`), read as `update_state!(::PrescribedAtmosphere)` reads it
(prescribed_atmosphere.jl:154-162) and handed to the interpolation of
interpolate_atmospheric_state.jl:57-60.

A window holds K snapshots of each variable in one device tensor per variable (K slots;
a time index takes a slot whose snapshot is neither in the current pair nor among the
snapshots prefetched after it). `update(t)` asks the library for the two
snapshots bracketing t and their weight (nesf_time_indices), makes both resident, and
returns what nesf_interpolate_atmosphere_state takes: per variable a view of the first
snapshot's slot, with the snapshot stride pointing at the second one's slot (negative
when that slot comes first). The snapshots after the pair are prefetched: a
reader thread fills pinned host slots from the source while the GPU works, and their
host-to-device copies run on a copy stream that waits for the last step that read the
slot; the caller's stream waits for a slot's copy before it reads it.

Sources: `ArraySource` (host arrays of shape (Nt, ...) per variable) and `NpySource`
(one `.npy` file per variable and time index, memory-mapped), both returning one
snapshot (Ny + 2Hy, Nx + 2Hx) of the atmosphere grid's parent layout.
"""
import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import _abi as A
from ._lib import check, load

VARIABLES = ("u", "v", "T", "q", "p", "rain", "snow", "sw", "lw")
INDEXING = {"cyclical": A.TIME_CYCLICAL, "linear": A.TIME_LINEAR, "clamp": A.TIME_CLAMP}


def time_indices(times, t, indexing="cyclical", period=0.0):
    """nesf_time_indices: (n1, n2, weight of n2), 0-based."""
    lib = load()
    ts = np.ascontiguousarray(times, dtype=np.float64)
    n1, n2, w = C.c_int32(), C.c_int32(), C.c_double()
    check(lib.nesf_time_indices(ts.ctypes.data_as(C.POINTER(C.c_double)), len(ts), INDEXING[indexing],
                                float(period or 0.0), float(t), C.byref(n1), C.byref(n2), C.byref(w)))
    return n1.value, n2.value, w.value


class ArraySource:
    """Snapshots held in host arrays: `arrays[name][n]` is snapshot n of `name`."""

    def __init__(self, arrays):
        self.arrays = arrays
        self.names = tuple(arrays)

    def read(self, name, n, out):
        np.copyto(out, self.arrays[name][n], casting="same_kind")


class NpySource:
    """One file per variable and time index, `{directory}/{name}_{n:05d}.npy`, memory-mapped
    on read (only the snapshot's bytes are touched)."""

    def __init__(self, directory, names):
        self.directory = directory
        self.names = tuple(names)

    def path(self, name, n):
        return os.path.join(self.directory, f"{name}_{n:05d}.npy")

    @staticmethod
    def write(directory, arrays):
        """Store host arrays (Nt, ...) per variable in the layout this source reads."""
        os.makedirs(directory, exist_ok=True)
        for name, a in arrays.items():
            for n in range(a.shape[0]):
                np.save(os.path.join(directory, f"{name}_{n:05d}.npy"), np.ascontiguousarray(a[n]))

    def read(self, name, n, out):
        np.copyto(out, np.load(self.path(name, n), mmap_mode="r"), casting="same_kind")


class FieldTimeSeriesWindow:
    """K device slots per variable of the snapshots `times` (seconds) from `source`."""

    def __init__(self, source, times, atmos_layout, slots=10, indexing="cyclical", period=0.0, dtype=None,
                 device="cuda", readers=2):
        import torch
        self.torch = torch
        self.source = source
        self.names = tuple(n for n in VARIABLES if n in source.names)
        self.times = np.ascontiguousarray(times, dtype=np.float64)
        self.nt = len(self.times)
        self.K = max(2, min(int(slots), self.nt))
        self.indexing, self.period = indexing, period
        self.layout = atmos_layout
        shape = atmos_layout.shape
        self.dtype = dtype or torch.float32
        self.ring = {n: torch.empty((self.K,) + tuple(shape), dtype=self.dtype, device=device) for n in self.names}
        self.host = {n: torch.empty((self.K,) + tuple(shape), dtype=self.dtype, pin_memory=True) for n in self.names}
        self.slot_elems = int(np.prod(shape))
        self.resident = [-1] * self.K        # the time index each slot holds (or is being filled with)
        self.slot_of = {}                    # time index -> slot
        self.ready = [None] * self.K         # copy-stream event: the slot's upload is done
        self.released = [None] * self.K      # caller-stream event: the last read of the slot is done
        self.pending = {}                    # slot -> future of the host read in flight
        self.copy_stream = torch.cuda.Stream(device=device)
        self.pool = ThreadPoolExecutor(max_workers=max(1, int(readers)))
        self.uploads = 0

    def close(self):
        self.pool.shutdown(wait=True)

    # ------------------------------------------------------------------ filling
    def _read_host(self, slot, n):
        np_view = {name: self.host[name][slot].numpy() for name in self.names}
        for name in self.names:
            self.source.read(name, n, np_view[name])

    def _schedule(self, n, keep):
        """Start filling a slot with time index n (the host read in the pool, the upload
        later), taking a slot whose snapshot is not in `keep`; returns the slot."""
        if n in self.slot_of:
            return self.slot_of[n]
        slot = next(k for k in range(self.K) if self.resident[k] not in keep)
        fut = self.pending.pop(slot, None)
        if fut is not None:
            fut.result()
        if self.ready[slot] is not None:
            # the host rewrites the pinned slot: the upload that read it must be done
            self.ready[slot].synchronize()
        self.slot_of.pop(self.resident[slot], None)
        self.resident[slot] = n
        self.slot_of[n] = slot
        self.ready[slot] = None
        self.pending[slot] = self.pool.submit(self._read_host, slot, n)
        return slot

    def _upload(self, slot):
        """Issue the slot's host-to-device copies once its host read is done."""
        fut = self.pending.pop(slot, None)
        if fut is None:
            return
        fut.result()
        torch = self.torch
        with torch.cuda.stream(self.copy_stream):
            if self.released[slot] is not None:
                self.copy_stream.wait_event(self.released[slot])
            for name in self.names:
                self.ring[name][slot].copy_(self.host[name][slot], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.copy_stream)
        self.ready[slot] = ev
        self.uploads += 1

    # ------------------------------------------------------------------ use
    def update(self, t, stream=None):
        """The snapshot pair of time t, resident on the device, and its weight: returns
        (arrays, atmos_stride_t, weight) for nesf_interpolate_atmosphere_state. The caller's
        `stream` (default: the current stream) waits for the pair's uploads; call `release`
        after the launches that read them."""
        torch = self.torch
        n1, n2, w = time_indices(self.times, t, self.indexing, self.period)
        # the pair, then the snapshots after it (prefetched), K in all
        if self.indexing == "cyclical":
            ahead = [(n2 + k) % self.nt for k in range(1, self.K - 1)]
        else:
            ahead = list(range(n2 + 1, min(self.nt, n2 + self.K - 1)))
        keep = {n1, n2, *ahead}
        s1 = self._schedule(n1, keep)
        s2 = self._schedule(n2, keep)
        for slot in (s1, s2):
            self._upload(slot)
        for n in ahead:
            self._schedule(n, keep)
        s = stream or torch.cuda.current_stream()
        for slot in (s1, s2):
            if self.ready[slot] is not None:
                s.wait_event(self.ready[slot])
        self._pair = (s1, s2)
        arrays = {name: self.ring[name][s1] for name in self.names}
        return arrays, (s2 - s1) * self.slot_elems, w

    def release(self, stream=None):
        """Mark the pair returned by the last `update` as read by the work enqueued on `stream`
        so far, and upload the prefetched snapshots whose host reads are done."""
        torch = self.torch
        s = stream or torch.cuda.current_stream()
        for slot in set(self._pair):
            ev = torch.cuda.Event()
            ev.record(s)
            self.released[slot] = ev
        for slot, fut in list(self.pending.items()):
            if fut.done() and slot not in self._pair:
                self._upload(slot)
