"""Ragged batches: many recordings of uneven length and mixed systems in one CUDA-graph launch.

A batch generalises ``acquire!`` (src/acquire.jl:54-89) to a list of recordings. Each item names
its plan (recordings with the same geometry share one), its samples and the PRNs to search. The
library packs every recording into one device arena and replays a single CUDA graph holding all
acquisitions (one graph branch per plan).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .api import (_RESULT_DTYPE, AcquisitionPlan, GNSSSystem, _as_samples, _check, _results, plan_acquire)

class BatchItemC(C.Structure):
    _fields_ = [("plan", C.c_void_p), ("dtype", C.c_int32), ("n_samples", C.c_int64),
                ("prns", C.POINTER(C.c_int32)), ("n_prns", C.c_int32), ("interm_freq_hz", C.c_double),
                ("flags", C.c_uint32)]


def _bind():
    lib = L.load()
    if getattr(lib, "_batch_bound", False):
        return lib
    P = C.c_void_p
    lib.acq_batch_create.argtypes = [C.POINTER(BatchItemC), C.c_int32, C.POINTER(P)]
    lib.acq_batch_destroy.argtypes = [P]
    lib.acq_batch_input_ptr.argtypes = [P, C.c_int32, C.POINTER(P)]
    lib.acq_batch_upload.argtypes = [P, C.POINTER(C.c_void_p)]
    lib.acq_batch_launch.argtypes = [P]
    lib.acq_batch_fetch.argtypes = [P, C.POINTER(L.Result)]
    lib.acq_batch_run.argtypes = [P, C.POINTER(C.c_void_p), C.POINTER(L.Result)]
    lib.acq_batch_stream.argtypes = [P, C.POINTER(P)]
    lib.acq_batch_launch_count.argtypes = [P, C.POINTER(C.c_int64)]
    for n in ("acq_batch_create", "acq_batch_destroy", "acq_batch_input_ptr", "acq_batch_upload", "acq_batch_launch",
              "acq_batch_fetch", "acq_batch_run", "acq_batch_stream", "acq_batch_launch_count"):
        getattr(lib, n).restype = C.c_int
    lib._batch_bound = True
    return lib


@dataclass
class BatchItem:
    plan: AcquisitionPlan
    samples: np.ndarray
    prns: list
    interm_freq: float = 0.0
    subsample_interpolation: bool = False


class AcquisitionBatch:
    """One CUDA graph over every item; ``run()`` = upload + one graph launch + results."""

    def __init__(self, items):
        lib = _bind()
        self.items = list(items)
        self._arrays = []
        arr = (BatchItemC * len(self.items))()
        self._prn_bufs = []
        for i, it in enumerate(self.items):
            a, dt, n = _as_samples(it.samples)
            self._arrays.append(a)
            pb = (C.c_int32 * len(it.prns))(*[int(p) for p in it.prns])
            self._prn_bufs.append(pb)
            arr[i].plan = it.plan.handle.value
            arr[i].dtype = dt
            arr[i].n_samples = int(n)
            arr[i].prns = pb
            arr[i].n_prns = len(it.prns)
            arr[i].interm_freq_hz = float(it.interm_freq)
            arr[i].flags = L.ACQ_FLAG_SUBSAMPLE_INTERP if it.subsample_interpolation else 0
        h = C.c_void_p()
        _check(lib.acq_batch_create(arr, len(self.items), C.byref(h)))
        self._h = h
        self.total = sum(len(it.prns) for it in self.items)

    def _ptrs(self, samples=None):
        if samples is not None:
            self._arrays = [_as_samples(s)[0] for s in samples]
        return (C.c_void_p * len(self._arrays))(*[a.ctypes.data for a in self._arrays])

    def upload(self, samples=None):
        _check(_bind().acq_batch_upload(self._h, self._ptrs(samples)))

    def launch(self):
        _check(_bind().acq_batch_launch(self._h))

    def fetch(self):
        res = (L.Result * self.total)()
        _check(_bind().acq_batch_fetch(self._h, res))
        recs = np.frombuffer(res, dtype=_RESULT_DTYPE)
        out, k = [], 0
        for it in self.items:
            n = len(it.prns)
            out.append(_results(it.plan, recs[k:k + n], [int(p) for p in it.prns], False, None))
            k += n
        return out

    def run(self, samples=None):
        """Upload the recordings, launch the graph once, return one result list per item."""
        self.upload(samples)
        self.launch()
        return self.fetch()

    def input_ptr(self, i: int) -> int:
        p = C.c_void_p()
        _check(_bind().acq_batch_input_ptr(self._h, int(i), C.byref(p)))
        return p.value

    def stream_handle(self) -> int:
        p = C.c_void_p()
        _check(_bind().acq_batch_stream(self._h, C.byref(p)))
        return p.value or 0

    def launch_count(self) -> int:
        n = C.c_int64()
        _check(_bind().acq_batch_launch_count(self._h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "_h", None):
            _bind().acq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


CONSTELLATION = {"GPSL1CA": 32, "GPSL5I": 32, "GalileoE1B": 36}


class PlanCache:
    """One plan per geometry (system, fs, coherent periods, accumulations, coverage), holding the
    whole constellation; every recording requests its own PRN subset."""

    def __init__(self, device: int = 0):
        self.device = device
        self.plans = {}

    def get(self, system: GNSSSystem, fs: float, *, n_coh: int = 1, n_nc: int = 1, cov: float = 7000.0,
            n_be: int = 1) -> AcquisitionPlan:
        key = (system.name, float(fs), int(n_coh), int(n_nc), float(cov), int(n_be))
        if key not in self.plans:
            prns = list(range(1, CONSTELLATION.get(system.name, 32) + 1))
            self.plans[key] = plan_acquire(system, fs, prns, min_doppler_coverage=cov,
                                           num_coherently_integrated_code_periods=n_coh,
                                           num_noncoherent_accumulations=n_nc, bit_edge_search_steps=n_be,
                                           device=self.device)
        return self.plans[key]


def batch_from_recordings(recordings, cache: PlanCache, subsample_interpolation: bool = False):
    """BatchItems for recordings as produced by ``synth.ragged_batch``."""
    items = []
    for r in recordings:
        plan = cache.get(r["system"], r["fs"], n_coh=r["n_coh"], n_nc=r["n_nc"], cov=r.get("cov", 7000.0))
        items.append(BatchItem(plan, r["samples"], r["prns"], r.get("interm_freq", 0.0), subsample_interpolation))
    return items
