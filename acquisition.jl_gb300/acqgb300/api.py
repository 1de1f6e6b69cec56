"""Python mirror of Acquisition.jl's public API over the C ABI (GB300 kernels underneath).

Names, argument meaning and errors follow the reference:

* ``plan_acquire``     — src/plan.jl:312-697
* ``acquire_b``        — ``acquire!``, src/acquire.jl:54-89 and :788-797 (``!`` is spelled ``_b``)
* ``acquire``          — src/acquire.jl:838-882
* ``AcquisitionResults`` — src/Acquisition.jl:81-109
* ``get_num_cells`` / ``is_detected`` — src/Acquisition.jl:124-142
* ``cfar_threshold``   — src/cfar.jl:64-85
* ``OppositeRowNoiseEstimator`` / ``GlobalMeanNoiseEstimator`` — src/est_signal_noise_power.jl:70,100

Every acquisition runs on the GPU through libacqgb300.so; nothing here computes on the CPU
beyond argument marshalling.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _lib as L


PRECISIONS = {"fp32": 0, "fp16": 1, "bf16": 2, "fp16_split": 3, "bf16_split": 4}


class ArgumentError(ValueError):
    """Mirror of Julia's ArgumentError (invalid plan or acquire! arguments)."""


class AcquisitionError(RuntimeError):
    """CUDA, allocation or device-wait failure inside the library."""


def _check(status: int):
    if status == L.ACQ_OK:
        return
    msg = L.last_error()
    if status in (L.ACQ_ERR_ARGUMENT, L.ACQ_ERR_SHORT_SIGNAL, L.ACQ_ERR_PRN_NOT_IN_PLAN):
        raise ArgumentError(msg)
    raise AcquisitionError(f"status {status}: {msg}")


# ---------------------------------------------------------------- systems and estimators
@dataclass(frozen=True)
class GNSSSystem:
    name: str
    sid: int
    code_length: int
    code_frequency: float
    center_frequency: float
    data_frequency: float
    secondary_code: tuple = ()

    @property
    def secondary_code_length(self) -> int:
        return max(1, len(self.secondary_code))

    def gen_code(self, n: int, prn: int, sampling_freq: float, code_frequency: Optional[float] = None,
                 start_phase: float = 0.0) -> np.ndarray:
        """GNSSSignals ``gen_code`` semantics (host, C++)."""
        out = np.empty(int(n), dtype=np.int8)
        _check(L.load().acq_gen_code(self.sid, int(prn), int(n), float(sampling_freq),
                                     float(code_frequency or 0.0), float(start_phase),
                                     out.ctypes.data_as(C.POINTER(C.c_int8))))
        return out


_NH10 = (1, 1, 1, 1, -1, -1, 1, -1, 1, -1)


def GPSL1CA() -> GNSSSystem:
    return GNSSSystem("GPSL1CA", L.ACQ_GPS_L1CA, 1023, 1.023e6, 1575.42e6, 50.0)


def GPSL5I() -> GNSSSystem:
    return GNSSSystem("GPSL5I", L.ACQ_GPS_L5I, 10230, 10.23e6, 1176.45e6, 100.0, _NH10)


def GalileoE1B() -> GNSSSystem:
    """Galileo E1B with seeded synthetic memory codes and a BOC(1,1) sub-carrier."""
    return GNSSSystem("GalileoE1B", L.ACQ_GALILEO_E1B, 4092, 1.023e6, 1575.42e6, 250.0)


class AbstractNoiseEstimator:
    code = -1


class OppositeRowNoiseEstimator(AbstractNoiseEstimator):
    code = L.ACQ_NOISE_OPPOSITE_ROW


class GlobalMeanNoiseEstimator(AbstractNoiseEstimator):
    code = L.ACQ_NOISE_GLOBAL_MEAN


# ---------------------------------------------------------------- results
class _Shared:
    """Fields every result of one request shares (the plan's system and geometry)."""
    __slots__ = ("system", "sampling_frequency", "dopplers", "num_blocks", "block_size", "num_secondary_rotations")

    def __init__(self, system, sampling_frequency, dopplers, num_blocks, block_size, num_secondary_rotations):
        self.system, self.sampling_frequency, self.dopplers = system, sampling_frequency, dopplers
        self.num_blocks, self.block_size, self.num_secondary_rotations = num_blocks, block_size, num_secondary_rotations


class AcquisitionResults:
    """One acquisition result (src/Acquisition.jl:81-109) plus the decision indices the GPU pipeline
    reports (0-based). The values are read from the request's own copy of the C result records,
    so a later acquisition on the plan leaves them unchanged; ``power_bins`` is the plan's cached
    per-PRN buffer, overwritten by the next acquisition that stores power bins (the reference's
    aliasing, test/plan.jl:350-355)."""
    __slots__ = ("_a", "_i", "_s", "power_bins")
    _FIELDS = ("system", "prn", "sampling_frequency", "carrier_doppler", "code_phase", "secondary_code_phase", "CN0",
               "noise_power", "peak_to_noise_ratio", "num_noncoherent_integrations", "power_bins", "dopplers",
               "num_blocks", "block_size", "num_secondary_rotations", "peak_power", "peak_doppler_bin",
               "peak_code_bin", "sign_pattern", "bit_edge")

    def __init__(self, records, index, shared, power_bins=None):
        self._a, self._i, self._s, self.power_bins = records, index, shared, power_bins

    def _f(self, name):
        return self._a[name][self._i]

    system = property(lambda self: self._s.system)
    sampling_frequency = property(lambda self: self._s.sampling_frequency)
    dopplers = property(lambda self: self._s.dopplers)
    num_blocks = property(lambda self: self._s.num_blocks)
    block_size = property(lambda self: self._s.block_size)
    num_secondary_rotations = property(lambda self: self._s.num_secondary_rotations)
    prn = property(lambda self: int(self._f("prn")))
    carrier_doppler = property(lambda self: float(self._f("carrier_doppler_hz")))
    code_phase = property(lambda self: float(self._f("code_phase")))
    CN0 = property(lambda self: float(self._f("cn0_dbhz")))
    noise_power = property(lambda self: np.float32(self._f("noise_power")))
    peak_to_noise_ratio = property(lambda self: np.float32(self._f("peak_to_noise_ratio")))
    peak_power = property(lambda self: np.float32(self._f("peak_power")))
    num_noncoherent_integrations = property(lambda self: int(self._f("num_noncoherent_integrations")))
    peak_doppler_bin = property(lambda self: int(self._f("peak_doppler_bin")))
    peak_code_bin = property(lambda self: int(self._f("peak_code_bin")))
    sign_pattern = property(lambda self: int(self._f("sign_pattern")))
    bit_edge = property(lambda self: int(self._f("bit_edge")))

    @property
    def secondary_code_phase(self) -> Optional[int]:
        v = int(self._f("secondary_code_phase"))
        return None if v < 0 else v

    def __eq__(self, other):
        if not isinstance(other, AcquisitionResults):
            return NotImplemented
        for f in self._FIELDS:
            a, b = getattr(self, f), getattr(other, f)
            if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
                if not (a is b or (a is not None and b is not None and np.array_equal(a, b))):
                    return False
            elif a != b:
                return False
        return True

    __hash__ = None

    def __repr__(self):
        return (f"AcquisitionResults: PRN {self.prn}, CN0 = {self.CN0:.2f} dB-Hz, Doppler = "
                f"{self.carrier_doppler} Hz, Code phase = {self.code_phase:.3f} chips")


def get_num_cells(result: AcquisitionResults) -> int:
    """src/Acquisition.jl:124-126."""
    return len(result.dopplers) * result.num_blocks * result.block_size * result.num_secondary_rotations


def cfar_threshold(pfa: float, num_cells: int, num_noncoherent_integrations: int = 1) -> float:
    """src/cfar.jl:64-85 (host C++)."""
    out = C.c_double()
    _check(L.load().acq_cfar_threshold(float(pfa), int(num_cells), int(num_noncoherent_integrations),
                                       C.byref(out)))
    return out.value


def is_detected(result: AcquisitionResults, pfa: float = 0.01) -> bool:
    """src/Acquisition.jl:135-142."""
    return float(result.peak_to_noise_ratio) > cfar_threshold(pfa, get_num_cells(result),
                                                              result.num_noncoherent_integrations)


# ---------------------------------------------------------------- plan
def _desc(system: GNSSSystem, sampling_freq, min_doppler_coverage, n_coh, n_be, n_nc, noise_estimator,
          use_secondary_code, max_rot, device) -> L.PlanDesc:
    d = L.PlanDesc()
    L.load().acq_plan_desc_init(C.byref(d))
    d.system = system.sid
    d.sampling_freq_hz = float(sampling_freq)
    d.min_doppler_coverage_hz = float(min_doppler_coverage)
    d.num_coherently_integrated_code_periods = int(n_coh)
    d.bit_edge_search_steps = int(n_be)
    d.num_noncoherent_accumulations = int(n_nc)
    est = noise_estimator() if isinstance(noise_estimator, type) else noise_estimator
    d.noise_estimator = est.code
    d.use_secondary_code = 1 if use_secondary_code else 0
    d.max_secondary_code_rotations = int(max_rot)
    d.device = int(device)
    return d


def plan_geometry(system: GNSSSystem, sampling_freq, **kw) -> L.Geometry:
    """Validation + geometry only (no GPU), the first half of plan_acquire."""
    d = _desc(system, sampling_freq, kw.get("min_doppler_coverage", 7000.0),
              kw.get("num_coherently_integrated_code_periods", 1), kw.get("bit_edge_search_steps", 1),
              kw.get("num_noncoherent_accumulations", 1), kw.get("noise_estimator", OppositeRowNoiseEstimator()),
              kw.get("use_secondary_code", True), kw.get("max_secondary_code_rotations", 32), kw.get("device", 0))
    g = L.Geometry()
    _check(L.load().acq_plan_query(C.byref(d), C.byref(g)))
    return g


class AcquisitionPlan:
    """Pre-computed FM-DBZP plan (src/plan.jl:81-174) owning its device memory and stream."""

    def __init__(self, system: GNSSSystem, sampling_freq: float, prns, desc: L.PlanDesc, codes=None):
        lib = L.load()
        self.system = system
        self.sampling_freq = float(sampling_freq)
        self.avail_prns = [int(p) for p in prns]
        arr = (C.c_int32 * len(self.avail_prns))(*self.avail_prns)
        codes_ptr = None
        if codes is not None:
            codes = np.ascontiguousarray(codes, dtype=np.int8)
            codes_ptr = codes.ctypes.data_as(C.POINTER(C.c_int8))
        h = C.c_void_p()
        _check(lib.acq_plan_create(C.byref(desc), arr, len(self.avail_prns), codes_ptr, C.byref(h)))
        self._h = h
        g = L.Geometry()
        _check(lib.acq_plan_get_geometry(h, C.byref(g)))
        self.geometry = g
        dop = np.empty(g.num_doppler_bins, dtype=np.float64)
        _check(lib.acq_plan_doppler_freqs(h, dop.ctypes.data_as(C.POINTER(C.c_double))))
        self.doppler_freqs = dop
        self.noise_estimator = desc.noise_estimator
        self.use_secondary_code = bool(desc.use_secondary_code)
        self.max_secondary_code_rotations = desc.max_secondary_code_rotations
        self.device = desc.device
        # per-PRN cached power-bin matrices (src/plan.jl:123-126): lazily allocated, reused
        self.result_buffers = [None] * len(self.avail_prns)

    # geometry fields under the reference's names
    samples_per_code = property(lambda s: s.geometry.samples_per_code)
    samples_per_code_eff = property(lambda s: s.geometry.samples_per_code_eff)
    num_blocks = property(lambda s: s.geometry.num_blocks)
    block_size = property(lambda s: s.geometry.block_size)
    fft_size = property(lambda s: s.geometry.fft_size)
    num_coherently_integrated_code_periods = property(lambda s: s.geometry.num_coherently_integrated_code_periods)
    num_data_bits = property(lambda s: s.geometry.num_data_bits)
    bit_edge_search_steps = property(lambda s: s.geometry.bit_edge_search_steps)
    num_noncoherent_accumulations = property(lambda s: s.geometry.num_noncoherent_accumulations)
    num_secondary_rotations = property(lambda s: s.geometry.num_secondary_rotations)
    num_doppler_bins = property(lambda s: s.geometry.num_doppler_bins)

    @property
    def handle(self):
        return self._h

    def stream_handle(self) -> int:
        s = C.c_void_p()
        _check(L.load().acq_plan_stream(self._h, C.byref(s)))
        return s.value or 0

    def last_launch_count(self) -> int:
        n = C.c_int64()
        _check(L.load().acq_plan_last_launch_count(self._h, C.byref(n)))
        return n.value

    def last_kernels(self) -> list:
        """Names of the kernels the last acquisition launched, in order (acq_plan_last_kernels)."""
        buf = C.create_string_buffer(8192)
        _check(L.load().acq_plan_last_kernels(self._h, buf, len(buf)))
        return [k for k in buf.value.decode().split(";") if k]

    def set_form(self, form: str) -> str:
        """'plain' (one kernel per stage, the default) or 'fused' (cluster kernel where supported).
        Returns the form in effect."""
        val = {"fused": L.ACQ_FORM_FUSED, "plain": L.ACQ_FORM_PLAIN}[form]
        eff = C.c_int64()
        _check(L.load().acq_plan_set_option(self._h, L.ACQ_OPT_FORM, val, C.byref(eff)))
        return "fused" if eff.value == L.ACQ_FORM_FUSED else "plain"

    def set_option(self, option: int, value: int) -> int:
        """acq_plan_set_option: returns the value in effect (see include/acqgb300.h)."""
        eff = C.c_int64()
        _check(L.load().acq_plan_set_option(self._h, int(option), int(value), C.byref(eff)))
        return eff.value

    def get_option(self, option: int) -> int:
        v = C.c_int64()
        _check(L.load().acq_plan_get_option(self._h, int(option), C.byref(v)))
        return v.value

    def set_rotation_precision(self, precision: str) -> str:
        """Arithmetic of the secondary-code rotation combine: 'fp32' (FFTs on the CUDA cores, the
        default) or a tensor-core variant 'fp16', 'bf16', 'fp16_split', 'bf16_split' (sub-block
        spectra rounded to FP16/BF16, or split hi + lo, FP32 accumulation). Returns the precision
        in effect ('fp32' where the plan's geometry has no tensor-core variant)."""
        val = PRECISIONS[precision]
        eff = C.c_int64()
        _check(L.load().acq_plan_set_option(self._h, L.ACQ_OPT_ROTATION_PRECISION, val, C.byref(eff)))
        return {v: k for k, v in PRECISIONS.items()}[eff.value]

    def set_doppler_precision(self, precision: str) -> str:
        """Simple path: the per-column Doppler DFT as a dense DFT-matrix GEMM on the tensor cores
        ('fp16', 'bf16', 'fp16_split', 'bf16_split'; ndop <= 250) or FP32 FFTs ('fp32', the
        default). Returns the precision in effect."""
        val = PRECISIONS[precision]
        eff = C.c_int64()
        _check(L.load().acq_plan_set_option(self._h, L.ACQ_OPT_DOPPLER_PRECISION, val, C.byref(eff)))
        return {v: k for k, v in PRECISIONS.items()}[eff.value]

    def set_mma_scale_log2(self, e: int | None):
        """Power-of-two scale of the spectra before FP16 rounding (None: by input type)."""
        _check(L.load().acq_plan_set_option(self._h, L.ACQ_OPT_MMA_SCALE_LOG2, 127 if e is None else int(e), None))

    def set_kernel_timing(self, enable: bool = True):
        _check(L.load().acq_plan_set_kernel_timing(self._h, 1 if enable else 0))

    def reset_kernel_times(self):
        _check(L.load().acq_plan_reset_kernel_times(self._h))

    def kernel_times(self) -> dict:
        """{kernel class: (total device ms, launches)} accumulated since the last reset."""
        ms = (C.c_double * L.KERNEL_KINDS)()
        n = (C.c_int64 * L.KERNEL_KINDS)()
        _check(L.load().acq_plan_kernel_times(self._h, ms, n, L.KERNEL_KINDS))
        return {L.KERNEL_NAMES[i]: (ms[i], n[i]) for i in range(L.KERNEL_KINDS) if n[i] > 0}

    def close(self):
        if getattr(self, "_h", None):
            L.load().acq_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_acquire(system: GNSSSystem, sampling_freq, prns, *, min_doppler_coverage=7000.0,
                 num_coherently_integrated_code_periods: int = 1, bit_edge_search_steps: int = 1,
                 num_noncoherent_accumulations: int = 1, noise_estimator=OppositeRowNoiseEstimator(),
                 use_secondary_code: bool = True, max_secondary_code_rotations: int = 32, device: int = 0,
                 codes=None, fft_flag=None) -> AcquisitionPlan:
    """plan_acquire (src/plan.jl:312-697). ``fft_flag`` is accepted and ignored (no FFTW)."""
    d = _desc(system, sampling_freq, min_doppler_coverage, num_coherently_integrated_code_periods,
              bit_edge_search_steps, num_noncoherent_accumulations, noise_estimator, use_secondary_code,
              max_secondary_code_rotations, device)
    return AcquisitionPlan(system, sampling_freq, list(np.atleast_1d(prns)), d, codes)


# ---------------------------------------------------------------- acquire!
def _as_samples(signal):
    """Return (contiguous array, dtype code, n_samples) for a host signal."""
    a = np.asarray(signal)
    if np.iscomplexobj(a):
        if a.dtype == np.complex64:
            return np.ascontiguousarray(a), L.ACQ_CF32, a.size
        if a.dtype == np.complex128:
            return np.ascontiguousarray(a), L.ACQ_CF64, a.size
        a = a.astype(np.complex64)
        return np.ascontiguousarray(a), L.ACQ_CF32, a.size
    if a.ndim >= 1 and a.shape[-1] == 2 and a.dtype in (np.int16, np.int8, np.float32, np.float64):
        code = {np.dtype(np.int16): L.ACQ_CI16, np.dtype(np.int8): L.ACQ_CI8,
                np.dtype(np.float32): L.ACQ_CF32, np.dtype(np.float64): L.ACQ_CF64}[a.dtype]
        return np.ascontiguousarray(a), code, a.size // 2
    if a.dtype.kind in "fiu":  # real samples -> ComplexF32(x)
        return np.ascontiguousarray(a.astype(np.complex64)), L.ACQ_CF32, a.size
    raise ArgumentError(f"unsupported signal dtype {a.dtype}")


_RESULT_DTYPE = np.dtype([("prn", "<i4"), ("secondary_code_phase", "<i4"), ("carrier_doppler_hz", "<f8"),
                          ("code_phase", "<f8"), ("cn0_dbhz", "<f8"), ("noise_power", "<f4"),
                          ("peak_to_noise_ratio", "<f4"), ("peak_power", "<f4"),
                          ("num_noncoherent_integrations", "<i4"), ("peak_doppler_bin", "<i4"),
                          ("peak_code_bin", "<i4"), ("sign_pattern", "<i4"), ("bit_edge", "<i4"),
                          ("detected", "<i4"), ("reserved", "<i4")])
assert _RESULT_DTYPE.itemsize == C.sizeof(L.Result)


def _results(plan: AcquisitionPlan, res_arr, prns, store_power_bins, bins):
    """AcquisitionResults over the C result records (a ctypes array of Result, or a structured numpy
    view of one), which this request owns: the records are read when a field is accessed."""
    g = plan.geometry
    a = res_arr if isinstance(res_arr, np.ndarray) else np.frombuffer(res_arr, dtype=_RESULT_DTYPE, count=len(prns))
    shared = _Shared(plan.system, plan.sampling_freq, plan.doppler_freqs, g.num_blocks, g.block_size,
                     g.num_secondary_rotations)
    if not store_power_bins:
        return [AcquisitionResults(a, i, shared) for i in range(len(prns))]
    out = []
    for i, p in enumerate(prns):
        slot = plan.avail_prns.index(p)
        if plan.result_buffers[slot] is None:
            plan.result_buffers[slot] = np.empty((g.num_doppler_bins, g.samples_per_code_eff), np.float32)
        np.copyto(plan.result_buffers[slot], bins[i])
        out.append(AcquisitionResults(a, i, shared, plan.result_buffers[slot]))
    return out


def _flags(subsample_interpolation, store_power_bins, chip_sorted=False):
    return ((L.ACQ_FLAG_SUBSAMPLE_INTERP if subsample_interpolation else 0)
            | (L.ACQ_FLAG_STORE_POWER_BINS if store_power_bins else 0)
            | (L.ACQ_FLAG_POWER_BINS_CHIP_SORTED if (store_power_bins and chip_sorted) else 0))


def chip_order(num_blocks: int, block_size: int, width: int, code_freq: float, sampling_freq: float):
    """(perm, chip_axis): the FM-DBZP column shown at each chip-sorted position and its code phase
    in chips (src/plot.jl:16-20,35-57, ``_fmdbzp_sort_by_chip``)."""
    perm = np.empty(int(width), np.int32)
    axis = np.empty(int(width), np.float64)
    _check(L.load().acq_chip_order(int(num_blocks), int(block_size), int(width), float(code_freq),
                                   float(sampling_freq), perm.ctypes.data_as(C.POINTER(C.c_int32)),
                                   axis.ctypes.data_as(C.POINTER(C.c_double))))
    return perm, axis


def plan_chip_axis(plan: "AcquisitionPlan") -> np.ndarray:
    """Code phase (chips) of every column of a chip-sorted power surface of this plan."""
    g = plan.geometry
    return chip_order(g.num_blocks, g.block_size, g.samples_per_code_eff, plan.system.code_frequency,
                      plan.sampling_freq)[1]


def acquire_b(plan: AcquisitionPlan, signal, prns, *, interm_freq: float = 0.0,
              subsample_interpolation: bool = False, store_power_bins: bool = False,
              chip_sorted_power_bins: bool = False):
    """``acquire!(plan, signal, prns; interm_freq, subsample_interpolation, store_power_bins)``.

    ``signal`` is a host array (complex64/complex128, or (..., 2) int16/int8 interleaved) or a
    CUDA tensor (see :func:`acquire_device`). A scalar ``prns`` returns one result.
    ``chip_sorted_power_bins`` returns the surfaces with columns in code-phase order
    (:func:`plan_chip_axis` gives the axis) instead of FM-DBZP order.
    """
    single = np.ndim(prns) == 0
    prn_list = [int(p) for p in np.atleast_1d(prns)]
    if _is_cuda_tensor(signal):
        out = acquire_device(plan, signal, prn_list, interm_freq=interm_freq,
                             subsample_interpolation=subsample_interpolation, store_power_bins=store_power_bins)
        return out[0] if single else out
    lib = L.load()
    arr, dt, n = _as_samples(signal)
    g = plan.geometry
    res = (L.Result * len(prn_list))()
    bins = None
    bins_ptr = None
    if store_power_bins:
        bins = np.empty((len(prn_list), g.num_doppler_bins, g.samples_per_code_eff), np.float32)
        bins_ptr = bins.ctypes.data_as(C.POINTER(C.c_float))
    prn_arr = (C.c_int32 * len(prn_list))(*prn_list)
    _check(lib.acq_acquire(plan.handle, arr.ctypes.data_as(C.c_void_p), dt, int(n), prn_arr, len(prn_list),
                           float(interm_freq), _flags(subsample_interpolation, store_power_bins,
                                                      chip_sorted_power_bins), res, bins_ptr))
    out = _results(plan, res, prn_list, store_power_bins, bins)
    return out[0] if single else out


def _is_cuda_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and hasattr(x, "data_ptr") and bool(x.is_cuda)


def _tensor_dtype(t):
    import torch
    if t.dtype == torch.complex64:
        return L.ACQ_CF32, t.numel()
    if t.dtype == torch.complex128:
        return L.ACQ_CF64, t.numel()
    if t.shape[-1] == 2 and t.dtype in (torch.int16, torch.int8, torch.float32, torch.float64):
        return {torch.int16: L.ACQ_CI16, torch.int8: L.ACQ_CI8, torch.float32: L.ACQ_CF32,
                torch.float64: L.ACQ_CF64}[t.dtype], t.numel() // 2
    raise ArgumentError(f"unsupported tensor dtype {t.dtype}")


def acquire_device_async(plan: AcquisitionPlan, tensor, prns, *, interm_freq: float = 0.0,
                         subsample_interpolation: bool = False, store_power_bins: bool = False):
    """Enqueue an acquisition on the plan's stream for a device-resident signal (no wait)."""
    if not tensor.is_contiguous():
        raise ArgumentError("device signal must be contiguous")
    dt, n = _tensor_dtype(tensor)
    prn_list = [int(p) for p in np.atleast_1d(prns)]
    prn_arr = (C.c_int32 * len(prn_list))(*prn_list)
    _check(L.load().acq_acquire_device_async(plan.handle, C.c_void_p(tensor.data_ptr()), dt, int(n), prn_arr,
                                             len(prn_list), float(interm_freq),
                                             _flags(subsample_interpolation, store_power_bins)))
    return prn_list


def fetch_results(plan: AcquisitionPlan, prns, store_power_bins: bool = False):
    g = plan.geometry
    prn_list = [int(p) for p in np.atleast_1d(prns)]
    res = (L.Result * len(prn_list))()
    bins = None
    bins_ptr = None
    if store_power_bins:
        bins = np.empty((len(prn_list), g.num_doppler_bins, g.samples_per_code_eff), np.float32)
        bins_ptr = bins.ctypes.data_as(C.POINTER(C.c_float))
    _check(L.load().acq_fetch_results(plan.handle, res, bins_ptr))
    return _results(plan, res, prn_list, store_power_bins, bins)


def acquire_device(plan: AcquisitionPlan, tensor, prns, *, interm_freq: float = 0.0,
                   subsample_interpolation: bool = False, store_power_bins: bool = False):
    """acquire! on a device-resident signal (a contiguous CUDA tensor)."""
    import torch
    torch.cuda.current_stream(tensor.device).synchronize()
    prn_list = acquire_device_async(plan, tensor, prns, interm_freq=interm_freq,
                                    subsample_interpolation=subsample_interpolation,
                                    store_power_bins=store_power_bins)
    return fetch_results(plan, prn_list, store_power_bins)


def acquire(system: GNSSSystem, signal, sampling_freq, prns, *, interm_freq: float = 0.0,
            min_doppler_coverage=7000.0, num_coherently_integrated_code_periods: int = 1,
            bit_edge_search_steps: int = 1, num_noncoherent_accumulations: int = 1,
            use_secondary_code: bool = True, max_secondary_code_rotations: int = 32,
            noise_estimator=OppositeRowNoiseEstimator(), subsample_interpolation: bool = False,
            store_power_bins: bool = False, fft_flag=None, device: int = 0):
    """acquire (src/acquire.jl:838-882): plan_acquire then acquire!."""
    single = np.ndim(prns) == 0
    prn_list = [int(p) for p in np.atleast_1d(prns)]
    plan = plan_acquire(system, sampling_freq, prn_list, min_doppler_coverage=min_doppler_coverage,
                        num_coherently_integrated_code_periods=num_coherently_integrated_code_periods,
                        bit_edge_search_steps=bit_edge_search_steps,
                        num_noncoherent_accumulations=num_noncoherent_accumulations,
                        noise_estimator=noise_estimator, use_secondary_code=use_secondary_code,
                        max_secondary_code_rotations=max_secondary_code_rotations, device=device)
    try:
        out = acquire_b(plan, signal, prn_list, interm_freq=interm_freq,
                        subsample_interpolation=subsample_interpolation, store_power_bins=store_power_bins)
    finally:
        if not store_power_bins:
            plan.close()
    return out[0] if single else out
