"""ctypes binding of libacqgb300.so (the C ABI declared in include/acqgb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# ACQ_CHECKED_LIBRARY=1 loads the bounds-checked build (device index checks, debug use) instead
LIB_PATH = os.path.join(_HERE, "libacqgb300_checked.so" if os.environ.get("ACQ_CHECKED_LIBRARY", "0") not in ("", "0")
                        else "libacqgb300.so")

ACQ_OK = 0
ACQ_ERR_ARGUMENT = 1
ACQ_ERR_SHORT_SIGNAL = 2
ACQ_ERR_PRN_NOT_IN_PLAN = 3
ACQ_ERR_CUDA = 4
ACQ_ERR_TIMEOUT = 5
ACQ_ERR_ALLOC = 6
ACQ_ERR_UNSUPPORTED = 7

ACQ_GPS_L1CA, ACQ_GPS_L5I, ACQ_GALILEO_E1B = 0, 1, 2
ACQ_CF32, ACQ_CI16, ACQ_CI8, ACQ_CF64 = 0, 1, 2, 3
ACQ_NOISE_OPPOSITE_ROW, ACQ_NOISE_GLOBAL_MEAN = 0, 1
ACQ_FLAG_SUBSAMPLE_INTERP = 1
ACQ_FLAG_STORE_POWER_BINS = 2
ACQ_FLAG_POWER_BINS_CHIP_SORTED = 4


class PlanDesc(C.Structure):
    _fields_ = [("system", C.c_int32), ("sampling_freq_hz", C.c_double), ("min_doppler_coverage_hz", C.c_double),
                ("num_coherently_integrated_code_periods", C.c_int32), ("bit_edge_search_steps", C.c_int32),
                ("num_noncoherent_accumulations", C.c_int32), ("noise_estimator", C.c_int32),
                ("use_secondary_code", C.c_int32), ("max_secondary_code_rotations", C.c_int32),
                ("device", C.c_int32)]


class Geometry(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "samples_per_code", "samples_per_code_eff", "num_blocks", "block_size", "fft_size",
        "num_coherently_integrated_code_periods", "num_data_bits", "bit_edge_search_steps",
        "num_noncoherent_accumulations", "num_doppler_bins", "num_secondary_rotations", "bit_period_codes",
        "num_prns", "path")] + [(n, C.c_double) for n in (
        "doppler_first_hz", "doppler_step_hz", "code_length", "code_freq_hz", "center_freq_hz",
        "cfar_threshold_pfa001")]


class NoiseStats(C.Structure):
    _fields_ = [("signal_power", C.c_float), ("noise_power", C.c_float), ("peak_power", C.c_float),
                ("peak_doppler_bin", C.c_int32), ("peak_code_bin", C.c_int32), ("reserved", C.c_int32)]


class Result(C.Structure):
    _fields_ = [("prn", C.c_int32), ("secondary_code_phase", C.c_int32), ("carrier_doppler_hz", C.c_double),
                ("code_phase", C.c_double), ("cn0_dbhz", C.c_double), ("noise_power", C.c_float),
                ("peak_to_noise_ratio", C.c_float), ("peak_power", C.c_float),
                ("num_noncoherent_integrations", C.c_int32), ("peak_doppler_bin", C.c_int32),
                ("peak_code_bin", C.c_int32), ("sign_pattern", C.c_int32), ("bit_edge", C.c_int32),
                ("detected", C.c_int32), ("reserved", C.c_int32)]


class SynthSat(C.Structure):
    _fields_ = [("prn", C.c_int32), ("data_bits", C.c_int32), ("cn0_dbhz", C.c_double), ("doppler_hz", C.c_double),
                ("code_phase", C.c_double), ("carrier_phase", C.c_double), ("bit_offset_s", C.c_double)]


class CorrCell(C.Structure):
    _fields_ = [("prn", C.c_int32), ("reserved", C.c_int32), ("code_phase", C.c_double), ("doppler_hz", C.c_double)]


class CorrResult(C.Structure):
    _fields_ = [("power", C.c_double), ("grad", C.c_double * 2), ("hess", C.c_double * 3), ("z_re", C.c_double),
                ("z_im", C.c_double), ("iterations", C.c_int32), ("status", C.c_int32)]


ACQ_CORR_OK, ACQ_CORR_NOT_CONVERGED, ACQ_CORR_BAD_PRN = 0, 1, 3

EXPORTED = ["acq_plan_desc_init", "acq_plan_query", "acq_plan_create", "acq_plan_destroy", "acq_plan_get_geometry",
            "acq_plan_doppler_freqs", "acq_acquire", "acq_acquire_device_async", "acq_fetch_results",
            "acq_plan_stream", "acq_plan_last_launch_count", "acq_cfar_threshold", "acq_gen_code",
            "acq_last_error", "acq_version", "acq_plan_set_kernel_timing", "acq_plan_kernel_times",
            "acq_plan_reset_kernel_times", "acq_est_signal_noise_power_noalloc", "acq_plan_set_option",
            "acq_batch_create", "acq_batch_destroy", "acq_batch_input_ptr", "acq_batch_upload", "acq_batch_launch",
            "acq_batch_fetch", "acq_batch_run", "acq_batch_stream", "acq_batch_launch_count",
            "acq_corr_create", "acq_corr_destroy", "acq_corr_eval", "acq_corr_vjp_samples", "acq_corr_refine",
            "acq_plan_get_option", "acq_chip_order", "acq_sort_power_bins_by_chip", "acq_gen_code_device",
            "acq_selftest_bounded_wait", "acq_synth_signal", "acq_plan_last_kernels"]
ACQ_OPT_FORM = 0
ACQ_OPT_ROTATION_PRECISION = 1
ACQ_OPT_MMA_SCALE_LOG2 = 2
ACQ_OPT_TILE_THREADS, ACQ_OPT_TILE_BLOCKS, ACQ_OPT_TILE_PAD = 3, 4, 5
ACQ_OPT_COLUMN_WIDTH, ACQ_OPT_COLUMN_CTAS_PER_SM = 6, 7
ACQ_OPT_DOPPLER_PRECISION = 8
ACQ_OPT_TILE_ROWS = 9
ACQ_OPT_TRANSFORM_LENGTH = 10
ACQ_OPT_TILE_MMA = 11
ACQ_OPT_COLUMN_WAIT_POLLS = 12
ACQ_OPT_SEARCH_WIDTH, ACQ_OPT_SEARCH_SPLIT = 13, 14
ACQ_FORM_FUSED, ACQ_FORM_PLAIN = 0, 1
KERNEL_KINDS = 8
KERNEL_NAMES = ["frontend", "tile", "column", "stats", "extract", "secondary", "fused", "k7"]

_lib = None


def load():
    """Load the library (once). Raises OSError when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: build it with `python acquisition.jl_gb300/build_lib.py` "
                      "(there is no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    lib.acq_plan_desc_init.argtypes = [C.POINTER(PlanDesc)]
    lib.acq_plan_desc_init.restype = None
    lib.acq_plan_query.argtypes = [C.POINTER(PlanDesc), C.POINTER(Geometry)]
    lib.acq_plan_create.argtypes = [C.POINTER(PlanDesc), C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int8),
                                    C.POINTER(P)]
    lib.acq_plan_destroy.argtypes = [P]
    lib.acq_plan_get_geometry.argtypes = [P, C.POINTER(Geometry)]
    lib.acq_plan_doppler_freqs.argtypes = [P, C.POINTER(C.c_double)]
    lib.acq_acquire.argtypes = [P, P, C.c_int32, C.c_int64, C.POINTER(C.c_int32), C.c_int32, C.c_double, C.c_uint32,
                                C.POINTER(Result), C.POINTER(C.c_float)]
    lib.acq_acquire_device_async.argtypes = [P, P, C.c_int32, C.c_int64, C.POINTER(C.c_int32), C.c_int32, C.c_double,
                                             C.c_uint32]
    lib.acq_fetch_results.argtypes = [P, C.POINTER(Result), C.POINTER(C.c_float)]
    lib.acq_plan_stream.argtypes = [P, C.POINTER(P)]
    lib.acq_plan_last_launch_count.argtypes = [P, C.POINTER(C.c_int64)]
    lib.acq_plan_last_kernels.argtypes = [P, C.c_char_p, C.c_size_t]
    lib.acq_cfar_threshold.argtypes = [C.c_double, C.c_int64, C.c_int32, C.POINTER(C.c_double)]
    lib.acq_gen_code.argtypes = [C.c_int32, C.c_int32, C.c_int64, C.c_double, C.c_double, C.c_double,
                                 C.POINTER(C.c_int8)]
    lib.acq_last_error.argtypes = [C.c_char_p, C.c_size_t]
    lib.acq_plan_set_kernel_timing.argtypes = [P, C.c_int32]
    lib.acq_plan_kernel_times.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int32]
    lib.acq_plan_reset_kernel_times.argtypes = [P]
    lib.acq_est_signal_noise_power_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_double, C.c_double,
                                                       C.c_int32, C.c_void_p, C.c_void_p]
    lib.acq_plan_set_option.argtypes = [P, C.c_int32, C.c_int64, C.POINTER(C.c_int64)]
    lib.acq_plan_get_option.argtypes = [P, C.c_int32, C.POINTER(C.c_int64)]
    lib.acq_chip_order.argtypes = [C.c_int32, C.c_int32, C.c_int64, C.c_double, C.c_double, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_double)]
    lib.acq_sort_power_bins_by_chip.argtypes = [P, P, C.c_int32, P, P]
    lib.acq_synth_signal.argtypes = [C.c_int32, C.c_double, C.c_int64, C.POINTER(SynthSat), C.c_int32, C.c_double,
                                     C.c_uint64, C.c_int32, C.c_int32, P, P]
    lib.acq_selftest_bounded_wait.argtypes = [C.c_int32, C.c_uint32, C.POINTER(C.c_int32)]
    lib.acq_gen_code_device.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_int64, C.c_double,
                                        C.c_double, C.c_double, P, P]
    lib.acq_corr_create.argtypes = [C.c_int32, C.c_double, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int8),
                                    C.POINTER(P)]
    lib.acq_corr_destroy.argtypes = [P]
    lib.acq_corr_eval.argtypes = [P, P, C.c_int32, C.c_int64, C.c_double, P, C.c_int32, C.c_int32, P, P]
    lib.acq_corr_vjp_samples.argtypes = [P, C.c_int64, C.c_double, P, P, C.c_int32, P, P]
    lib.acq_corr_refine.argtypes = [P, P, C.c_int32, C.c_int64, C.c_double, P, C.c_int32, C.c_int32, C.c_double,
                                    C.c_double, C.c_double, C.c_double, P, P]
    lib.acq_version.restype = C.c_char_p
    for name in EXPORTED:
        if name not in ("acq_plan_desc_init", "acq_version"):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    load().acq_last_error(buf, len(buf))
    return buf.value.decode("utf-8", "replace")
