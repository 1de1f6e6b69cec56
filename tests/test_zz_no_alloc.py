"""The no-allocation statistics entry point against acq_acquire, through the C ABI.

acq_est_signal_noise_power_noalloc serves callers that cannot allocate device memory while
running (a receiver's real-time processing thread, where cudaMalloc/cudaFree may synchronise
the device and stall it, or a plugin whose host framework owns all device memory). Given the
power surface that acq_acquire stored, it must report the same peak cell and, within the
tolerance of the parity tests, the same noise power, on consecutive calls that share its
static scratch; and the oracle's estimators (src/est_signal_noise_power.jl:109-243) run on that
same surface must agree. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import _lib as L
from acqgb300 import synth
from oracle import acq_oracle as O
from oracle import gnss_codes as G

pytestmark = pytest.mark.gpu

RTOL = 1e-4   # SCALAR_RTOL of tests/test_gpu_parity.py


def _noalloc(power_bins: np.ndarray, fs: float, fc: float, estimator: int) -> L.NoiseStats:
    import torch
    surf = torch.from_numpy(np.ascontiguousarray(power_bins, dtype=np.float32)).cuda()
    out = torch.zeros(C.sizeof(L.NoiseStats), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    st = L.load().acq_est_signal_noise_power_noalloc(C.c_void_p(surf.data_ptr()), surf.shape[0], surf.shape[1],
                                                     fs, fc, estimator, C.c_void_p(out.data_ptr()), None)
    assert st == L.ACQ_OK, L.last_error()
    torch.cuda.synchronize()
    return L.NoiseStats.from_buffer_copy(out.cpu().numpy().tobytes())


KW = dict(min_doppler_coverage=5000, num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)


def _acquired(estimator):
    fs = 5e6
    sats = [synth.Satellite(3, 44.0, 2300.0, 411.7), synth.Satellite(9, 41.0, -1800.0, 77.2)]
    plan = A.plan_acquire(A.GPSL1CA(), fs, [3, 9, 12], noise_estimator=estimator, **KW)
    x = synth.synth(A.GPSL1CA(), fs, 2 * 10 * plan.samples_per_code, sats, seed=31).astype(np.complex64)
    return A.acquire_b(plan, x, [3, 9, 12], store_power_bins=True), fs


def _check(stats: L.NoiseStats, r, fs, est):
    assert (stats.peak_doppler_bin, stats.peak_code_bin) == (r.peak_doppler_bin, r.peak_code_bin)
    assert stats.peak_power == float(r.peak_power)
    assert stats.noise_power == pytest.approx(float(r.noise_power), rel=RTOL)
    assert stats.signal_power == pytest.approx(float(r.peak_power) - float(r.noise_power), rel=RTOL)
    # the oracle's peak (lowest column, then lowest row) and FP64 noise estimate on the same surface
    oplan = O.plan_acquire(G.GPSL1CA, fs, [r.prn], precision="f64",
                           noise_estimator="global_mean" if est == L.ACQ_NOISE_GLOBAL_MEAN else "opposite_row", **KW)
    surf = O.PrnSurface(r.power_bins.astype(np.float64), np.zeros(r.power_bins.shape, np.int32), "materialised")
    peak, row, col = O.find_peak(surf, oplan)
    assert (stats.peak_doppler_bin, stats.peak_code_bin) == (row, col)
    assert stats.peak_power == np.float32(peak)
    assert stats.noise_power == pytest.approx(O.noise_power(surf, oplan, row, col), rel=RTOL)


def test_noalloc_matches_acquire_on_consecutive_calls():
    fc = A.GPSL1CA().code_frequency
    res_or, fs = _acquired(A.OppositeRowNoiseEstimator())
    res_gm, _ = _acquired(A.GlobalMeanNoiseEstimator())
    # several calls in a row share (and re-clear) the static scratch
    for r, est in [(res_or[0], L.ACQ_NOISE_OPPOSITE_ROW), (res_gm[1], L.ACQ_NOISE_GLOBAL_MEAN),
                   (res_or[2], L.ACQ_NOISE_OPPOSITE_ROW), (res_gm[0], L.ACQ_NOISE_GLOBAL_MEAN)]:
        _check(_noalloc(r.power_bins, fs, fc, est), r, fs, est)


@pytest.mark.parametrize("est", [L.ACQ_NOISE_OPPOSITE_ROW, L.ACQ_NOISE_GLOBAL_MEAN])
def test_noalloc_reference_known_answers(est):
    # test/est_signal_noise_power.jl:1-98: a 29 x 1023 unit surface (fs 4 MHz, fc 1 MHz) with a 15 dB
    # peak in the middle and at both corners, and for the opposite-row estimator an inflated band
    # in the peak's row that the opposite row does not see
    cases = [(10, 488, False), (0, 0, False), (28, 1022, False)]
    if est == L.ACQ_NOISE_OPPOSITE_ROW:
        cases.append((10, 488, True))
    for r, c, band in cases:
        P = np.ones((29, 1023), np.float32)
        if band:
            P[r, :] = 5.0
        P[r, c] += np.float32(10 ** 1.5)
        st = _noalloc(P, 4e6, 1e6, est)
        assert (st.peak_doppler_bin, st.peak_code_bin) == (r, c)
        assert st.noise_power == pytest.approx(1.0, rel=1e-6)
        assert st.signal_power == pytest.approx(float(P[r, c]) - 1.0, rel=1e-6)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(C.sizeof(L.NoiseStats), dtype=torch.uint8, device="cuda")
    st = L.load().acq_est_signal_noise_power_noalloc(C.c_void_p(dummy.data_ptr()), 5000, 100, 5e6, 1.023e6,
                                                     L.ACQ_NOISE_OPPOSITE_ROW, C.c_void_p(out.data_ptr()), None)
    assert st == L.ACQ_ERR_ARGUMENT
    assert "4096" in L.last_error()
