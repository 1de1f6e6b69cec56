"""The reference's end-to-end behaviour tests, run through the GPU path (acquire! on the device).

Each test makes the assertions of one reference testset (cited per test) on seeded recordings of
the reference's signal model (src/generate_test_signal.jl:45-68, restated by the oracle), the same
recordings the oracle's own versions of these tests use.
"""
import math

import numpy as np
import pytest

import acqgb300 as A
from oracle import acq_oracle as O
from oracle import gnss_codes as G

pytestmark = pytest.mark.gpu


def _sig(system, prn, n, fs, doppler, cp, cn0, seed):
    rng = np.random.default_rng(seed)
    noise = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
    x = (O.clean_signal(system, prn, n, fs, doppler, cp, 0.0, amplitude=10 ** (cn0 / 20))
         + noise * 10 ** (10 * math.log10(fs) / 20))
    return x.astype(np.complex64)


def _step(plan):
    d = plan.doppler_freqs
    return float(d[1] - d[0])


def test_cn0_is_per_hz_independent_of_coherent_length():
    # test/acquire.jl:462-520
    fs, reported = 4e6, []
    for n in (1, 2, 4, 5, 10):
        plan = A.plan_acquire(A.GPSL1CA(), fs, [1], num_coherently_integrated_code_periods=n,
                              min_doppler_coverage=25_000)
        est = []
        for k in range(1, 9):
            r = A.acquire_b(plan, _sig(G.GPSL1CA, 1, 4000 * n + 100, fs, 1234.0, (k - 0.5) * 1023 / 8 + 0.137, 45,
                                       700 + k), 1, subsample_interpolation=True)
            if A.is_detected(r):
                est.append(float(r.CN0))
        assert len(est) >= 5, n
        reported.append(sum(est) / len(est))
    assert all(abs(c - 45) <= 6.0 for c in reported), reported
    assert max(reported) - min(reported) < 4.0 and reported[-1] - reported[0] < 2.0, reported


def test_peak_to_noise_ratio_consistent_with_cn0():
    # test/cfar.jl:117-133
    plan = A.plan_acquire(A.GPSL1CA(), 2.048e6, [1])
    strong = A.acquire_b(plan, _sig(G.GPSL1CA, 1, 2048, 2.048e6, 1000.0, 200.0, 55, 11), 1)
    weak = A.acquire_b(plan, _sig(G.GPSL1CA, 1, 2048, 2.048e6, 1000.0, 200.0, 35, 11), 1)
    assert strong.peak_to_noise_ratio > weak.peak_to_noise_ratio and strong.CN0 > weak.CN0


@pytest.mark.parametrize("n_coh", [40, 60])
def test_data_bit_transition_at_zero_doppler_keeps_the_peak(n_coh):
    # test/noncoherent_integration.jl:602-701 (data bits +1 -1 and +1 -1 +1)
    fs = 2.048e6
    clean = _sig(G.GPSL1CA, 1, n_coh * 2048, fs, 0.0, 0.0, 60, 42)
    flipped = clean.copy()
    flipped[20 * 2048:40 * 2048] *= -1
    plan = A.plan_acquire(A.GPSL1CA(), fs, [1], min_doppler_coverage=10_000,
                          num_coherently_integrated_code_periods=n_coh)
    ref = A.acquire_b(plan, clean, 1)
    got = A.acquire_b(plan, flipped, 1)
    assert float(got.peak_power) == pytest.approx(float(ref.peak_power), rel=0.1)
    assert (got.peak_doppler_bin, got.peak_code_bin) == (ref.peak_doppler_bin, ref.peak_code_bin)


def test_multistep_two_prns_planted_and_absent():
    # test/acquire.jl:137-156
    plan = A.plan_acquire(A.GPSL1CA(), 2.048e6, [1, 2], num_noncoherent_accumulations=2)
    r1, r2 = A.acquire_b(plan, _sig(G.GPSL1CA, 1, 2 * 2048, 2.048e6, 800.0, 150.0, 45, 13), [1, 2])
    assert A.is_detected(r1) and abs(r1.code_phase - 150.0) <= 1.5
    assert not A.is_detected(r2)


def test_one_step_and_two_step_paths_agree():
    # test/acquire.jl:158-195 (48 dB-Hz: see the oracle's version of this test)
    fs, cp, dop = 2.048e6, 100.0, 1500.0
    x = _sig(G.GPSL1CA, 1, 2 * 2048, fs, dop, cp, 48, 123)
    for n_nc, seg in ((1, x[:2048]), (2, x)):
        plan = A.plan_acquire(A.GPSL1CA(), fs, [1], num_noncoherent_accumulations=n_nc)
        r = A.acquire_b(plan, seg, 1)
        assert A.is_detected(r) and abs(r.code_phase - cp) < 1.0 and abs(r.carrier_doppler - dop) < _step(plan)


@pytest.mark.parametrize("cov,n_coh,dop,cp", [(5000, 40, 500.0, 100.0), (10_000, 40, 0.0, 333.0),
                                              (20_000, 10, 1500.0, 100.0)])
def test_sign_search_and_large_doppler_grids(cov, n_coh, dop, cp):
    # test/acquire.jl:197-230 (two data bits: Doppler without a half-band offset) and :290-341 (more
    # than 320 Doppler bins)
    fs = 2.048e6
    plan = A.plan_acquire(A.GPSL1CA(), fs, [1], min_doppler_coverage=cov, num_coherently_integrated_code_periods=n_coh)
    r = A.acquire_b(plan, _sig(G.GPSL1CA, 1, n_coh * 2048, fs, dop, cp, 45, 31 if cov == 5000 else 17), 1)
    assert A.is_detected(r) and abs(r.code_phase - cp) <= 1.0 and abs(r.carrier_doppler - dop) < _step(plan)


def test_global_mean_estimator_on_the_one_step_path():
    # test/acquire.jl:355-386
    fs = 2.048e6
    x = _sig(G.GPSL1CA, 4, 2048, fs, 750.0, 512.0, 45, 21)
    pg = A.plan_acquire(A.GPSL1CA(), fs, [4], noise_estimator=A.GlobalMeanNoiseEstimator())
    po = A.plan_acquire(A.GPSL1CA(), fs, [4])
    rg, ro = A.acquire_b(pg, x, 4), A.acquire_b(po, x, 4)
    assert A.is_detected(rg)
    assert (rg.code_phase, rg.carrier_doppler) == (ro.code_phase, ro.carrier_doppler)
    assert rg.noise_power != ro.noise_power
    rs = A.acquire_b(pg, x, 4, store_power_bins=True)
    P = np.asarray(rs.power_bins, np.float64)
    half = int(fs // 1.023e6)
    keep = np.ones(P.shape[1], bool)
    keep[max(0, rs.peak_code_bin - half):min(P.shape[1], rs.peak_code_bin + half + 1)] = False
    assert float(rs.noise_power) == pytest.approx(P[:, keep].sum() / (keep.sum() * P.shape[0]), rel=1e-5)


def test_multistep_interpolation_and_stored_surface():
    # test/acquire.jl:435-460
    fs, cp = 2.048e6, 700.4
    plan = A.plan_acquire(A.GPSL1CA(), fs, [1], num_noncoherent_accumulations=4)
    x = _sig(G.GPSL1CA, 1, 4 * 2048, fs, 500.0, cp, 42, 8)
    r = A.acquire_b(plan, x, 1, subsample_interpolation=True, store_power_bins=True)
    assert A.is_detected(r) and abs(r.code_phase - cp) <= 1.0
    first = np.array(r.power_bins)
    assert first.shape == (len(plan.doppler_freqs), plan.samples_per_code_eff)
    r2 = A.acquire_b(plan, x, 1, subsample_interpolation=True, store_power_bins=True)
    assert np.array_equal(np.asarray(r2.power_bins), first)


@pytest.mark.parametrize("M,n_coh,cn0", [(2, 4, 40), (4, 4, 38), (8, 1, 42)])
def test_weak_signal_passes_the_noncoherent_threshold(M, n_coh, cn0):
    # test/cfar.jl:91-115
    plan = A.plan_acquire(A.GPSL1CA(), 2.048e6, list(range(1, 33)), num_coherently_integrated_code_periods=n_coh,
                          num_noncoherent_accumulations=M)
    r = A.acquire_b(plan, _sig(G.GPSL1CA, 7, n_coh * 2048 * M, 2.048e6, 500.0, 100.0, cn0, 9999 + M), 7)
    assert A.is_detected(r, pfa=0.01) and abs(r.code_phase - 100.0) < 1.0


def test_l5i_gain_recovery_over_the_opt_out():
    # test/secondary_code_search.jl:133-175
    fs = 10.24e6
    primary = G.gen_code(10240, G.GPSL5I, 1, fs).astype(np.complex64)
    x = np.concatenate([np.float32(G.NH10[k]) * primary for k in range(10)])
    peaks = []
    for use in (True, False):
        plan = A.plan_acquire(A.GPSL5I(), fs, [1], min_doppler_coverage=5000, num_coherently_integrated_code_periods=10,
                              use_secondary_code=use)
        peaks.append(float(np.max(A.acquire_b(plan, x, 1, store_power_bins=True).power_bins)))
    assert peaks[0] / peaks[1] > 8


@pytest.mark.parametrize("cp,dop,n_nc", [(1234.5, 1000.0, 1), (5115.0, 1000.0, 1), (1234.5, 5000.0, 4)])
def test_l5i_rotation_search_code_phase_and_doppler(cp, dop, n_nc):
    # test/secondary_code_search.jl:177-206,294-386
    fs = 12e6
    plan = A.plan_acquire(A.GPSL5I(), fs, [1], num_coherently_integrated_code_periods=10,
                          num_noncoherent_accumulations=n_nc)
    assert plan.num_secondary_rotations == 10
    r = A.acquire_b(plan, _sig(G.GPSL5I, 1, n_nc * 10 * 12000, fs, dop, cp, 45, 29), 1)
    assert A.is_detected(r)
    assert abs(r.code_phase - cp) <= (1.5 if n_nc > 1 else 1.0)
    assert abs(r.carrier_doppler - dop) < _step(plan)


def test_secondary_code_phase_exact_across_code_phase_and_doppler():
    # test/secondary_code_search.jl:260-292 (the full 4 x 4 x 2 sweep)
    fs = 12e6
    plan = A.plan_acquire(A.GPSL5I(), fs, [1], num_coherently_integrated_code_periods=10)
    for cp in (0.0, 2000.0, 5115.0, 9000.0):
        primary = G.gen_code(12000, G.GPSL5I, 1, fs, start_phase=cp).astype(np.complex64)
        for r0 in (0, 3, 7, 9):
            base = np.concatenate([np.float32(G.NH10[(k + r0) % 10]) * primary for k in range(10)])
            for dop in (0.0, 1300.0):
                x = base if dop == 0.0 else (base * np.exp(2j * np.pi * dop / fs * np.arange(len(base)))).astype(
                    np.complex64)
                assert A.acquire_b(plan, x, 1).secondary_code_phase == r0, (cp, r0, dop)


def test_cfar_detection_with_synthetic_signal():
    # test/cfar.jl:31-52: the planted PRN clears the threshold, at most 3 of the 31 absent ones do
    fs = 2.048e6
    plan = A.plan_acquire(A.GPSL1CA(), fs, list(range(1, 33)))
    res = A.acquire_b(plan, _sig(G.GPSL1CA, 1, 2048, fs, 1000.0, 200.0, 45, 1), list(range(1, 33)))
    thr = A.cfar_threshold(0.01, A.get_num_cells(res[0]))
    assert res[0].prn == 1 and res[0].peak_to_noise_ratio > thr
    assert sum(r.peak_to_noise_ratio > thr for r in res[1:]) <= 3


def test_l5i_rotation_multi_symbol_data_flip():
    # test/secondary_code_search.jl:208-258: 20 ms = two NH10 periods with a data flip between them
    fs, n, cp, fd = 12e6, 20, 1234.5, 1000.0
    primary = G.gen_code(12000, G.GPSL5I, 1, fs, start_phase=cp).astype(np.complex64)
    x = np.concatenate([np.float32(G.NH10[k % 10] * (1 if k < 10 else -1)) * primary for k in range(n)])
    x = (x * np.exp(2j * np.pi * fd / fs * np.arange(len(x)))).astype(np.complex64)
    plan = A.plan_acquire(A.GPSL5I(), fs, [1], num_coherently_integrated_code_periods=n)
    assert plan.num_secondary_rotations == 10
    r = A.acquire_b(plan, x, 1)
    assert A.is_detected(r) and abs(r.code_phase - cp) < 1.0 and abs(r.carrier_doppler - fd) < _step(plan)
    assert r.secondary_code_phase == 0 and r.sign_pattern == 1
