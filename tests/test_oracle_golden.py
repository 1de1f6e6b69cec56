"""Pin the oracle against the reference's own known-answer tests and golden vector.

Every case cites the reference test it restates (paths inside Acquisition.jl v2.6.4).
The expected numbers live in tests/golden/reference_known_answers.json.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import acq_oracle as O
from oracle import gnss_codes as G

HERE = os.path.dirname(__file__)
KA = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))


# ---------------------------------------------------------------- code generators
def test_l1ca_first_ten_chips_octal():
    # IS-GPS-200 Table 3-Ia "first 10 chips" (octal) of the C/A code.
    for prn, octal in KA["l1ca_first10_octal"].items():
        if prn.startswith("_"):
            continue
        bits = (1 - G.l1ca_chips(int(prn))[:10]) // 2
        assert int("".join(map(str, bits)), 2) == int(octal, 8)


def test_l1ca_gold_three_valued_crosscorrelation():
    a = G.l1ca_chips(1).astype(np.int64)
    for prn in (2, 7, 19, 32):
        b = G.l1ca_chips(prn).astype(np.int64)
        cc = np.array([np.dot(a, np.roll(b, k)) for k in range(1023)])
        assert set(np.unique(cc)) <= {-65, -1, 63}
    ac = np.array([np.dot(a, np.roll(a, k)) for k in range(1, 1023)])
    assert set(np.unique(ac)) <= {-65, -1, 63}


def test_l5_xb_advance_matches_initial_states():
    # IS-GPS-705 Table 3-Ia: XB code advance and XB initial state must agree.
    for prn, state in KA["l5i_xb_initial_state"].items():
        if prn.startswith("_"):
            continue
        r = [1] * 13
        for _ in range(G._L5I_XB_ADVANCE[int(prn) - 1]):
            r = G._l5_xb_step(r)
        assert "".join(map(str, r)) == state


def test_nh10_literal():
    # test/sign_patterns.jl:45-46
    assert list(G.NH10) == KA["nh10"]


def test_l5i_code_balanced_and_baked_secondary():
    c = G.l5i_primary_chips(1)
    assert len(c) == 10230 and abs(int(c.astype(int).sum())) < 200
    full = G.GPSL5I.full_chips(1)
    assert np.array_equal(full[10230 * 4:10230 * 5], -c)       # NH10[4] = -1


# ---------------------------------------------------------------- geometry
@pytest.mark.parametrize("case", KA["geometry"], ids=lambda c: c["src"])
def test_geometry(case):
    g = O.plan_geometry(G.SYSTEMS[case["system"]], case["fs"], case["min_doppler_coverage"],
                        case.get("n_coh", 1), case.get("n_be", 1), case.get("n_nc", 1))
    for k, v in case["expect"].items():
        if k == "step":
            assert g["step"] == pytest.approx(v)
        elif k == "first":
            assert g["freqs"][0] == pytest.approx(v)
        else:
            assert g[k] == v, k


@pytest.mark.parametrize("kw", [
    dict(n_coh=30), dict(n_coh=20, n_be=3), dict(n_coh=1, n_be=2), dict(n_nc=0), dict(n_coh=0),
    dict(n_be=0), dict(min_doppler_coverage=1.1e6)])
def test_plan_validation_errors(kw):
    # test/plan.jl:146-168
    args = dict(min_doppler_coverage=7000.0, n_coh=1, n_be=1, n_nc=1)
    args.update(kw)
    with pytest.raises(O.ArgumentError):
        O.plan_geometry(G.GPSL1CA, 2.048e6, **args)


def test_secondary_code_errors():
    # test/plan.jl:70-121
    with pytest.raises(O.ArgumentError) as e:
        O.plan_geometry(G.GPSL5I, 10.24e6, 1000.0, 15)
    assert "secondary" in str(e.value).lower() and "15" in str(e.value) and "10" in str(e.value)
    with pytest.raises(O.ArgumentError) as e:
        O.plan_geometry(G.GPSL5I, 10.24e6, 1000.0, 5)
    m = str(e.value)
    assert "68" in m and "num_noncoherent_accumulations" in m and "use_secondary_code" in m
    assert O.plan_geometry(G.GPSL5I, 10.24e6, 1000.0, 10)["R"] == 10
    assert O.plan_geometry(G.GPSL5I, 10.24e6, 1000.0, 5, use_secondary_code=False)["R"] == 1
    # cap (test/plan.jl:123-144 uses L1C-P, L=1800): same check with a cap below L=10
    with pytest.raises(O.ArgumentError) as e:
        O.plan_geometry(G.GPSL5I, 10.24e6, 1000.0, 10, max_secondary_code_rotations=8)
    assert "max_secondary_code_rotations" in str(e.value)


def test_conj_code_spectrum_layout():
    # test/plan.jl:170-192
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [1, 2], min_doppler_coverage=10_000)
    assert plan.prn_conj_ffts[1].shape == (plan.num_blocks, plan.fft_size)
    assert plan.fft_size == 2 * plan.block_size == 128
    assert not np.array_equal(plan.prn_conj_ffts[1], plan.prn_conj_ffts[2])
    code = G.gen_code(plan.samples_per_code, G.GPSL1CA, 1, 2.048e6)
    blk = np.zeros(plan.fft_size, complex)
    blk[:plan.block_size] = code[:plan.block_size]
    assert np.allclose(plan.prn_conj_ffts[1][0], np.conj(np.fft.fft(blk)), atol=1e-3)


def test_column_to_tau():
    # test/plot.jl:18-41
    for c, tau in [(0, 0), (1, 1), (8, 24), (16, 16), (24, 8)]:
        assert O.fmdbzp_column_to_tau(c, 4, 8) == tau
    assert O.fmdbzp_column_to_tau(0, 32, 64) == 0
    assert sorted(O.fmdbzp_column_to_tau(c, 4, 8) for c in range(32)) == list(range(32))


def test_coherent_matrix_peak_columns():
    # test/coherent_integration.jl:4-78 (CN0 = 100, zero Doppler)
    fs = 2.048e6
    plan = O.plan_acquire(G.GPSL1CA, fs, [1], min_doppler_coverage=5000)
    assert (plan.num_blocks, plan.block_size) == (16, 128)
    for cp, exp_col in [(991.0, 65), (923.097656, 1993)]:
        amp = 10 ** (100 / 20)
        sig = O.clean_signal(G.GPSL1CA, 1, plan.samples_per_code, fs, 0.0, cp, amplitude=amp)
        rng = np.random.default_rng(1)
        sig = sig + math.sqrt(fs) * (rng.standard_normal(len(sig)) + 1j * rng.standard_normal(len(sig)))
        S = O.all_segment_ffts(plan, sig, 0.0)[0]
        cim = O.coherent_matrix(S, plan.prn_conj_ffts[1], plan)
        assert int(np.argmax(np.abs(cim[0]))) + 1 == exp_col


# ---------------------------------------------------------------- CFAR
def test_cfar_closed_form_and_monotonic():
    # test/cfar.jl:5-31
    assert O.cfar_threshold(0.01, 1) == pytest.approx(-math.log(0.01))
    assert O.cfar_threshold(0.001, 1) == pytest.approx(-math.log(0.001))
    assert O.cfar_threshold(0.01, 10000) > O.cfar_threshold(0.01, 100)
    assert O.cfar_threshold(0.001, 1000) > O.cfar_threshold(0.1, 1000)
    assert O.cfar_threshold(0.01, 1000, 3) < O.cfar_threshold(0.01, 1000, 1)
    for bad in [(0.0, 100), (1.0, 100), (-0.1, 100), (0.01, 0)]:
        with pytest.raises(O.ArgumentError):
            O.cfar_threshold(*bad)


# ---------------------------------------------------------------- sign patterns
def test_sign_patterns_known_answers():
    # test/sign_patterns.jl:1-122
    assert np.array_equal(O.sign_patterns(None, 1, 1, 1, 4, False), np.ones((4, 1), np.float32))
    p = O.sign_patterns(None, 1, 2, 1, 20, False)
    assert p.shape == (20, 2) and np.all(p[:, 0] == 1) and np.all(p[:10, 1] == 1) and np.all(p[10:, 1] == -1)
    p = O.sign_patterns(G.GPSL5I, 1, 1, 10, 10, True)
    assert list(p[:, 0]) == KA["nh10"]
    for r in range(10):
        assert list(p[:, r]) == [G.NH10[(k + r) % 10] for k in range(10)]
    assert np.array_equal(O.sign_patterns(G.GPSL5I, 1, 1, 10, 10, False), np.ones((10, 1), np.float32))
    ramp = O.combined_phase_patterns(O.sign_patterns(None, 1, 1, 1, 10, False), 10)
    for s in range(10):
        for k in range(10):
            assert ramp[k, 0, s] == pytest.approx(np.exp(-2j * np.pi * k * s / 10), rel=1e-6)
    comb = O.combined_phase_patterns(O.sign_patterns(G.GPSL5I, 1, 1, 10, 10, True), 10)
    tiled = O.tile_phase_patterns(comb, 150)
    for w in (0, 7, 149):
        assert np.array_equal(tiled[w], comb[:, :, w % 10])


# ---------------------------------------------------------------- noise estimators
def _surf(P):
    return O.PrnSurface(P.astype(np.float64), np.zeros(P.shape, np.int32), "materialised")


@pytest.mark.parametrize("est", ["opposite_row", "global_mean"])
def test_noise_estimators_constructed(est):
    # test/est_signal_noise_power.jl:4-98
    plan = O.plan_acquire(G.GPSL1CA, 4e6, [1])
    plan.noise_estimator = est
    plan.sampling_freq, plan.system = 4e6, G.System("x", 1023, 1e6, 1575.42e6, 0.0)
    for (r, c) in [(10, 488), (0, 0), (28, 1022)]:
        P = np.ones((29, 1023))
        P[r, c] += 10 ** 1.5
        s = _surf(P)
        peak, row, col = O.find_peak(s, plan)
        assert (row, col) == (r, c)
        n = O.noise_power(s, plan, row, col)
        assert n == pytest.approx(1) and peak - n == pytest.approx(10 ** 1.5)
    if est == "opposite_row":
        P = np.ones((29, 1023))
        P[10, :] = 5.0
        P[10, 488] = 5.0 + 10 ** 1.5
        s = _surf(P)
        peak, row, col = O.find_peak(s, plan)
        assert O.noise_power(s, plan, row, col) == pytest.approx(1.0)


# ---------------------------------------------------------------- code drift
def test_code_drift_shift_known_answer():
    # test/noncoherent_integration.jl:493-530 (shift ~ 36 samples at 7 kHz, step 100)
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [1], min_doppler_coverage=10_000,
                          num_coherently_integrated_code_periods=40, num_noncoherent_accumulations=200)
    row = int(np.argmin(np.abs(plan.doppler_freqs - 7000)))
    dur = 40 * plan.samples_per_code / 2.048e6
    exp = round(plan.doppler_freqs[row] * 100 * dur * 2.048e6 / 1575.42e6)
    assert exp == KA["drift_shift_7khz_step100"]
    assert O.code_drift_shifts(plan, 100)[row] == exp
    assert np.all(O.code_drift_shifts(plan, 0) == 0)


def test_fused_drift_scatter_equals_unfused_circshift():
    # test/noncoherent_integration.jl:4-86: scatter into destination rows == fftshift then circshift.
    rng = np.random.default_rng(20260526)
    for ndop, spc, step in [(64, 256, 5), (321, 128, 3), (8, 5000, 7), (32, 2048, 0)]:
        P = rng.random((ndop, spc))
        freqs = -16000 + np.arange(ndop) * 32000 / ndop
        raw = np.array([round(f * step * (spc / 5e6) * 5e6 / 1.57542e9) for f in freqs])
        srt = np.fft.fftshift(P, axes=0)
        ref = np.stack([np.roll(srt[r], raw[r]) for r in range(ndop)])
        fused = np.zeros_like(P)
        rows = np.arange(ndop)[:, None]
        fused[rows, (np.arange(spc)[None, :] + (raw % spc)[:, None]) % spc] += srt
        assert np.allclose(fused, ref)


# ---------------------------------------------------------------- numeric golden vector
def test_secondary_code_opt_out_golden_vector():
    # test/secondary_code_search.jl:89-131 (L5I, 10.24 MHz, N = 10, opt-out pilot path)
    gv = KA["l5i_optout_golden"]
    fs = 10.24e6
    primary = G.gen_code(10240, G.GPSL5I, 1, fs).astype(np.complex64)
    sig = np.concatenate([np.float32(G.NH10[k]) * primary for k in range(10)])
    plan = O.plan_acquire(G.GPSL5I, fs, [1], min_doppler_coverage=1000,
                          num_coherently_integrated_code_periods=10, use_secondary_code=False)
    nim = O.acquire_b(plan, sig, [1], store_power_bins=True)[0].power_bins
    assert nim.shape == tuple(gv["shape"])
    assert nim.max() == pytest.approx(gv["max"], rel=1e-4)
    assert nim.astype(np.float64).sum() == pytest.approx(gv["sum"], rel=1e-4)
    assert nim[0, 99] == pytest.approx(gv["nim_1_100"], rel=1e-4)
    assert nim[-1, -1] == pytest.approx(gv["nim_end_end"], rel=1e-4)
    am = np.unravel_index(np.argmax(nim), nim.shape)
    assert [int(am[0]) + 1, int(am[1]) + 1] in gv["argmax_1based_any_of"]
    assert nim[16, 0] == pytest.approx(nim[24, 0], rel=1e-3)


def test_rotation_discovery_every_phase():
    # test/secondary_code_search.jl:32-87: secondary_code_phase == r and peak_on > 5 peak_off
    fs = 10.24e6
    primary = G.gen_code(10240, G.GPSL5I, 1, fs).astype(np.complex64)
    plan = O.plan_acquire(G.GPSL5I, fs, [1], min_doppler_coverage=1000,
                          num_coherently_integrated_code_periods=10)
    plan_off = O.plan_acquire(G.GPSL5I, fs, [1], min_doppler_coverage=1000,
                              num_coherently_integrated_code_periods=10, use_secondary_code=False)
    ref = np.concatenate([np.float32(G.NH10[k]) * primary for k in range(10)])
    peak_off = O.acquire_b(plan_off, ref, [1], store_power_bins=True)[0].power_bins.max()
    for r in range(10):
        sig = np.concatenate([np.float32(G.NH10[(k + r) % 10]) * primary for k in range(10)])
        res = O.acquire_b(plan, sig, [1], store_power_bins=True)[0]
        assert res.power_bins.max() > 5 * peak_off
        assert res.secondary_code_phase == r


def test_rotation_multi_symbol_data_flip():
    # test/secondary_code_search.jl:194-258 (N = 20 = 2L, data flip between symbols)
    fs, N, L, true_cp, fd = 12e6, 20, 10, 1234.5, 1000.0
    primary = G.gen_code(12000, G.GPSL5I, 1, fs, start_phase=true_cp).astype(np.complex64)
    sig = np.concatenate([np.float32(G.NH10[k % L] * (1 if k < L else -1)) * primary for k in range(N)])
    sig = (sig * np.exp(1j * 2 * np.pi * fd / fs * np.arange(len(sig)))).astype(np.complex64)
    plan = O.plan_acquire(G.GPSL5I, fs, [1], num_coherently_integrated_code_periods=N)
    assert plan.num_secondary_rotations == L and plan.num_data_bits == 2
    res = O.acquire_b(plan, sig, [1])[0]
    assert O.is_detected(res)
    assert abs(res.code_phase - true_cp) < 1.0
    assert abs(res.carrier_doppler - fd) < plan.doppler_step
    assert res.secondary_code_phase == 0
    assert res.sign_pattern == 1          # second symbol flipped relative to the first


# ---------------------------------------------------------------- end to end (tolerances)
def _test_signal(system, prn, n, fs, doppler, cp, cn0, seed, interm_freq=0.0):
    # src/generate_test_signal.jl:45-68 model (unit_noise_power = false)
    rng = np.random.default_rng(seed)
    noise = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)   # Julia randn(ComplexF64)
    return (O.clean_signal(system, prn, n, fs, doppler, cp, interm_freq, amplitude=10 ** (cn0 / 20))
            + noise * 10 ** (10 * math.log10(fs) / 20))


def test_acquire_strong_signal():
    # test/acquire.jl:3-21
    sig = _test_signal(G.GPSL1CA, 1, 2048, 2.048e6, 1000.0, 200.0, 45, 1)
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [1])
    r = O.acquire_b(plan, sig, [1])[0]
    assert abs(r.code_phase - 200.0) < 1.0 and O.is_detected(r)


def test_acquire_multistep_weak_signal():
    # test/acquire.jl:23-46
    sig = _test_signal(G.GPSL1CA, 3, 40 * 2048, 2.048e6, 500.0, 100.0, 30, 7777)
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [3], num_coherently_integrated_code_periods=20,
                          num_noncoherent_accumulations=2)
    r = O.acquire_b(plan, sig, [3])[0]
    assert O.is_detected(r) and abs(r.code_phase - 100.0) < 2.0


def test_acquire_interpolation_and_if():
    # test/acquire.jl:48-99
    sig = _test_signal(G.GPSL1CA, 2, 2048, 2.048e6, 0.0, 300.7, 45, 5555)
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [2])
    rg = O.acquire_b(plan, sig, [2])[0]
    ri = O.acquire_b(plan, sig, [2], subsample_interpolation=True)[0]
    assert abs(rg.code_phase - 300.7) < 2.0 and abs(ri.code_phase - 300.7) <= abs(rg.code_phase - 300.7) + 0.5
    sig = _test_signal(G.GPSL1CA, 5, 2048, 2.048e6, 500.0, 150.0, 45, 3333, interm_freq=1000.0)
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [5])
    r = O.acquire_b(plan, sig, [5], interm_freq=1000.0)[0]
    assert abs(r.code_phase - 150.0) < 1.5


def test_acquire_argument_errors():
    # test/acquire.jl:232-242
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [1, 2])
    with pytest.raises(O.ArgumentError):
        O.acquire_b(plan, np.zeros(2048, np.complex64), [3])
    with pytest.raises(O.ArgumentError):
        O.acquire_b(plan, np.zeros(100, np.complex64), [1])


def test_fp32_oracle_against_fp64_oracle():
    # FP32 error of the restated pipeline against its FP64 twin on a cfg-1-like case.
    sig = _test_signal(G.GPSL1CA, 1, 4000, 4e6, 1234.0, 300.5, 45, 11)
    p32 = O.plan_acquire(G.GPSL1CA, 4e6, [1, 2], precision="f32")
    p64 = O.plan_acquire(G.GPSL1CA, 4e6, [1, 2], precision="f64")
    r32, s32 = O.acquire_b(p32, sig, [1, 2], return_surfaces=True)
    r64, s64 = O.acquire_b(p64, sig, [1, 2], return_surfaces=True)
    for a, b, sa, sb in zip(r32, r64, s32, s64):
        rel = np.abs(sa.power - sb.power).max() / sb.power.max()
        assert rel < 1e-5
        assert (a.peak_doppler_bin, a.peak_code_bin) == (b.peak_doppler_bin, b.peak_code_bin)


def test_cn0_is_per_hz_independent_of_coherent_length():
    # test/acquire.jl:462-520: C/N0 divides the coherent time back out, so the estimate does not
    # climb with num_coherently_integrated_code_periods (mean over 8 code phases, detected trials)
    fs, true_cn0 = 4e6, 45
    reported = []
    for n in (1, 2, 4, 5, 10):
        plan = O.plan_acquire(G.GPSL1CA, fs, [1], num_coherently_integrated_code_periods=n,
                              min_doppler_coverage=25_000.0)
        est = []
        for k in range(1, 9):
            sig = _test_signal(G.GPSL1CA, 1, 4000 * n + 100, fs, 1234.0, (k - 0.5) * 1023 / 8 + 0.137, true_cn0,
                               700 + k)
            r = O.acquire_b(plan, sig, [1], subsample_interpolation=True)[0]
            if O.is_detected(r):
                est.append(r.CN0)
        assert len(est) >= 5, n
        reported.append(sum(est) / len(est))
    assert all(abs(c - true_cn0) <= 6.0 for c in reported), reported
    assert max(reported) - min(reported) < 4.0, reported
    assert reported[-1] - reported[0] < 2.0, reported


def test_peak_to_noise_ratio_consistent_with_cn0():
    # test/cfar.jl:117-133: a stronger signal has both the larger PNR and the larger C/N0
    plan = O.plan_acquire(G.GPSL1CA, 2.048e6, [1])
    strong = O.acquire_b(plan, _test_signal(G.GPSL1CA, 1, 2048, 2.048e6, 1000.0, 200.0, 55, 11), [1])[0]
    weak = O.acquire_b(plan, _test_signal(G.GPSL1CA, 1, 2048, 2.048e6, 1000.0, 200.0, 35, 11), [1])[0]
    assert strong.peak_to_noise_ratio > weak.peak_to_noise_ratio
    assert strong.CN0 > weak.CN0


@pytest.mark.parametrize("n_coh,flipped", [(40, [(20, 40)]), (60, [(20, 40)])])
def test_bit_transitions_at_zero_doppler_keep_the_peak(n_coh, flipped):
    # test/noncoherent_integration.jl:602-701: data bits +1 -1 (40 ms) and +1 -1 +1 (60 ms) at 0 Hz;
    # the data-bit search recovers the peak of the same signal without transitions (rtol 0.1) and
    # the pattern it picks flips the second bit against the first
    fs = 2.048e6
    clean = _test_signal(G.GPSL1CA, 1, n_coh * 2048, fs, 0.0, 0.0, 60, 42)
    sig = clean.copy()
    for a, b in flipped:
        sig[a * 2048:b * 2048] *= -1
    plan = O.plan_acquire(G.GPSL1CA, fs, [1], min_doppler_coverage=10_000.0,
                          num_coherently_integrated_code_periods=n_coh)
    assert plan.num_data_bits == n_coh // 20
    ref = O.acquire_b(plan, clean, [1])[0]
    got = O.acquire_b(plan, sig, [1])[0]
    assert got.peak_power == pytest.approx(ref.peak_power, rel=0.1)
    assert (got.peak_doppler_bin, got.peak_code_bin) == (ref.peak_doppler_bin, ref.peak_code_bin)
    assert ref.sign_pattern == 0 and got.sign_pattern != 0


def test_multistep_two_prns_planted_and_absent():
    # test/acquire.jl:137-156: the multistep path over two PRNs finds the planted one and not the other
    fs = 2.048e6
    plan = O.plan_acquire(G.GPSL1CA, fs, [1, 2], num_noncoherent_accumulations=2)
    sig = _test_signal(G.GPSL1CA, 1, 2 * 2048, fs, 800.0, 150.0, 45, 13).astype(np.complex64)
    r1, r2 = O.acquire_b(plan, sig, [1, 2])
    assert O.is_detected(r1) and abs(r1.code_phase - 150.0) <= 1.5
    assert not O.is_detected(r2)


def test_one_step_and_two_step_paths_agree():
    # test/acquire.jl:158-195: one segment at N_nc = 1 and two at N_nc = 2 give the same decisions
    # (48 dB-Hz instead of the reference's 45: over 1 ms, 45 dB-Hz is detected in 3 of 5 seeds of
    # this noise generator, 48 dB-Hz in all of them)
    fs, cp, dop = 2.048e6, 100.0, 1500.0
    sig = _test_signal(G.GPSL1CA, 1, 2 * 2048, fs, dop, cp, 48, 123).astype(np.complex64)
    p1 = O.plan_acquire(G.GPSL1CA, fs, [1])
    p2 = O.plan_acquire(G.GPSL1CA, fs, [1], num_noncoherent_accumulations=2)
    for plan, x in ((p1, sig[:2048]), (p2, sig)):
        r = O.acquire_b(plan, x, [1])[0]
        step = r.dopplers[1] - r.dopplers[0]
        assert O.is_detected(r) and abs(r.code_phase - cp) < 1.0 and abs(r.carrier_doppler - dop) < step


def test_sign_search_reports_the_doppler_without_a_half_band_offset():
    # test/acquire.jl:197-230: with two data bits the reported Doppler lies within one bin of the truth
    fs, cp, dop = 2.048e6, 100.0, 500.0
    plan = O.plan_acquire(G.GPSL1CA, fs, [1], num_coherently_integrated_code_periods=40)
    assert plan.num_data_bits == 2
    r = O.acquire_b(plan, _test_signal(G.GPSL1CA, 1, 40 * 2048, fs, dop, cp, 45, 31).astype(np.complex64), [1])[0]
    step = r.dopplers[1] - r.dopplers[0]
    assert O.is_detected(r) and abs(r.code_phase - cp) <= 1.0 and abs(r.carrier_doppler - dop) < step


@pytest.mark.parametrize("cov,n_coh,dop,cp", [(10_000.0, 40, 0.0, 333.0), (20_000.0, 10, 1500.0, 100.0)])
def test_doppler_grids_above_320_bins(cov, n_coh, dop, cp):
    # test/acquire.jl:290-341: more than 320 Doppler bins (the reference's per-column FFT branches)
    fs = 2.048e6
    plan = O.plan_acquire(G.GPSL1CA, fs, [1], min_doppler_coverage=cov, num_coherently_integrated_code_periods=n_coh)
    assert plan.num_doppler_bins > 320
    r = O.acquire_b(plan, _test_signal(G.GPSL1CA, 1, n_coh * 2048, fs, dop, cp, 45, 17).astype(np.complex64), [1])[0]
    assert O.is_detected(r) and abs(r.code_phase - cp) < 1.0


def test_global_mean_estimator_on_the_one_step_path():
    # test/acquire.jl:355-386: same peak as the opposite-row estimator, a different noise power, and
    # the global mean of the stored surface outside +-floor(fs/fc) columns of the peak
    # (src/est_signal_noise_power.jl:150-170)
    fs = 2.048e6
    sig = _test_signal(G.GPSL1CA, 4, 2048, fs, 750.0, 512.0, 45, 21).astype(np.complex64)
    pg = O.plan_acquire(G.GPSL1CA, fs, [4], noise_estimator="global_mean")
    po = O.plan_acquire(G.GPSL1CA, fs, [4])
    rg = O.acquire_b(pg, sig, [4])[0]
    ro = O.acquire_b(po, sig, [4])[0]
    assert O.is_detected(rg)
    assert (rg.code_phase, rg.carrier_doppler) == (ro.code_phase, ro.carrier_doppler)
    assert rg.noise_power != ro.noise_power
    rs = O.acquire_b(pg, sig, [4], store_power_bins=True)[0]
    P = rs.power_bins.astype(np.float64)
    half = int(fs // G.GPSL1CA.code_freq)
    keep = np.ones(P.shape[1], bool)
    keep[max(0, rs.peak_code_bin - half):min(P.shape[1], rs.peak_code_bin + half + 1)] = False
    assert rs.noise_power == pytest.approx(P[:, keep].sum() / (keep.sum() * P.shape[0]), rel=1e-6)


def test_multistep_interpolation_and_stored_surface():
    # test/acquire.jl:435-460: N_nc = 4 with interpolation and the stored surface, reproducible
    fs, cp = 2.048e6, 700.4
    plan = O.plan_acquire(G.GPSL1CA, fs, [1], num_noncoherent_accumulations=4)
    sig = _test_signal(G.GPSL1CA, 1, 4 * 2048, fs, 500.0, cp, 42, 8).astype(np.complex64)
    r = O.acquire_b(plan, sig, [1], subsample_interpolation=True, store_power_bins=True)[0]
    assert O.is_detected(r) and abs(r.code_phase - cp) <= 1.0
    assert r.power_bins.shape == (plan.num_doppler_bins, plan.samples_per_code_eff)
    r2 = O.acquire_b(plan, sig, [1], subsample_interpolation=True, store_power_bins=True)[0]
    assert np.array_equal(r2.power_bins, r.power_bins)


@pytest.mark.parametrize("M,n_coh,cn0", [(2, 4, 40), (4, 4, 38), (8, 1, 42)])
def test_weak_signal_passes_the_noncoherent_threshold(M, n_coh, cn0):
    # test/cfar.jl:91-115: with M > 1 accumulations a real signal still clears the CFAR threshold
    fs = 2.048e6
    plan = O.plan_acquire(G.GPSL1CA, fs, list(range(1, 33)), num_coherently_integrated_code_periods=n_coh,
                          num_noncoherent_accumulations=M)
    sig = _test_signal(G.GPSL1CA, 7, n_coh * 2048 * M, fs, 500.0, 100.0, cn0, 9999 + M).astype(np.complex64)
    r = O.acquire_b(plan, sig, [7])[0]
    assert O.is_detected(r, pfa=0.01) and abs(r.code_phase - 100.0) < 1.0


def test_l5i_gain_recovery_over_the_opt_out():
    # test/secondary_code_search.jl:133-175: the rotation search recovers more than 8x the peak power
    # of the search without the secondary code (theory 25x; the opt-out picks its best misalignment)
    fs = 10.24e6
    primary = G.gen_code(10240, G.GPSL5I, 1, fs).astype(np.complex64)
    sig = np.concatenate([np.float32(G.NH10[k]) * primary for k in range(10)])
    peaks = []
    for use in (True, False):
        plan = O.plan_acquire(G.GPSL5I, fs, [1], min_doppler_coverage=5000.0, num_coherently_integrated_code_periods=10,
                              use_secondary_code=use)
        peaks.append(O.acquire_b(plan, sig, [1], store_power_bins=True)[0].power_bins.max())
    assert peaks[0] / peaks[1] > 8


@pytest.mark.parametrize("cp,dop,n_nc", [(1234.5, 1000.0, 1), (5115.0, 1000.0, 1), (1234.5, 5000.0, 4)])
def test_l5i_rotation_search_code_phase_and_doppler(cp, dop, n_nc):
    # test/secondary_code_search.jl:177-206,294-386: the rotation search reports the Doppler without a
    # half-band offset, also at the worst-case code phase (5115 chips: the primary-code wrap in the
    # middle of a block) and with the code drift of four accumulation steps
    fs = 12e6
    plan = O.plan_acquire(G.GPSL5I, fs, [1], num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=n_nc)
    assert plan.num_secondary_rotations == 10
    sig = _test_signal(G.GPSL5I, 1, n_nc * 10 * 12000, fs, dop, cp, 45, 29).astype(np.complex64)
    r = O.acquire_b(plan, sig, [1])[0]
    assert O.is_detected(r)
    assert abs(r.code_phase - cp) <= (1.5 if n_nc > 1 else 1.0)
    assert abs(r.carrier_doppler - dop) < plan.doppler_step


@pytest.mark.parametrize("r0", [0, 3, 7, 9])
def test_secondary_code_phase_exact_across_code_phase_and_doppler(r0):
    # test/secondary_code_search.jl:260-292: the despread estimate is exact at every code phase
    # (including the 5115-chip worst case) and Doppler
    fs = 12e6
    plan = O.plan_acquire(G.GPSL5I, fs, [1], num_coherently_integrated_code_periods=10)
    for cp in (0.0, 2000.0, 5115.0, 9000.0):
        primary = G.gen_code(12000, G.GPSL5I, 1, fs, start_phase=cp).astype(np.complex64)
        base = np.concatenate([np.float32(G.NH10[(k + r0) % 10]) * primary for k in range(10)])
        for dop in (0.0, 1300.0):
            sig = base if dop == 0.0 else (base * np.exp(2j * np.pi * dop / fs * np.arange(len(base)))).astype(np.complex64)
            assert O.acquire_b(plan, sig, [1])[0].secondary_code_phase == r0, (cp, dop)
