"""The coherent tile as a time-domain correlation GEMM on the tensor cores (ACQ_OPT_TILE_MMA)
against the FP32 FFT tile and the FP64 oracle.

The GEMM multiplies exact FP16 code samples with the signal split into FP16 hi + lo (22
significant bits) and accumulates in FP32, so its surfaces agree with the FFT tile's within FP32
rounding: decisions equal, |P_mma - P_fft| <= 2e-6 of the surface peak, noise power and
peak-to-noise ratio within 1e-5.
"""
import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import synth
from oracle import acq_oracle as O
from oracle import gnss_codes as G

pytestmark = pytest.mark.gpu
OPT_TILE_MMA = 11
RTOL = 2e-6


def _surfaces(plan, x, prns, **kw):
    res = A.acquire_b(plan, x, prns, store_power_bins=True, **kw)
    return [(r.peak_doppler_bin, r.peak_code_bin, float(r.noise_power), float(r.peak_to_noise_ratio),
             np.asarray(r.power_bins).copy()) for r in res]


def _compare(a_list, b_list, label):
    for a, b in zip(a_list, b_list):
        assert a[:2] == b[:2], label
        assert a[2] == pytest.approx(b[2], rel=1e-5), label
        assert a[3] == pytest.approx(b[3], rel=1e-5), label
        assert np.abs(a[4] - b[4]).max() <= RTOL * b[4].max(), (label, np.abs(a[4] - b[4]).max() / b[4].max())


def _both(plan, x, prns, **kw):
    assert plan.get_option(OPT_TILE_MMA) == 1
    got = _surfaces(plan, x, prns, **kw)
    assert plan.set_option(OPT_TILE_MMA, 0) == 0
    ref = _surfaces(plan, x, prns, **kw)
    assert plan.set_option(OPT_TILE_MMA, 1) == 1
    return got, ref


@pytest.mark.parametrize("quant", ["ci16", "ci8", None])
def test_tile_mma_matches_the_fft_tile(quant):
    # L1 C/A 5 MHz, 10 ms x 2 (first Doppler pass on the time-domain rows); 10 PRNs = 200 code
    # rows, two blocks of 128 rows, the second one partly empty
    sats = [synth.Satellite(3, 44.0, 1500.0, 200.25), synth.Satellite(9, 40.0, -2200.0, 800.5)]
    prns = list(range(1, 11))
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)
    x = synth.synth(A.GPSL1CA(), 5e6, 100_000, sats, 4)
    x = synth.to_ci16(x) if quant == "ci16" else synth.to_ci8_3bit(x) if quant == "ci8" else x.astype(np.complex64)
    got, ref = _both(plan, x, prns)
    _compare(got, ref, quant)


@pytest.mark.parametrize("fs", [2.5e6, 3.2e6])
def test_tile_mma_block_sizes(fs):
    # 2.5 MHz: block size 125 (odd; one lag half of 128, 8 K steps); 3.2 MHz: block size 200
    # (two lag halves, 13 K steps)
    sats = [synth.Satellite(6, 45.0, 700.0, 333.25)]
    prns = [6, 7, 8]
    plan = A.plan_acquire(A.GPSL1CA(), fs, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=2, num_noncoherent_accumulations=2)
    assert plan.geometry.block_size == {2.5e6: 125, 3.2e6: 200}[fs]
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), fs, 4 * plan.samples_per_code, sats, 3))
    got, ref = _both(plan, x, prns)
    _compare(got, ref, fs)


def test_tile_mma_with_an_intermediate_frequency_and_one_coherent_period():
    # 4 MHz, 1 ms, IF 100 kHz: the operand kernel wipes the IF off per sample like the front end
    sats = [synth.Satellite(1, 45.0, 1234.0, 300.5)]
    prns = [1, 2, 3]
    plan = A.plan_acquire(A.GPSL1CA(), 4e6, prns, min_doppler_coverage=7000)
    x = synth.synth(A.GPSL1CA(), 4e6, 4000, sats, 2, interm_freq=100e3).astype(np.complex64)
    got, ref = _both(plan, x, prns, interm_freq=100e3)
    _compare(got, ref, "if")


def test_tile_mma_without_the_first_pass_on_the_rows(monkeypatch):
    # ACQ_NO_PREPASS: rows are the plain blocks and the column stage runs the whole Doppler FFT
    monkeypatch.setenv("ACQ_NO_PREPASS", "1")
    sats = [synth.Satellite(7, 44.0, -800.0, 1200.5)]
    prns = [7, 8]
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=2, num_noncoherent_accumulations=2)
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 5e6, 20_000, sats, 5))
    got, ref = _both(plan, x, prns)
    _compare(got, ref, "no-prepass")


def test_tile_mma_many_prns_and_a_subset():
    # 32 PRNs = 640 code rows (five full blocks), then a request for 3 of them (one partial block)
    sats = [synth.Satellite(12, 44.0, 900.0, 4000.25), synth.Satellite(30, 42.0, -3100.0, 10.5)]
    prns = list(range(1, 33))
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=2, num_noncoherent_accumulations=3)
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 5e6, 30_000, sats, 6))
    got, ref = _both(plan, x, prns)
    _compare(got, ref, "32")
    sub = [30, 12, 5]
    got, ref = _both(plan, x, sub)
    _compare(got, ref, "subset")


def test_tile_mma_per_step_for_the_bit_edge_search():
    # data-bit / bit-edge search (40 ms, 2 data bits, 4 edges): one tile launch per step
    sats = [synth.Satellite(5, 44.0, 1200.0, 512.5)]
    prns = [5, 6, 7]
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=40, bit_edge_search_steps=4)
    assert plan.geometry.path == 1
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 5e6, 40 * 5000, sats, 21))
    got, ref = _both(plan, x, prns)
    _compare(got, ref, "bit-edge")


def test_tile_mma_per_step_for_the_rotation_search():
    # secondary-code rotation search (L5I 5 MHz, 10 ms x 2, CI8): one tile launch per step
    sats = [synth.Satellite(7, 47.0, 3300.0, 9000.5)]
    prns = [7, 8]
    plan = A.plan_acquire(A.GPSL5I(), 5e6, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)
    assert plan.geometry.path == 2
    x = synth.to_ci8_3bit(synth.synth(A.GPSL5I(), 5e6, 2 * 10 * 5000, sats, 22))
    got, ref = _both(plan, x, prns)
    _compare(got, ref, "rotation")


def test_tile_mma_against_the_fp64_oracle():
    sats = [synth.Satellite(3, 43.0, 1500.0, 200.25)]
    prns = [3, 4]
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, prns, min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)
    assert plan.get_option(OPT_TILE_MMA) == 1
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 5e6, 100_000, sats, 9))
    osig = (x[:, 0].astype(np.float32) + 1j * x[:, 1].astype(np.float32)).astype(np.complex64)
    res = A.acquire_b(plan, x, prns, store_power_bins=True)
    op = O.plan_acquire(G.GPSL1CA, 5e6, prns, min_doppler_coverage=5000, num_coherently_integrated_code_periods=10,
                        num_noncoherent_accumulations=2, precision="f64")
    r64, s64 = O.acquire_b(op, osig, prns, return_surfaces=True)
    for g, b, sb in zip(res, r64, s64):
        p64 = sb.power
        err = np.abs(np.asarray(g.power_bins, dtype=np.float64) - p64).max() / p64.max()
        print("tile MMA vs FP64 oracle", g.prn, err)
        assert err <= 1e-5
        assert (g.peak_doppler_bin, g.peak_code_bin) == (b.peak_doppler_bin, b.peak_code_bin)


def test_tile_mma_option():
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, [1], min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=2)
    assert plan.get_option(OPT_TILE_MMA) == 1
    with pytest.raises(A.ArgumentError):
        plan.set_option(OPT_TILE_MMA, 2)
    # block size above 256: the FFT tile only
    big = A.plan_acquire(A.GalileoE1B(), 12e6, [1], min_doppler_coverage=8000)
    assert big.geometry.block_size > 256
    assert big.get_option(OPT_TILE_MMA) == 0
    assert big.set_option(OPT_TILE_MMA, 1) == 0
