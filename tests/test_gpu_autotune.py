"""Launch shapes chosen by the autotuner move work between threads and CTAs; only the order of
the accumulation sums can change, so every shape gives the same decisions and power surfaces
within 1e-6 of the surface peak (the fused form, which accumulates in a different order, within
1e-5)."""
import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import autotune as T
from acqgb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
L_TILE_ROWS = 9
L_TILE_MMA = 11


def _case():
    sats = [synth.Satellite(3, 44.0, 1500.0, 200.25), synth.Satellite(9, 40.0, -2200.0, 800.5)]
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, list(range(1, 11)), min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 5e6, 100_000, sats, 4))
    return plan, x


def _run(plan, x):
    res = A.acquire_b(plan, x, list(range(1, 11)), store_power_bins=True)
    return [(r.peak_doppler_bin, r.peak_code_bin, r.peak_to_noise_ratio, np.asarray(r.power_bins).copy()) for r in res]


def test_shapes_give_the_same_results():
    plan, x = _case()
    assert plan.set_option(L_TILE_MMA, 0) == 0   # the FFT tile, whose knobs these shapes move
    start = T.current(plan)
    ref = _run(plan, x)
    shapes = [{"tile_threads": 64, "tile_blocks": 3, "tile_pad": 1},
              {"tile_threads": 256, "tile_blocks": 20, "tile_pad": 0},
              {"tile_rows": 2}, {"tile_rows": 2, "tile_threads": 256, "tile_blocks": 4},
              {"column_width": 8, "column_ctas_per_sm": 1}, {"column_width": 12}, {"column_width": 20},
              {"column_width": 24, "column_ctas_per_sm": 2}, {"column_width": 32}, {"form": "fused"}]
    for sh in shapes:
        eff = T.apply(plan, sh)
        got = _run(plan, x)
        tol = 1e-5 if sh.get("form") == "fused" else 1e-6
        for a, b in zip(ref, got):
            assert a[:2] == b[:2], (sh, eff)
            assert np.abs(a[3] - b[3]).max() <= tol * a[3].max(), (sh, eff)
        if "tile_threads" in sh or "tile_rows" in sh:     # the tile stage does not reorder sums: identical
            assert all(np.array_equal(a[3], b[3]) for a, b in zip(ref, got)), sh
        T.apply(plan, start)


def test_two_tile_rows_per_cta_with_an_odd_row_count():
    # 5 coherent periods: the last CTA of each code-block class holds one row, not two
    sats = [synth.Satellite(7, 46.0, -1300.0, 321.75)]
    plan = A.plan_acquire(A.GPSL1CA(), 5e6, [7, 8], min_doppler_coverage=5000,
                          num_coherently_integrated_code_periods=5, num_noncoherent_accumulations=3)
    assert plan.geometry.num_coherently_integrated_code_periods % 2 == 1
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 5e6, 90_000, sats, 11))
    if plan.get_option(L_TILE_ROWS) == 0:
        pytest.skip("no specialised tile kernel for this FFT size")
    ref = [np.asarray(r.power_bins).copy() for r in A.acquire_b(plan, x, [7, 8], store_power_bins=True)]
    assert plan.set_option(L_TILE_ROWS, 2) == 2
    got = [np.asarray(r.power_bins).copy() for r in A.acquire_b(plan, x, [7, 8], store_power_bins=True)]
    assert all(np.array_equal(a, b) for a, b in zip(ref, got))
    with pytest.raises(A.ArgumentError):
        plan.set_option(L_TILE_ROWS, 3)
    assert plan.get_option(L_TILE_ROWS) == 2


def test_doppler_first_pass_on_the_spectra_matches_the_column_fft(monkeypatch):
    # the first pass of the Doppler FFT (over the coherent periods) applied to the signal spectra
    # before the coherent tile, against the full FFT in the column stage: same decisions, power
    # surfaces within FP32 rounding
    ref_plan, x = _case()
    got = _run(ref_plan, x)
    monkeypatch.setenv("ACQ_NO_PREPASS", "1")
    plan, _ = _case()
    ref = _run(plan, x)
    for a, b in zip(ref, got):
        assert a[:2] == b[:2]
        assert np.abs(a[3] - b[3]).max() <= 1e-5 * a[3].max()


def test_doppler_group_column_stage_matches_the_full_tile_form(monkeypatch):
    # tiles of one Doppler group (nb rows x W columns) against tiles of all ndop rows: the same
    # sums per cell in the same step order, so the same decisions and surfaces within rounding
    plan, x = _case()
    got = _run(plan, x)
    assert plan.get_option(6) >= 8
    monkeypatch.setenv("ACQ_NO_COL_K1", "1")
    ref_plan, _ = _case()
    ref = _run(ref_plan, x)
    monkeypatch.delenv("ACQ_NO_COL_K1")   # read again whenever a plan's column shape is set up
    for a, b in zip(ref, got):
        assert a[:2] == b[:2]
        assert np.abs(a[3] - b[3]).max() <= 1e-6 * a[3].max()
    for w in (32, 64, 256):
        assert plan.set_option(6, w) == w
        for a, b in zip(ref, _run(plan, x)):
            assert a[:2] == b[:2], w
            assert np.abs(a[3] - b[3]).max() <= 1e-6 * a[3].max(), w


def test_column_widths_with_several_tma_boxes(monkeypatch):
    # 500 Doppler bins: a tile is loaded as several boxes of rows (at most 256 each), and each box
    # must start on a 128-byte boundary of the shared tile, which depends on the width (the full
    # column FFT, without the first pass on the spectra)
    monkeypatch.setenv("ACQ_NO_PREPASS", "1")
    sats = [synth.Satellite(5, 45.0, 2100.0, 1234.5)]
    plan = A.plan_acquire(A.GPSL1CA(), 12.5e6, [5, 6], min_doppler_coverage=16000,
                          num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)
    assert plan.num_doppler_bins == 500 and plan.geometry.fft_size == 500
    x = synth.to_ci16(synth.synth(A.GPSL1CA(), 12.5e6, 270_000, sats, 8))
    assert plan.get_option(6) == 16
    start = T.current(plan)
    ref = [(r.peak_doppler_bin, r.peak_code_bin, np.asarray(r.power_bins).copy())
           for r in A.acquire_b(plan, x, [5, 6], store_power_bins=True)]
    for w in (8, 12, 16):
        assert plan.set_option(6, w) == w
        got = A.acquire_b(plan, x, [5, 6], store_power_bins=True)
        for a, r in zip(ref, got):
            assert a[:2] == (r.peak_doppler_bin, r.peak_code_bin), w
            assert np.abs(a[2] - np.asarray(r.power_bins)).max() <= 1e-6 * a[2].max(), w
    # a width whose tiles exceed shared memory keeps the previous shape
    assert plan.set_option(6, 32) == 16
    T.apply(plan, start)


def test_tune_applies_and_caches(tmp_path):
    plan, x = _case()
    dev = torch.as_tensor(x, device="cuda")
    cache = str(tmp_path / "tune.json")
    out = T.tune(plan, dev, list(range(1, 11)), reps=1, passes=1, cache=cache)
    assert out["ms"] > 0 and out["trials"] >= 2
    assert T.current(plan)["tile_threads"] == out["settings"]["tile_threads"]
    entry = T.apply_cached(plan, str(dev.dtype), cache)
    assert entry is not None and entry["settings"] == out["settings"]


def test_option_validation():
    plan, _ = _case()
    with pytest.raises(A.ArgumentError):
        plan.set_option(3, 48)          # tile threads not a multiple of 32
    with pytest.raises(A.ArgumentError):
        plan.set_option(6, 13)          # column width odd
    with pytest.raises(A.ArgumentError):
        plan.set_option(6, 258)         # column width above 256
    assert plan.get_option(0) in (0, 1)


def test_repeated_requests_replay_the_same_results():
    # the second identical request captures the launch sequence as a CUDA graph and later ones
    # replay it; an option change or another input buffer leads back to a fresh capture
    plan, x = _case()
    dev = torch.as_tensor(x, device="cuda")
    runs = [A.acquire_device(plan, dev, list(range(1, 11)), store_power_bins=True) for _ in range(4)]
    ref = [(r.peak_doppler_bin, r.peak_code_bin, np.asarray(r.power_bins).copy()) for r in runs[0]]
    for out in runs[1:]:
        for a, r in zip(ref, out):
            assert a[:2] == (r.peak_doppler_bin, r.peak_code_bin)
            assert np.array_equal(a[2], np.asarray(r.power_bins))
    assert plan.set_option(4, 2) == 2          # tile blocks per round: same sums, new capture
    dev2 = dev.clone()                          # another input buffer
    for sig in (dev, dev, dev2, dev2, dev2):
        out = A.acquire_device(plan, sig, list(range(1, 11)), store_power_bins=True)
        for a, r in zip(ref, out):
            assert a[:2] == (r.peak_doppler_bin, r.peak_code_bin)
            assert np.array_equal(a[2], np.asarray(r.power_bins))
