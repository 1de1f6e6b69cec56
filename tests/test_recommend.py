"""Sampling-frequency recommendation against the reference's tests
(test/recommend_sampling_freq.jl) — host only."""
import pytest

import acqgb300 as A
from acqgb300 import recommend as R


def test_code_length_code_freq_form():
    rs = R.recommend_sampling_freqs(10_000, 36e6, fs_min=36e6, fs_max=40e6, min_doppler_coverage=10_000,
                                    num_coherently_integrated_code_periods=36, num_alternatives=5, max_prime=7,
                                    sort_by="cost", fs_step=1000)
    assert 0 < len(rs) <= 5
    for r in rs:
        assert r.inner_max_prime <= 7 and r.num_doppler_bins_max_prime <= 7
        assert r.samples_per_code % r.num_blocks == 0 and r.block_size == r.samples_per_code // r.num_blocks
        assert r.inner_fft_size == R.nextprod_2357(2 * r.block_size) >= 2 * r.block_size
        assert r.num_doppler_bins == 36 * r.num_blocks and r.doppler_coverage >= 2 * 10_000
    costs = [r.cost for r in rs]
    assert costs == sorted(costs)


def test_smoothness_sort():
    rs = R.recommend_sampling_freqs(10_000, 36e6, fs_min=36e6, fs_max=40e6, min_doppler_coverage=10_000,
                                    num_coherently_integrated_code_periods=36, sort_by="smoothness")
    primes = [r.num_doppler_bins_max_prime for r in rs]
    assert rs and primes == sorted(primes)


def test_column_fft_is_the_only_gate():
    rs = R.recommend_for_system(A.GPSL1CA(), fs_min=16.36e6, fs_max=16.40e6, min_doppler_coverage=7000,
                                num_alternatives=20)
    assert 16_368_000 in [round(r.sampling_freq) for r in rs]
    rs2 = R.recommend_for_system(A.GPSL1CA(), fs_min=1.540e6, fs_max=1.545e6, min_doppler_coverage=7000,
                                 num_alternatives=20)
    assert all(round(r.sampling_freq) != 1_542_000 for r in rs2)


def test_system_form_and_geometry_agrees_with_plan():
    rs = R.recommend_for_system(A.GPSL1CA(), fs_min=2e6, fs_max=5e6, min_doppler_coverage=7000, num_alternatives=3)
    assert 0 < len(rs) <= 3
    r = rs[0]
    assert r.samples_per_code == -(-int(r.sampling_freq) // 1000)
    g = A.plan_geometry(A.GPSL1CA(), r.sampling_freq, min_doppler_coverage=7000)
    assert (g.num_blocks, g.block_size, g.fft_size, g.num_doppler_bins) == (r.num_blocks, r.block_size,
                                                                               r.inner_fft_size, r.num_doppler_bins)
    assert len(R.recommend_for_system(A.GPSL1CA(), fs_min=2e6, fs_max=10e6, num_alternatives=2)) <= 2


@pytest.mark.parametrize("kw", [dict(sort_by="nonsense"), dict(num_alternatives=0), dict(max_prime=1),
                                dict(num_coherently_integrated_code_periods=0), dict(fs_min=5e6, fs_max=1e6),
                                dict(fs_step=0)])
def test_argument_validation(kw):
    with pytest.raises(A.ArgumentError):
        R.recommend_sampling_freqs(1023, 1.023e6, **kw)


def test_factor_string():
    f = R.factor_string
    assert [f(1), f(2), f(8), f(744), f(2048), f(10080)] == ["1", "2", "2³", "2³·3·31", "2¹¹", "2⁵·3²·5·7"]
