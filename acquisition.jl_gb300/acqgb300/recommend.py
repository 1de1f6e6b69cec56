"""Sampling-frequency recommendation (src/recommend_sampling_freq.jl:118,196-307), with the
reference's FFT cost model and, on request, the acquisition time measured on the GPU.

``recommend_sampling_freqs`` sweeps [fs_min, fs_max] in fs_step, mirrors plan_acquire's geometry
(smallest valid num_blocks, inner FFT padded to a 7-smooth size, column FFT = num_doppler_bins)
and keeps candidates whose column FFT is ``max_prime``-smooth, ranked by
cost = 2 nb F log2 F + spc ndop log2 ndop (``sort_by="cost"``) or by smoothness. With
``measure=...`` the best candidates are re-ranked by the measured time of one acquisition on
the GPU (plan, device-generated noise recording, CUDA events); hardware sample-rate plans
(SDR clock plans) are not modelled.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field


@dataclass
class SamplingFreqRecommendation:
    sampling_freq: float
    samples_per_code: int
    num_blocks: int
    block_size: int
    inner_fft_size: int
    num_doppler_bins: int
    doppler_coverage: float
    inner_max_prime: int
    num_doppler_bins_max_prime: int
    cost: float
    measured_ms: float | None = field(default=None)


def prime_factors(n: int) -> list:
    if n <= 1:
        return []
    out, p = [], 2
    while p * p <= n:
        while n % p == 0:
            out.append(p)
            n //= p
        p += 1
    if n > 1:
        out.append(n)
    return out


def largest_prime_factor(n: int) -> int:
    f = prime_factors(n)
    return max(f) if f else 1


_SUP = "⁰¹²³⁴⁵⁶⁷⁸⁹"


def factor_string(n: int) -> str:
    """2³·3·31 style factorisation (src/recommend_sampling_freq.jl:63-79)."""
    if n <= 1:
        return str(n)
    counts = {}
    for p in prime_factors(n):
        counts[p] = counts.get(p, 0) + 1
    return "·".join(str(p) + ("".join(_SUP[int(d)] for d in str(k)) if k > 1 else "") for p, k in sorted(counts.items()))


def nextprod_2357(n: int) -> int:
    m = max(1, int(n))
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def _smallest_valid_num_blocks(spc: int, min_num_blocks: int):
    for d in range(max(1, min_num_blocks), spc + 1):
        if spc % d == 0:
            return d
    return None


def fft_cost(spc: int, nb: int, ndop: int, inner: int) -> float:
    return 2.0 * nb * inner * math.log2(inner) + float(spc) * ndop * math.log2(ndop)


def recommend_sampling_freqs(code_length: int, code_freq: float, *, fs_min=None, fs_max=None,
                             min_doppler_coverage: float = 7000.0, num_coherently_integrated_code_periods: int = 1,
                             num_alternatives: int = 5, max_prime: int = 7, sort_by: str = "cost",
                             fs_step: float = 1000.0, measure=None, measure_top: int = 8):
    """src/recommend_sampling_freq.jl:196-290. ``measure``: a GNSSSystem to time the best
    ``measure_top`` candidates on the GPU (acquisition of 32 PRNs, or the system's count), which
    then re-ranks them by measured time."""
    from .api import ArgumentError
    if sort_by not in ("cost", "smoothness"):
        raise ArgumentError(f"sort_by must be :cost or :smoothness, got :{sort_by}")
    if num_alternatives < 1:
        raise ArgumentError("num_alternatives must be >= 1")
    if max_prime < 2:
        raise ArgumentError("max_prime must be >= 2")
    if num_coherently_integrated_code_periods < 1:
        raise ArgumentError("num_coherently_integrated_code_periods must be >= 1")
    fs_min = float(code_freq) if fs_min is None else float(fs_min)
    fs_max = 1.5 * fs_min if fs_max is None else float(fs_max)
    if not fs_min <= fs_max:
        raise ArgumentError("fs_min must be <= fs_max")
    if not fs_step > 0:
        raise ArgumentError("fs_step must be > 0")
    n_coh = num_coherently_integrated_code_periods
    t_code = code_length / float(code_freq)
    seen, cands = set(), []
    fs = fs_min
    while fs <= fs_max:
        spc = math.ceil(t_code * fs)
        if spc not in seen:
            seen.add(spc)
            bin_width = fs / spc
            min_nb = math.ceil(2 * min_doppler_coverage / bin_width + 2 / n_coh)
            nb = _smallest_valid_num_blocks(spc, min_nb)
            if nb is not None:
                bs = spc // nb
                inner = nextprod_2357(2 * bs)
                ndop = n_coh * nb
                ndb_p = largest_prime_factor(ndop)
                if ndb_p <= max_prime:
                    cands.append(SamplingFreqRecommendation(fs, spc, nb, bs, inner, ndop, nb * bin_width,
                                                            largest_prime_factor(inner), ndb_p,
                                                            fft_cost(spc, nb, ndop, inner)))
        fs += fs_step
    if sort_by == "cost":
        cands.sort(key=lambda c: (c.cost, c.num_doppler_bins_max_prime))
    else:
        cands.sort(key=lambda c: (c.num_doppler_bins_max_prime, c.cost))
    if measure is None:
        return cands[:num_alternatives]
    top = cands[:max(num_alternatives, measure_top)]
    for c in top:
        c.measured_ms = measure_acquisition_ms(measure, c.sampling_freq, min_doppler_coverage, n_coh)
    top.sort(key=lambda c: c.measured_ms)
    return top[:num_alternatives]


def recommend_for_system(system, **kw):
    """src/recommend_sampling_freq.jl:301-307: code length and rate from the system."""
    kw.setdefault("fs_min", system.code_frequency)
    return recommend_sampling_freqs(system.code_length, system.code_frequency, **kw)


def measure_acquisition_ms(system, fs: float, min_doppler_coverage: float, n_coh: int, reps: int = 3) -> float:
    """Median device time (ms) of one acquisition over every PRN of the system at ``fs`` on a
    device-generated noise recording."""
    import statistics

    import torch

    from .api import acquire_device, acquire_device_async, fetch_results, plan_acquire
    from .batch import CONSTELLATION
    from .synth import synth_device
    prns = list(range(1, CONSTELLATION.get(system.name, 32) + 1))
    plan = plan_acquire(system, fs, prns, min_doppler_coverage=min_doppler_coverage,
                        num_coherently_integrated_code_periods=n_coh)
    x = synth_device(system, fs, n_coh * plan.samples_per_code, [], 1)
    stream = torch.cuda.ExternalStream(plan.stream_handle(), device=x.device)
    acquire_device(plan, x, prns)
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        acquire_device_async(plan, x, prns)
        e1.record(stream)
        fetch_results(plan, prns)
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)
