"""Detection statistics of the whole CUDA path (acquire! through the C ABI), as the reference
tests them end to end:

* test/cfar.jl:54-89: on all-noise input, the false alarms of 50 trials x 32 PRNs against
  cfar_threshold(0.01, cells; M) stay within 3x the nominal count, for M = 2, 4, 8 one-code
  accumulations and M = 4 of four code periods;
* test/noncoherent_integration.jl:532-600: at C/N0 30 dB-Hz with 10 ms coherent integration,
  the detection probability rises from M = 1 (< 0.3) to M = 8 (> 0.7), the false-alarm rate
  of each stays below 3 pfa, and the M = 1 threshold applied to M = 8 results is the wrong one
  (it detects less often than the right one).
Noise is complex white Gaussian of unit power (randn(ComplexF64)); signals follow
src/generate_test_signal.jl (no data bits).
"""
import math

import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import synth

pytestmark = pytest.mark.gpu


def _cnoise(rng, n):
    return ((rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)).astype(np.complex64)


@pytest.mark.parametrize("M,num_code_cycles", [(2, 1), (4, 1), (8, 1), (4, 4)])
def test_cfar_false_alarm_rate_with_noncoherent_integration(M, num_code_cycles):
    fs, pfa, n_trials = 2.048e6, 0.01, 50
    prns = list(range(1, 33))
    plan = A.plan_acquire(A.GPSL1CA(), fs, prns, num_coherently_integrated_code_periods=num_code_cycles,
                          num_noncoherent_accumulations=M)
    seg_len = num_code_cycles * 2048 * M
    num_cells = plan.num_doppler_bins * plan.num_blocks * plan.block_size
    threshold = A.cfar_threshold(pfa, num_cells, num_noncoherent_integrations=M)
    rng = np.random.default_rng(0xC0FFEE + M * 1000 + num_code_cycles)
    false_alarms = 0
    for _ in range(n_trials):
        res = A.acquire_b(plan, _cnoise(rng, seg_len), prns)
        false_alarms += sum(float(r.peak_to_noise_ratio) > threshold for r in res)
    expected = n_trials * 32 * pfa
    print(f"[cfar M={M} n_coh={num_code_cycles}] false alarms {false_alarms} (nominal {expected:.0f}), "
          f"threshold {threshold:.4f}")
    assert false_alarms <= math.ceil(3 * expected)


def test_detection_probability_rises_with_noncoherent_integration():
    a = A.GPSL1CA()
    fs, prn, pfa, n_trials, n_coh = 2.048e6, 1, 0.01, 100, 10
    kw = dict(min_doppler_coverage=10000, num_coherently_integrated_code_periods=n_coh)
    plan1 = A.plan_acquire(a, fs, [prn], num_noncoherent_accumulations=1, **kw)
    plan8 = A.plan_acquire(a, fs, [prn], num_noncoherent_accumulations=8, **kw)
    n1, n8 = n_coh * 2048, 8 * n_coh * 2048
    sat = synth.Satellite(prn, 30.0, 1500.0, 100.0, data_bits=False)
    rng = np.random.default_rng(20260423)
    det1 = det8 = det8_wrong = fa1 = fa8 = 0
    for seed in range(1, n_trials + 1):
        s1 = synth.synth(a, fs, n1, [sat], seed).astype(np.complex64)
        s8 = synth.synth(a, fs, n8, [sat], seed).astype(np.complex64)
        r1 = A.acquire_b(plan1, s1, [prn])[0]
        r8 = A.acquire_b(plan8, s8, [prn])[0]
        det1 += A.is_detected(r1, pfa=pfa)
        det8 += A.is_detected(r8, pfa=pfa)
        thr1 = A.cfar_threshold(pfa, A.get_num_cells(r8), num_noncoherent_integrations=1)
        det8_wrong += float(r8.peak_to_noise_ratio) > thr1
        fa1 += A.is_detected(A.acquire_b(plan1, _cnoise(rng, n1), [prn])[0], pfa=pfa)
        fa8 += A.is_detected(A.acquire_b(plan8, _cnoise(rng, n8), [prn])[0], pfa=pfa)
    pd1, pd8, pd8w = det1 / n_trials, det8 / n_trials, det8_wrong / n_trials
    pfa1, pfa8 = fa1 / n_trials, fa8 / n_trials
    print(f"[pd] M=1 {pd1:.2f}  M=8 {pd8:.2f}  M=8 with the M=1 threshold {pd8w:.2f}  "
          f"false alarms M=1 {pfa1:.2f} M=8 {pfa8:.2f}")
    assert pd8 > pd1
    assert pd1 < 0.3
    assert pd8 > 0.7
    assert pfa1 < 3 * pfa
    assert pfa8 < 3 * pfa
    assert pd8w < pd8
