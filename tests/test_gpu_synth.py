"""Device signal generator (src/generate_test_signal.jl:32-82 model) against the host model, and
a ragged batch fed straight from it (no host round trip)."""
import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import batch as B
from acqgb300 import synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [(A.GPSL1CA(), 5e6, [synth.Satellite(3, 50.0, 1500.0, 200.25, 0.3, False)]),
         (A.GalileoE1B(), 12e6, [synth.Satellite(11, 48.0, -2500.0, 2000.75, 1.0, False)]),
         (A.GPSL5I(), 20e6, [synth.Satellite(4, 45.0, 3100.0, 4321.5, 2.0, False),
                             synth.Satellite(9, 42.0, -700.0, 10.25, 0.5, False)])]


@pytest.mark.parametrize("system,fs,sats", CASES, ids=["l1", "e1b", "l5i"])
def test_signal_matches_host_model(system, fs, sats):
    n = 100_000
    host = synth.synth(system, fs, n, sats, 1, interm_freq=1000.0, noise=False)
    dev = synth.synth_device(system, fs, n, sats, 1, interm_freq=1000.0, noise=False, dtype="cf64").cpu().numpy()
    assert np.max(np.abs(dev - host)) <= 1e-9 * np.max(np.abs(host))
    q_host = synth.to_ci16(host * 200)
    q_dev = synth.synth_device(system, fs, n, [synth.Satellite(s.prn, s.cn0 + 20 * np.log10(200), s.doppler,
                                                                 s.code_phase, s.phase, False) for s in sats],
                               1, interm_freq=1000.0, noise=False, dtype="ci16").cpu().numpy()
    assert np.mean(np.abs(q_dev.astype(int) - q_host.astype(int)) > 1) == 0.0


def test_noise_statistics_and_data_bits():
    n = 1_000_000
    x = synth.synth_device(A.GPSL1CA(), 5e6, n, [], 7, noise=True).cpu().numpy().astype(np.complex128)
    assert abs(x.real.mean()) < 3e-3 and abs(x.imag.mean()) < 3e-3
    assert x.real.var() == pytest.approx(0.5, rel=0.01) and x.imag.var() == pytest.approx(0.5, rel=0.01)
    assert abs(np.mean(x.real * x.imag)) < 3e-3
    # data bits: +-1 factors constant over each 20 ms bit (L1 C/A, 50 Hz), both signs present
    s_bits = [synth.Satellite(5, 60.0, 0.0, 0.0, 0.0, True, 0.0)]
    s_none = [synth.Satellite(5, 60.0, 0.0, 0.0, 0.0, False, 0.0)]
    m = 500_000                                   # 100 ms at 5 MHz = 5 bits
    a = synth.synth_device(A.GPSL1CA(), 5e6, m, s_bits, 3, noise=False, dtype="cf64").cpu().numpy()
    b = synth.synth_device(A.GPSL1CA(), 5e6, m, s_none, 3, noise=False, dtype="cf64").cpu().numpy()
    ratio = np.real(a / b).reshape(5, -1)
    assert np.all(np.abs(np.abs(ratio) - 1) < 1e-12)
    assert np.all(ratio == ratio[:, :1])


def test_ragged_batch_fed_from_the_device_generator():
    cache = B.PlanCache()
    recs = []
    rng = np.random.default_rng(11)
    for i, (system, fs, n_coh, cov) in enumerate([(A.GPSL1CA(), 5e6, 1, 8000.0), (A.GalileoE1B(), 12e6, 1, 8000.0),
                                                   (A.GPSL5I(), 25e6, 10, 8000.0), (A.GPSL1CA(), 5e6, 1, 8000.0)]):
        prn = int(rng.integers(1, 30))
        sat = synth.Satellite(prn, 50.0, float(rng.uniform(-6000, 6000)), float(rng.uniform(0, system.code_length)),
                              0.2, False)
        plan = cache.get(system, fs, n_coh=n_coh, n_nc=2, cov=cov)
        n = 2 * n_coh * plan.samples_per_code
        recs.append((plan, n, sorted({prn, prn + 1, prn + 2}), sat, system, fs))
    items = [B.BatchItem(p, np.zeros(n, np.complex64), prns) for p, n, prns, _, _, _ in recs]
    bt = B.AcquisitionBatch(items)
    for i, (p, n, prns, sat, system, fs) in enumerate(recs):
        synth.synth_device(system, fs, n, [sat], 100 + i, out=bt.input_ptr(i))
    torch.cuda.synchronize()
    bt.launch()
    out = bt.fetch()
    for (p, n, prns, sat, system, fs), res in zip(recs, out):
        r = {x.prn: x for x in res}[sat.prn]
        assert A.is_detected(r), (system.name, sat.prn)
        assert abs(r.carrier_doppler - sat.doppler) <= p.geometry.doppler_step_hz


def test_recommendation_with_measured_gpu_cost():
    from acqgb300 import recommend as R
    rs = R.recommend_for_system(A.GPSL1CA(), fs_min=2e6, fs_max=5e6, min_doppler_coverage=7000, num_alternatives=3,
                                measure=A.GPSL1CA(), measure_top=4)
    assert 0 < len(rs) <= 3
    ms = [r.measured_ms for r in rs]
    assert all(m is not None and m > 0 for m in ms) and ms == sorted(ms)
