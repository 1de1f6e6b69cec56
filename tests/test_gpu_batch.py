"""Ragged batches through one CUDA-graph launch agree with one acquire! per recording."""
import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import batch as B
from acqgb300 import synth

pytestmark = pytest.mark.gpu


def test_ragged_batch_matches_single_acquisitions():
    recs = synth.ragged_batch(seed=11, n_recordings=9, max_nnc=3)
    cache = B.PlanCache()
    items = B.batch_from_recordings(recs, cache)
    bt = B.AcquisitionBatch(items)
    assert bt.launch_count() > 0
    for rep in range(2):                       # the graph is replayed
        got = bt.run()
        for r, it, res in zip(recs, items, got):
            ref = A.acquire_b(it.plan, r["samples"], r["prns"])
            assert [x.prn for x in res] == r["prns"]
            for a, b in zip(res, ref):
                assert (a.peak_doppler_bin, a.peak_code_bin) == (b.peak_doppler_bin, b.peak_code_bin)
                assert A.is_detected(a) == A.is_detected(b)
                assert a.secondary_code_phase == b.secondary_code_phase
                assert float(a.noise_power) == pytest.approx(float(b.noise_power), rel=1e-5)
                assert float(a.peak_to_noise_ratio) == pytest.approx(float(b.peak_to_noise_ratio), rel=1e-5)
    bt.close()


def test_batch_upload_from_pinned_memory():
    # page-locked recordings go through the k_copy_in gather, one launch for every item; the
    # results equal those of the same recordings in pageable memory (copy engines)
    import torch
    recs = synth.ragged_batch(seed=13, n_recordings=6, max_nnc=2)
    cache = B.PlanCache()
    bt = B.AcquisitionBatch(B.batch_from_recordings(recs, cache))
    ref = bt.run([np.array(r["samples"]) for r in recs])
    pinned = [torch.from_numpy(np.ascontiguousarray(r["samples"])).pin_memory() for r in recs]
    for rep in range(2):
        got = bt.run([p.numpy() for p in pinned])
        for res, rr in zip(got, ref):
            for a, b in zip(res, rr):
                assert (a.peak_doppler_bin, a.peak_code_bin, a.noise_power) == (b.peak_doppler_bin, b.peak_code_bin,
                                                                               b.noise_power)
    bt.close()


def test_batch_detects_planted_satellites():
    recs = synth.ragged_batch(seed=5, n_recordings=6, max_nnc=4)
    cache = B.PlanCache()
    bt = B.AcquisitionBatch(B.batch_from_recordings(recs, cache))
    got = bt.run()
    hits = total = 0
    for r, res in zip(recs, got):
        strong = [s for s in r["sats"] if s.cn0 >= 42]
        by_prn = {x.prn: x for x in res}
        for s in strong:
            total += 1
            hits += A.is_detected(by_prn[s.prn])
    assert total == 0 or hits >= 0.8 * total


def test_batch_rejects_store_power_bins_and_bad_prn():
    recs = synth.ragged_batch(seed=2, n_recordings=1, max_nnc=1)
    cache = B.PlanCache()
    item = B.batch_from_recordings(recs, cache)[0]
    item.prns = [40]
    with pytest.raises(A.ArgumentError):
        B.AcquisitionBatch([item])
