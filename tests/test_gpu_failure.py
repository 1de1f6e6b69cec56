"""Failure detection without a GPU fault: a bounded device wait on an mbarrier that nothing
arrives on gives up, reports ACQ_ERR_TIMEOUT to the host, and the context stays usable."""
import ctypes as C

import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import _lib as L

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable():
    st = C.c_int32(-1)
    assert L.load().acq_selftest_bounded_wait(0, 1000, C.byref(st)) == 0, L.last_error()
    assert st.value == L.ACQ_ERR_TIMEOUT
    plan = A.plan_acquire(A.GPSL1CA(), 4e6, [1, 2])
    x = np.zeros(4000, np.complex64)
    res = A.acquire_b(plan, x, [1, 2])
    assert len(res) == 2


def test_column_stage_give_up_path_and_recovery():
    # The Doppler-group column stage of the simple path with a zero poll limit: every block gives
    # up at its first tile, takes one block-wide decision, waits with the full limit for the copies
    # it issued and leaves; acq_fetch_results reports ACQ_ERR_TIMEOUT. The same plan, with the
    # default limit back, then acquires exactly as before.
    from acqgb300 import synth
    a = A.GPSL1CA()
    kw = dict(min_doppler_coverage=5000, num_coherently_integrated_code_periods=10, num_noncoherent_accumulations=2)
    x = synth.to_ci16(synth.synth(a, 5e6, 2 * 10 * 5000, [synth.Satellite(3, 45.0, 1500.0, 200.0)], 3))
    plan = A.plan_acquire(a, 5e6, [3, 4], **kw)
    ref = A.acquire_b(plan, x, [3, 4], store_power_bins=True)
    ref_pb = [r.power_bins.copy() for r in ref]
    assert plan.get_option(L.ACQ_OPT_COLUMN_WAIT_POLLS) == 1 << 24
    assert plan.set_option(L.ACQ_OPT_COLUMN_WAIT_POLLS, 0) == 0
    with pytest.raises(A.AcquisitionError, match="status 5"):
        A.acquire_b(plan, x, [3, 4])
    assert "k_col_tma_k1<20>" in plan.last_kernels(), plan.last_kernels()
    assert plan.set_option(L.ACQ_OPT_COLUMN_WAIT_POLLS, 1 << 24) == 1 << 24
    for _ in range(2):   # the second identical request replays a captured graph
        again = A.acquire_b(plan, x, [3, 4], store_power_bins=True)
        for r0, p0, r1 in zip(ref, ref_pb, again):
            assert (r1.peak_doppler_bin, r1.peak_code_bin) == (r0.peak_doppler_bin, r0.peak_code_bin)
            assert A.is_detected(r1) == A.is_detected(r0)
            assert np.abs(r1.power_bins - p0).max() <= 1e-6 * p0.max()
    assert A.is_detected(again[0])
