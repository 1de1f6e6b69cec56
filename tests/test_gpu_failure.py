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
