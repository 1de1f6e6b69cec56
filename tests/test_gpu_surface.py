"""Chip-sorted power-surface export (src/plot.jl:35-57) on the GPU: the sorted surface equals
the FM-DBZP surface with its columns permuted by the oracle's restatement of
``_fmdbzp_sort_by_chip`` (an exact gather)."""
import ctypes as C

import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import _lib as L
from acqgb300 import synth
from oracle import acq_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sys_name,fs,n_coh,cov", [("GPSL1CA", 2.048e6, 1, 5000.0), ("GPSL1CA", 5e6, 10, 5000.0),
                                                   ("GPSL5I", 10.24e6, 10, 1000.0)])
def test_chip_sorted_surfaces(sys_name, fs, n_coh, cov):
    a_sys = {"GPSL1CA": A.GPSL1CA, "GPSL5I": A.GPSL5I}[sys_name]()
    plan = A.plan_acquire(a_sys, fs, [1, 2], min_doppler_coverage=cov, num_coherently_integrated_code_periods=n_coh)
    n = n_coh * plan.samples_per_code
    x = synth.synth(a_sys, fs, n, [synth.Satellite(1, 47.0, 600.0, 123.4)], 3).astype(np.complex64)
    raw = A.acquire_b(plan, x, [1, 2], store_power_bins=True)
    raw_bins = [r.power_bins.copy() for r in raw]   # power_bins alias the plan's buffers (test/plan.jl:350-355)
    srt = A.acquire_b(plan, x, [1, 2], store_power_bins=True, chip_sorted_power_bins=True)
    g = plan.geometry
    axis = A.plan_chip_axis(plan)
    for r, rb, s in zip(raw, raw_bins, srt):
        o_axis, o_sorted, _ = O.fmdbzp_sort_by_chip(rb, g.num_blocks, g.block_size,
                                                    a_sys.code_frequency, fs)
        assert np.array_equal(s.power_bins, o_sorted)
        assert np.array_equal(axis, o_axis)
        assert (r.peak_doppler_bin, r.peak_code_bin) == (s.peak_doppler_bin, s.peak_code_bin)


def test_device_sort_entry_point():
    plan = A.plan_acquire(A.GPSL1CA(), 4e6, [1])
    g = plan.geometry
    rng = np.random.default_rng(0)
    surf = rng.random((3, g.num_doppler_bins, g.samples_per_code_eff), dtype=np.float32)
    d_in = torch.as_tensor(surf, device="cuda")
    d_out = torch.empty_like(d_in)
    st = torch.cuda.current_stream().cuda_stream
    assert L.load().acq_sort_power_bins_by_chip(plan.handle, C.c_void_p(d_in.data_ptr()), 3,
                                                 C.c_void_p(d_out.data_ptr()), C.c_void_p(st)) == 0
    got = d_out.cpu().numpy()
    for k in range(3):
        assert np.array_equal(got[k], O.fmdbzp_sort_by_chip(surf[k], g.num_blocks, g.block_size, 1.023e6, 4e6)[1])
    assert L.load().acq_sort_power_bins_by_chip(plan.handle, C.c_void_p(d_in.data_ptr()), 3,
                                                 C.c_void_p(d_in.data_ptr()), C.c_void_p(st)) == L.ACQ_ERR_ARGUMENT
