"""Device-side code sampling (the plan precompute's codes) equals the host gen_code restatement
bit for bit, on the exact-integer and the FP64 phase paths, with BOC(1,1) and secondary codes."""
import ctypes as C

import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import _lib as L

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("system,fs,fc,start,n", [
    (A.GPSL1CA(), 4e6, 0.0, 0.0, 4000), (A.GPSL1CA(), 5e6, 1.023e6 + 0.81, 123.456, 50_000),
    (A.GPSL1CA(), 2.048e6, 0.0, 0.0, 2048), (A.GPSL5I(), 20e6, 0.0, 0.0, 200_000),
    (A.GPSL5I(), 12e6, 10.23e6 + 7.8, 5115.3, 120_000), (A.GalileoE1B(), 12e6, 0.0, 0.0, 48_000),
    (A.GalileoE1B(), 12e6, 1.023e6 + 1.1, 2000.25, 48_000), (A.GPSL1CA(), 16.368e6, 0.0, 0.0, 16_368)])
def test_device_codes_match_host(system, fs, fc, start, n):
    prns = [1, 7, 19, 32]
    out = torch.empty(len(prns) * n, dtype=torch.int8, device="cuda")
    pa = (C.c_int32 * len(prns))(*prns)
    st = torch.cuda.current_stream().cuda_stream
    assert L.load().acq_gen_code_device(system.sid, pa, len(prns), n, fs, fc, start, C.c_void_p(out.data_ptr()),
                                        C.c_void_p(st)) == 0, L.last_error()
    dev = out.cpu().numpy().reshape(len(prns), n)
    for i, p in enumerate(prns):
        assert np.array_equal(dev[i], system.gen_code(n, p, fs, fc or None, start)), (system.name, p)
