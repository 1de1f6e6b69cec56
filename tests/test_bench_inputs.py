"""The CPU legs of bench.py synthesise their input with the oracle's restatement of the signal
model (no product library on that path); it must give the same bytes as the product's host
generator that feeds the GPU arm, for every benchmark workload, so both arms time one input."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


@pytest.mark.parametrize("config", ["cfg1", "cfg2", "cfg2b", "cfg4"])
def test_oracle_signal_model_matches_product_generator(config):
    bench.set_config(config)
    a, sats_a = bench.make_input()
    b, sats_b = bench.make_input(host_model=True)
    assert a.dtype == b.dtype and a.shape == b.shape
    assert np.array_equal(a, b)
    assert bench.input_digest(a) == bench.input_digest(b)
    assert [(s.prn, s.cn0, s.doppler, s.code_phase) for s in sats_a] == \
           [(s.prn, s.cn0, s.doppler, s.code_phase) for s in sats_b]
    bench.set_config("cfg2")
