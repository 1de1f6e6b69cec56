"""Tensor-core rotation combine (FP16 / BF16, single or split hi + lo operands) against the FP64
oracle and the FP32 path on secondary-code rotation searches.

Bars (power relative to the surface peak of the FP64 oracle):
* split hi + lo (FP16 or BF16): power within 1e-4, every decision equal to the FP32 path's;
* single FP16: power within 2e-3; single BF16: within 2e-2; detected set, peak cells and
  secondary-code phase equal on these strong-signal cases.
"""
import numpy as np
import pytest

import acqgb300 as A
from acqgb300 import synth
from oracle import acq_oracle as O
from oracle import gnss_codes as G

pytestmark = pytest.mark.gpu

BARS = {"fp16_split": 1e-4, "bf16_split": 1e-4, "fp16": 2e-3, "bf16": 2e-2}
CASES = {
    "l5i-10ms": dict(fs=10.24e6, prns=[2, 3, 7], n_coh=10, n_nc=1, cov=5000.0, quant="ci8",
                     sats=[synth.Satellite(2, 50.0, -1700.0, 333.3), synth.Satellite(7, 47.0, 2100.0, 7000.0)]),
    "l5i-20msx2": dict(fs=12e6, prns=[1, 4, 5], n_coh=20, n_nc=2, cov=5000.0, quant=None,
                       sats=[synth.Satellite(1, 46.0, 900.0, 1234.5), synth.Satellite(4, 44.0, -3100.0, 6000.0)]),
}


def _signal(c, seed=2):
    n = c["n_nc"] * c["n_coh"] * int(np.ceil(10230 / 10.23e6 * c["fs"]))
    x = synth.synth(A.GPSL5I(), c["fs"], n, c["sats"], seed)
    if c["quant"] == "ci8":
        q = synth.to_ci8_3bit(x)
        return q, (q[:, 0].astype(np.float32) + 1j * q[:, 1].astype(np.float32)).astype(np.complex64)
    return x.astype(np.complex64), x.astype(np.complex64)


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    c = CASES[request.param]
    sig, osig = _signal(c)
    op = O.plan_acquire(G.GPSL5I, c["fs"], c["prns"], min_doppler_coverage=c["cov"],
                        num_coherently_integrated_code_periods=c["n_coh"], num_noncoherent_accumulations=c["n_nc"],
                        precision="f64")
    ref = O.acquire_b(op, osig, c["prns"], return_surfaces=True)
    plan = A.plan_acquire(A.GPSL5I(), c["fs"], c["prns"], min_doppler_coverage=c["cov"],
                          num_coherently_integrated_code_periods=c["n_coh"], num_noncoherent_accumulations=c["n_nc"])
    base = A.acquire_b(plan, sig, c["prns"], store_power_bins=True)
    return request.param, c, sig, plan, ref, base


def _surf(ref, prn):
    out, surfs = ref
    for x, s in zip(out, surfs):
        if x.prn == prn:
            return np.asarray(s.power, dtype=np.float64)
    raise KeyError(prn)


@pytest.mark.parametrize("prec", sorted(BARS))
def test_tensor_core_combine(case, prec):
    name, c, sig, plan, ref, base = case
    assert plan.set_rotation_precision(prec) == prec
    try:
        res = A.acquire_b(plan, sig, c["prns"], store_power_bins=True)
    finally:
        plan.set_rotation_precision("fp32")
    for r, b in zip(res, base):
        p64 = _surf(ref, r.prn)
        err = np.max(np.abs(np.asarray(r.power_bins, dtype=np.float64) - p64)) / np.max(p64)
        print(f"{name} {prec} PRN {r.prn}: max power error / peak = {err:.2e}")
        assert err <= BARS[prec], (prec, r.prn, err)
        assert A.is_detected(r) == A.is_detected(b)
        if A.is_detected(b):
            assert (r.peak_doppler_bin, r.peak_code_bin, r.secondary_code_phase) == \
                   (b.peak_doppler_bin, b.peak_code_bin, b.secondary_code_phase)
        if prec.endswith("split"):
            assert (r.peak_doppler_bin, r.peak_code_bin, r.sign_pattern) == \
                   (b.peak_doppler_bin, b.peak_code_bin, b.sign_pattern)


def test_precision_option_falls_back_where_not_instantiated():
    plan = A.plan_acquire(A.GPSL1CA(), 4e6, [1])
    assert plan.set_rotation_precision("fp16_split") == "fp32"


# ---- simple path: the Doppler DFT as a dense DFT-matrix GEMM on the tensor cores
SIMPLE = {
    "l1-5MHz-10msx2-ci16": dict(sys="GPSL1CA", fs=5e6, prns=[3, 9, 17], n_coh=10, n_nc=2, cov=5000.0, quant="ci16",
                                sats=[synth.Satellite(3, 44.0, 4950.0, 100.5), synth.Satellite(9, 42.0, -1200.0, 700.25)]),
    "l1-4MHz-1ms": dict(sys="GPSL1CA", fs=4e6, prns=[1, 2], n_coh=1, n_nc=1, cov=7000.0, quant=None,
                        sats=[synth.Satellite(1, 48.0, 1234.0, 300.5)]),
    "e1b-12MHz": dict(sys="GalileoE1B", fs=12e6, prns=[11, 12], n_coh=1, n_nc=1, cov=8000.0, quant=None,
                      sats=[synth.Satellite(11, 50.0, 2500.0, 2000.25, data_bits=False)]),
}
SYS = {"GPSL1CA": (A.GPSL1CA, G.GPSL1CA), "GalileoE1B": (A.GalileoE1B, G.GalileoE1B)}


@pytest.fixture(scope="module", params=sorted(SIMPLE))
def simple_case(request):
    c = SIMPLE[request.param]
    a_sys, o_sys = SYS[c["sys"]]
    a_sys = a_sys()
    plan = A.plan_acquire(a_sys, c["fs"], c["prns"], min_doppler_coverage=c["cov"],
                          num_coherently_integrated_code_periods=c["n_coh"], num_noncoherent_accumulations=c["n_nc"])
    n = c["n_nc"] * c["n_coh"] * plan.samples_per_code
    x = synth.synth(a_sys, c["fs"], n, c["sats"], 6)
    if c["quant"] == "ci16":
        sig = synth.to_ci16(x)
        osig = (sig[:, 0].astype(np.float32) + 1j * sig[:, 1].astype(np.float32)).astype(np.complex64)
    else:
        sig = osig = x.astype(np.complex64)
    op = O.plan_acquire(o_sys, c["fs"], c["prns"], min_doppler_coverage=c["cov"],
                        num_coherently_integrated_code_periods=c["n_coh"], num_noncoherent_accumulations=c["n_nc"],
                        precision="f64")
    ref = O.acquire_b(op, osig, c["prns"], return_surfaces=True)
    base = A.acquire_b(plan, sig, c["prns"], store_power_bins=True)
    base = [(b, b.power_bins.copy()) for b in base]
    return request.param, c, sig, plan, ref, base


@pytest.mark.parametrize("prec", sorted(BARS))
def test_tensor_core_doppler_dft(simple_case, prec):
    name, c, sig, plan, ref, base = simple_case
    assert plan.set_doppler_precision(prec) == prec
    try:
        res = A.acquire_b(plan, sig, c["prns"], store_power_bins=True)
    finally:
        plan.set_doppler_precision("fp32")
    for r, (b, bpb) in zip(res, base):
        p64 = _surf(ref, r.prn)
        err = np.max(np.abs(np.asarray(r.power_bins, dtype=np.float64) - p64)) / np.max(p64)
        print(f"{name} {prec} PRN {r.prn}: max power error / peak = {err:.2e}")
        assert err <= BARS[prec], (prec, r.prn, err)
        assert A.is_detected(r) == A.is_detected(b)
        if A.is_detected(b):
            assert (r.peak_doppler_bin, r.peak_code_bin) == (b.peak_doppler_bin, b.peak_code_bin)
