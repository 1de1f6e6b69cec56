"""Continuous correlator on the GPU (acq_corr_*) against the FP64 CPU oracle.

Tolerances are relative to the natural scale of each quantity at the planted peak: P_s (power),
P_s per chip and P_s T per Hz (gradient), P_s, P_s T, P_s T^2 (Hessian), T = coherent time.
FP32 sums over 200 000 samples are required to agree within 1e-4 of those scales (power,
gradient, sample adjoint) and 1e-3 for the Hessian: its second derivative of the replica is
piecewise constant, so a sample that lies within rounding distance of a spline knot takes
either side in the device's fixed-point position and the oracle's FP64 one. Finite
differences of the GPU power (h = 1e-3 chip, 1e-2 Hz) agree within 1e-2.
"""
import numpy as np
import pytest

import acqgb300 as A
from oracle import corr_oracle as O
from oracle import gnss_codes as G

torch = pytest.importorskip("torch")
from acqgb300 import corr as CR  # noqa: E402

pytestmark = pytest.mark.gpu

FS = 10e6
N = 200_000
T = N / FS
TAU, FD = 412.37, 1234.5
RTOL = 1e-4
HESS_RTOL = 1e-3
FD_RTOL = 1e-2


@pytest.fixture(scope="module")
def case():
    sig = O.synth_signal(G.GPSL1CA, 7, FS, N, TAU, FD, 45.0, seed=5).astype(np.complex64)
    corr = CR.Correlator(A.GPSL1CA(), FS, [7, 9, 21])
    x = torch.as_tensor(sig, device="cuda")
    Ps = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, TAU, FD))[0]
    return sig, corr, x, Ps


def _cells():
    rng = np.random.default_rng(3)
    prns = np.array([7] * 12 + [9, 21])
    taus = np.concatenate([[TAU, TAU + 0.02, TAU - 0.3, TAU + 0.6], TAU + rng.uniform(-1, 1, 8), [55.5, 900.25]])
    fds = np.concatenate([[FD, FD - 3.0, FD + 11.0, FD - 24.0], FD + rng.uniform(-50, 50, 8), [0.0, -3000.0]])
    return prns, taus, fds


def test_eval_power_gradient_hessian_match_fp64(case):
    sig, corr, x, Ps = case
    prns, taus, fds = _cells()
    e = corr.eval(x, prns, taus, fds, hessian=True)
    assert np.all(e.status == 0)
    gs = np.array([Ps, Ps * T])
    hs = np.array([Ps, Ps * T, Ps * T * T])
    worst = np.zeros(3)
    for i, (p, t, f) in enumerate(zip(prns, taus, fds)):
        d = O.correlate(sig, G.GPSL1CA, int(p), FS, t, f)
        P, g, h = O.power_derivatives(d)
        worst = np.maximum(worst, [abs(e.power[i] - P) / Ps, np.max(np.abs(e.grad[i] - g) / gs),
                                   np.max(np.abs(e.hess[i] - h) / hs)])
        assert abs(e.z[i] - d["z"]) <= RTOL * np.sqrt(Ps)
    assert np.all(worst[:2] <= RTOL) and worst[2] <= HESS_RTOL, worst


def test_eval_without_hessian_gives_same_power_and_gradient(case):
    sig, corr, x, Ps = case
    prns, taus, fds = _cells()
    a = corr.eval(x, prns, taus, fds, hessian=True)
    b = corr.eval(x, prns, taus, fds, hessian=False)
    assert np.array_equal(a.power, b.power) and np.array_equal(a.grad, b.grad)
    assert np.all(b.hess == 0)


def test_gradient_matches_central_finite_differences_of_gpu_power(case):
    sig, corr, x, Ps = case
    ht, hf = 1e-3, 1e-2
    taus = np.array([TAU + 0.05, TAU - 0.4, TAU + 0.21, TAU])
    fds = np.array([FD + 5.0, FD - 14.0, FD + 30.0, FD + 8.0])
    prns = np.full(4, 7)
    g = corr.eval(x, prns, taus, fds).grad
    P = lambda t, f: corr.eval(x, prns, t, f).power
    fdt = (P(taus + ht, fds) - P(taus - ht, fds)) / (2 * ht)
    fdf = (P(taus, fds + hf) - P(taus, fds - hf)) / (2 * hf)
    assert np.all(np.abs(g[:, 0] - fdt) <= FD_RTOL * Ps), (g[:, 0], fdt)
    assert np.all(np.abs(g[:, 1] - fdf) <= FD_RTOL * Ps * T), (g[:, 1], fdf)


def test_vjp_samples_matches_fp64(case):
    sig, corr, x, Ps = case
    cells = [(7, TAU + 0.01, FD - 2.0), (7, TAU - 0.7, FD + 20.0), (9, 300.0, 500.0)]
    prns, taus, fds = (np.array(c) for c in zip(*cells))
    z = corr.eval(x, prns, taus, fds).z
    w = np.array([1.0, -0.5, 2.0])
    zbar = 2 * w * z
    xb = corr.vjp_samples(N, prns, taus, fds, zbar).cpu().numpy()
    ref = O.vjp_samples(N, G.GPSL1CA, FS, cells, zbar)
    assert np.max(np.abs(xb - ref)) <= RTOL * np.max(np.abs(ref))


def test_autograd_function_backward(case):
    sig, corr, x, Ps = case
    taus = torch.tensor([TAU + 0.03, TAU - 0.2], dtype=torch.float64, device="cuda", requires_grad=True)
    fds = torch.tensor([FD + 4.0, FD - 9.0], dtype=torch.float64, device="cuda", requires_grad=True)
    xs = x.clone().requires_grad_(True)
    w = torch.tensor([1.0, 0.5], dtype=torch.float64, device="cuda")
    P = CR.correlator_power(corr, xs, [7, 7], taus, fds)
    (w * P).sum().backward()
    cells = [(7, float(t), float(f)) for t, f in zip(taus.detach().cpu(), fds.detach().cpu())]
    zs, gs = [], []
    for p, t, f in cells:
        d = O.correlate(sig, G.GPSL1CA, p, FS, t, f)
        zs.append(d["z"])
        gs.append(O.power_derivatives(d)[1])
    gs = np.array(gs)
    wn = w.cpu().numpy()
    assert np.allclose(taus.grad.cpu().numpy(), wn * gs[:, 0], rtol=0, atol=RTOL * Ps)
    assert np.allclose(fds.grad.cpu().numpy(), wn * gs[:, 1], rtol=0, atol=RTOL * Ps * T)
    ref = O.vjp_samples(N, G.GPSL1CA, FS, cells, 2 * wn * np.array(zs))
    got = xs.grad.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= RTOL * np.max(np.abs(ref))


@pytest.mark.parametrize("system,a_sys,prn,fs,n,tau,f", [
    (G.GPSL1CA, A.GPSL1CA(), 7, FS, N, TAU, FD),
    (G.GalileoE1B, A.GalileoE1B(), 11, 12e6, 96_000, 2001.3, -2222.2),
    (G.GPSL5I, A.GPSL5I(), 4, 20e6, 200_000, 4321.75, 3100.0)])
def test_newton_refine_reaches_planted_parameters(system, a_sys, prn, fs, n, tau, f):
    sig = O.synth_signal(system, prn, fs, n, tau, f, np.inf, seed=0).astype(np.complex64)
    corr = CR.Correlator(a_sys, fs, [prn])
    x = torch.as_tensor(sig, device="cuda")
    rng = np.random.default_rng(1)
    m = 64
    chip_bin = system.code_freq / fs          # one code-phase bin (a sample) in chips
    dop_bin = fs / n
    t0 = tau + rng.uniform(-0.5, 0.5, m) * chip_bin
    f0 = f + rng.uniform(-0.5, 0.5, m) * dop_bin
    r = corr.refine(x, np.full(m, prn), t0, f0, max_iterations=30)
    assert np.all(r.status == 0), r.status
    assert np.all(np.abs(r.code_phase - tau) < 2e-3), np.max(np.abs(r.code_phase - tau))
    assert np.all(np.abs(r.doppler - f) < 0.01 * dop_bin), np.max(np.abs(r.doppler - f))
    P0 = corr.eval(x, np.full(m, prn), t0, f0).power
    assert np.all(r.power >= P0)


def test_newton_refine_matches_fp64_rule_with_noise(case):
    sig, corr, x, Ps = case
    starts = [(TAU + 0.04, FD + 10.0), (TAU - 0.045, FD - 20.0)]
    r = corr.refine(x, [7, 7], [s[0] for s in starts], [s[1] for s in starts], max_iterations=30)
    for i, (t0, f0) in enumerate(starts):
        t1, f1, P, it, ok = O.newton_refine(sig.astype(np.complex128), G.GPSL1CA, 7, FS, t0, f0, max_iter=30)
        assert ok and r.status[i] == 0
        assert abs(r.code_phase[i] - t1) < 1e-3 and abs(r.doppler[i] - f1) < 0.05


def test_int16_samples_and_bad_prn(case):
    sig, corr, x, Ps = case
    q = np.stack([np.rint(sig.real * 1024), np.rint(sig.imag * 1024)], axis=-1).astype(np.int16)
    xq = torch.as_tensor(q, device="cuda")
    a = corr.eval(xq, [7, 30], [TAU, TAU], [FD, FD])
    xf = torch.as_tensor((q[:, 0] + 1j * q[:, 1]).astype(np.complex64), device="cuda")
    b = corr.eval(xf, [7], [TAU], [FD])
    assert a.power[0] == b.power[0]
    assert a.status[1] == 3 and a.power[1] == 0.0


def test_argument_errors(case):
    sig, corr, x, Ps = case
    with pytest.raises(A.ArgumentError):
        CR.Correlator(A.GPSL1CA(), FS, [0])
    with pytest.raises(A.ArgumentError):
        corr.refine(x, [7], [TAU], [FD], max_iterations=0)
