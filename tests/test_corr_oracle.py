"""CPU checks of the FP64 continuous-correlator oracle: closed-form derivatives against
forward-mode dual numbers and central finite differences, the sample adjoint against a
directional derivative, and Newton refinement against planted parameters."""
import numpy as np
import pytest

from oracle import corr_oracle as O
from oracle import gnss_codes as G

FS = 10e6
N = 200_000        # 20 ms at 10 MHz


@pytest.fixture(scope="module")
def sig():
    return O.synth_signal(G.GPSL1CA, 7, FS, N, 412.37, 1234.5, 48.0, seed=5)


@pytest.mark.parametrize("dtau,df", [(0.0, 0.0), (0.3, -12.0), (-0.55, 20.0), (0.12, 31.0)])
def test_closed_form_gradient_matches_dual_numbers_and_fd(sig, dtau, df):
    tau, f = 412.37 + dtau, 1234.5 + df
    P, g, h = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, tau, f))
    Pd, gd = O.power_gradient_dual(sig, G.GPSL1CA, 7, FS, tau, f)
    assert P == pytest.approx(Pd, rel=1e-12)
    scale = np.array([P, P * N / FS])          # natural gradient scales: per chip, per Hz
    assert np.all(np.abs(g - gd) <= 1e-9 * scale)
    ht, hf = 1e-3, 1e-2
    fd = np.array([(O.power(sig, G.GPSL1CA, 7, FS, tau + ht, f) - O.power(sig, G.GPSL1CA, 7, FS, tau - ht, f)) / (2 * ht),
                   (O.power(sig, G.GPSL1CA, 7, FS, tau, f + hf) - O.power(sig, G.GPSL1CA, 7, FS, tau, f - hf)) / (2 * hf)])
    assert np.all(np.abs(g - fd) <= 2e-4 * scale), (g, fd)


def test_closed_form_hessian_matches_fd_of_gradient(sig):
    tau, f = 412.37 + 0.08, 1234.5 - 7.0
    P, g, h = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, tau, f))
    ht, hf = 1e-3, 1e-2
    gp = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, tau + ht, f))[1]
    gm = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, tau - ht, f))[1]
    fp = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, tau, f + hf))[1]
    fm = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, tau, f - hf))[1]
    htt, hft = (gp - gm) / (2 * ht)
    htf, hff = (fp - fm) / (2 * hf)
    T = N / FS
    assert h[0] == pytest.approx(htt, rel=2e-2, abs=1e-3 * P)
    assert h[1] == pytest.approx(0.5 * (hft + htf), rel=2e-2, abs=1e-3 * P * T)
    assert h[2] == pytest.approx(hff, rel=2e-2, abs=1e-3 * P * T * T)


def test_hessian_negative_definite_at_planted_peak(sig):
    P, g, h = O.power_derivatives(O.correlate(sig, G.GPSL1CA, 7, FS, 412.37, 1234.5))
    assert h[0] < 0 and h[0] * h[2] - h[1] ** 2 > 0


def test_vjp_matches_directional_derivative():
    n = 40_000
    x = O.synth_signal(G.GPSL1CA, 3, FS, n, 100.2, -800.0, 52.0, seed=1)
    cells = [(3, 100.25, -790.0), (3, 99.9, -805.0), (5, 10.0, 0.0)]
    w = np.array([1.0, -0.5, 0.25])
    z = np.array([O.correlate(x, G.GPSL1CA, p, FS, t, f)["z"] for p, t, f in cells])
    xbar = O.vjp_samples(n, G.GPSL1CA, FS, cells, 2 * w * z)
    rng = np.random.default_rng(0)
    dx = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    L = lambda xx: sum(wi * O.power(xx, G.GPSL1CA, p, FS, t, f) for wi, (p, t, f) in zip(w, cells))
    eps = 1e-3
    fd = (L(x + eps * dx) - L(x - eps * dx)) / (2 * eps)
    lin = float(np.sum(xbar.real * dx.real + xbar.imag * dx.imag))
    assert lin == pytest.approx(fd, rel=1e-8)


@pytest.mark.parametrize("system,prn,fs,tau,f", [(G.GPSL1CA, 7, FS, 412.37, 1234.5),
                                                  (G.GalileoE1B, 11, 12e6, 2001.3, -2222.2)])
def test_newton_refine_reaches_planted_parameters(system, prn, fs, tau, f):
    n = int(round(fs * 0.02)) if system is G.GPSL1CA else int(round(fs * 0.008))
    x = O.synth_signal(system, prn, fs, n, tau, f, np.inf, seed=0)
    bin_hz = fs / n
    t1, f1, P, it, ok = O.newton_refine(x, system, prn, fs, tau + 0.07, f + 0.4 * bin_hz)
    assert ok and abs(t1 - tau) < 5e-3 and abs(f1 - f) < 0.02 * bin_hz, (t1 - tau, f1 - f, it)
