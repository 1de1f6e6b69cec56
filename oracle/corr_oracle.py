"""Oracle (test infrastructure only): FP64 CPU continuous correlator of the fine search.

Only ``tests/`` and ``bench.py``'s CPU legs may import this module, as the checker. The
product is the CUDA correlator of libacqgb300 (acq_corr_* in include/acqgb300.h).

The reference refines a detected peak by a parabola through neighbouring grid cells
(src/acquire.jl:9-13,713-740) over the correlation of the signal model of
src/generate_test_signal.jl:45-68. The continuous correlator evaluates that correlation at
any (code phase tau, Doppler f):

    phi_n   = tau + n (f_code + f f_code / f_carrier) / fs
    theta_n = 2 pi (IF + f) n / fs
    z       = sum_n x[n] c(phi_n) exp(-i theta_n),      P = |z|^2

with the code replica c(phi) = S(M phi), S the quadratic-B-spline smoothing of the chip table
(M = 2 half-chip entries per chip for BOC(1,1), else 1; secondary code folded in). There is no
reference implementation of this model: parity is pinned by agreement between three
independent FP64 evaluations here (closed-form derivatives, forward-mode dual numbers, central
finite differences) and against the signal model's planted parameters.
"""
from __future__ import annotations

import math

import numpy as np

from . import gnss_codes as G


def replica_table(system: G.System, prn: int):
    """(table of +-1 float64 entries, entries per chip M)."""
    full = system.full_chips(prn).astype(np.float64)
    if system.boc11:
        t = np.empty(2 * full.size)
        t[0::2] = full
        t[1::2] = -full
        return t, 2
    return full, 1


def spline(tab: np.ndarray, psi: np.ndarray):
    """S, S', S'' of the quadratic-B-spline replica at table coordinates psi."""
    Lt = tab.size
    jf = np.floor(psi)
    t = psi - jf - 0.5
    j = np.mod(jf.astype(np.int64), Lt)
    a, b, d = tab[(j - 1) % Lt], tab[j], tab[(j + 1) % Lt]
    alpha, beta, gamma = (a + 6 * b + d) / 8, (d - a) / 2, (a - 2 * b + d) / 2
    return alpha + t * (beta + gamma * t), beta + 2 * gamma * t, 2 * gamma


def _carrier(n, fs, interm_freq, f):
    cyc = np.mod((interm_freq + f) / fs * n, 1.0)
    return np.exp(-2j * np.pi * cyc)


def correlate(x, system: G.System, prn: int, fs: float, tau: float, f: float, interm_freq: float = 0.0):
    """FP64 z and its first and second derivatives: dict z, zt, zf, ztt, ztf, zff."""
    x = np.asarray(x, dtype=np.complex128)
    n = np.arange(x.size, dtype=np.float64)
    tab, M = replica_table(system, prn)
    fc, fcar = system.code_freq, system.center_freq
    rho = (fc + f * fc / fcar) / fs
    S, S1, S2 = spline(tab, M * (tau + n * rho))
    y = x * _carrier(n, fs, interm_freq, f)
    kap, bc = fc / (fcar * fs), 2 * np.pi / fs
    return dict(
        z=np.sum(y * S), zt=M * np.sum(y * S1), ztt=M * M * np.sum(y * S2),
        zf=np.sum(n * y * (M * kap * S1 - 1j * bc * S)),
        ztf=np.sum(n * y * (M * M * kap * S2 - 1j * bc * M * S1)),
        zff=np.sum(n * n * y * (M * M * kap * kap * S2 - 2j * bc * kap * M * S1 - bc * bc * S)))


def power_derivatives(d: dict):
    """P, gradient (dP/dtau, dP/df) and Hessian (tt, tf, ff) from ``correlate``'s output."""
    rc = lambda p, q: (np.conj(p) * q).real
    z, zt, zf = d["z"], d["zt"], d["zf"]
    P = abs(z) ** 2
    g = np.array([2 * rc(z, zt), 2 * rc(z, zf)])
    h = np.array([2 * (rc(zt, zt) + rc(z, d["ztt"])), 2 * (rc(zt, zf) + rc(z, d["ztf"])),
                  2 * (rc(zf, zf) + rc(z, d["zff"]))])
    return P, g, h


def power(x, system, prn, fs, tau, f, interm_freq=0.0) -> float:
    x = np.asarray(x, dtype=np.complex128)
    n = np.arange(x.size, dtype=np.float64)
    tab, M = replica_table(system, prn)
    rho = (system.code_freq + f * system.code_freq / system.center_freq) / fs
    S, _, _ = spline(tab, M * (tau + n * rho))
    return float(abs(np.sum(x * S * _carrier(n, fs, interm_freq, f))) ** 2)


class Dual:
    """Forward-mode dual number over (tau, f): value plus two partials (numpy broadcasting)."""

    __array_ufunc__ = None   # numpy arrays defer to the reflected operators below

    def __init__(self, v, dt=0.0, df=0.0):
        self.v, self.dt, self.df = v, dt, df

    def _w(self, o):
        return o if isinstance(o, Dual) else Dual(o)

    def __add__(self, o):
        o = self._w(o)
        return Dual(self.v + o.v, self.dt + o.dt, self.df + o.df)

    __radd__ = __add__

    def __sub__(self, o):
        o = self._w(o)
        return Dual(self.v - o.v, self.dt - o.dt, self.df - o.df)

    def __rsub__(self, o):
        return self._w(o) - self

    def __mul__(self, o):
        o = self._w(o)
        return Dual(self.v * o.v, self.dt * o.v + self.v * o.dt, self.df * o.v + self.v * o.df)

    __rmul__ = __mul__

    def sum(self):
        return Dual(np.sum(self.v), np.sum(self.dt), np.sum(self.df))


def power_gradient_dual(x, system, prn, fs, tau, f, interm_freq=0.0):
    """P and its gradient by forward-mode dual numbers through the same model (ForwardDiff's
    role: differentiate the evaluation itself, with floor() of the table index constant)."""
    x = np.asarray(x, dtype=np.complex128)
    n = np.arange(x.size, dtype=np.float64)
    tab, M = replica_table(system, prn)
    fc, fcar = system.code_freq, system.center_freq
    T, F = Dual(tau, 1.0, 0.0), Dual(f, 0.0, 1.0)
    psi = M * (T + n * ((fc + F * (fc / fcar)) * (1.0 / fs)))
    Lt = tab.size
    jf = np.floor(psi.v)
    t = psi - (jf + 0.5)
    j = np.mod(jf.astype(np.int64), Lt)
    a, b, d = tab[(j - 1) % Lt], tab[j], tab[(j + 1) % Lt]
    S = (a + 6 * b + d) / 8 + t * ((d - a) / 2 + ((a - 2 * b + d) / 2) * t)
    e = _carrier(n, fs, interm_freq, f)
    # d exp(-i theta) / df = -i 2 pi n / fs exp(-i theta)
    E = Dual(e, 0.0, -2j * np.pi * n / fs * e)
    z = (x * S * E).sum()
    P = abs(z.v) ** 2
    return P, np.array([2 * (np.conj(z.v) * z.dt).real, 2 * (np.conj(z.v) * z.df).real])


def synth_signal(system, prn, fs, n, tau, f, cn0_dbhz, seed, interm_freq=0.0, phase=0.3):
    """Data-free signal of src/generate_test_signal.jl:45-68's model (code at the Doppler-shifted
    rate, carrier exp(+i theta)) plus unit-power complex white noise (cn0 = inf: no noise)."""
    fc = system.code_freq + f * system.code_freq / system.center_freq
    code = G.gen_code(n, system, prn, fs, fc, tau).astype(np.float64)
    t = np.arange(n, dtype=np.float64)
    amp = 1.0 if not np.isfinite(cn0_dbhz) else math.sqrt(10 ** (cn0_dbhz / 10) / fs)
    x = amp * code * np.exp(1j * (2 * np.pi * np.mod((interm_freq + f) / fs * t, 1.0) + phase))
    if np.isfinite(cn0_dbhz):
        rng = np.random.default_rng(seed)
        x = x + (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
    return x


def vjp_samples(n_samples, system, fs, cells, zbar, interm_freq=0.0):
    """x_bar[n] = sum_c zbar_c S(psi_{c,n}) exp(+i theta_{c,n}) (complex128)."""
    n = np.arange(n_samples, dtype=np.float64)
    out = np.zeros(n_samples, dtype=np.complex128)
    fc, fcar = system.code_freq, system.center_freq
    for (prn, tau, f), zb in zip(cells, zbar):
        tab, M = replica_table(system, prn)
        S, _, _ = spline(tab, M * (tau + n * (fc + f * fc / fcar) / fs))
        out += zb * S * np.conj(_carrier(n, fs, interm_freq, f))
    return out


def newton_refine(x, system, prn, fs, tau, f, interm_freq=0.0, max_iter=20, tol=(1e-4, 1e-3), step=(0.25, None)):
    """FP64 restatement of the library's refinement rule (Newton inside a box trust region,
    scaled gradient ascent where the Hessian is not negative definite, step halving when the
    power drops). Returns (tau, f, P, iterations, converged)."""
    st_t = step[0]
    st_f = step[1] if step[1] is not None else 0.25 * fs / len(x)
    prev = None
    stp = (0.0, 0.0)
    it = 0
    while True:
        P, g, h = power_derivatives(correlate(x, system, prn, fs, tau, f, interm_freq))
        if prev is not None and P < prev[2]:
            stp = (0.5 * stp[0], 0.5 * stp[1])
            if abs(stp[0]) < tol[0] and abs(stp[1]) < tol[1]:
                return prev[0], prev[1], prev[2], it + 1, True
            tau, f = prev[0] + stp[0], prev[1] + stp[1]
        else:
            prev = (tau, f, P)
            det = h[0] * h[2] - h[1] ** 2
            if h[0] < 0 and det > 0:
                dt = -(h[2] * g[0] - h[1] * g[1]) / det
                df = -(-h[1] * g[0] + h[0] * g[1]) / det
            else:
                a, b = g[0] * st_t, g[1] * st_f
                nrm = math.hypot(a, b)
                dt, df = (st_t * a / nrm, st_f * b / nrm) if nrm > 0 else (0.0, 0.0)
            sc = 1.0
            if abs(dt) > st_t:
                sc = min(sc, st_t / abs(dt))
            if abs(df) > st_f:
                sc = min(sc, st_f / abs(df))
            dt, df = dt * sc, df * sc
            if abs(dt) < tol[0] and abs(df) < tol[1]:
                return tau, f, P, it + 1, True
            stp = (dt, df)
            tau, f = tau + dt, f + df
        it += 1
        if it >= max_iter:
            return prev[0], prev[1], prev[2], it, False
