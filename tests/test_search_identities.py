"""CPU checks of the identity the half-spectrum bit-edge search (k_col_sign_fold) rests on,
against the oracle's sign-search stage (src/noncoherent_integration.jl:60-115).

For two data bits, candidate (edge e, pattern p) of a column x is |DFT_ND(f)|^2 with
f[i] = s(p, 0) x[o + i] + s(p, 1) x[o + SUB + i] for i < SUB = ND / 2, zero beyond, o = e * edge_step.
From edge to edge f moves by a cyclic shift (s(p, 0) = s(p, 1)) or a negacyclic one
(s(p, 0) = -s(p, 1)), so the even bins (cyclic) or the odd bins (negacyclic) keep their power.
"""
import numpy as np
import pytest

from oracle import acq_oracle as O
from oracle import gnss_codes as G


def _half_spectrum(f, n1, n2, parity):
    """The kernel's four-step form: pass 1 over n1 < N1/2 (odd bins pre-twiddled by W_N1^n1),
    twiddle W_ND^(n2 k1), pass 2 over n2 for every k1 of the parity."""
    nd = n1 * n2
    out = np.zeros(nd, complex)
    p1 = np.zeros((n1, n2), complex)
    m = np.arange(n1 // 2)
    for b in range(n2):
        z = f[b + n2 * m]
        if parity:
            z = z * np.exp(-2j * np.pi * m / n1)
        zf = np.fft.fft(z)
        for j in range(n1 // 2):
            k1 = 2 * j + parity
            p1[k1, b] = zf[j] * np.exp(-2j * np.pi * b * k1 / nd)
    for j in range(n1 // 2):
        k1 = 2 * j + parity
        out[k1 + n1 * np.arange(n2)] = np.fft.fft(p1[k1])
    return out


@pytest.mark.parametrize("n1,n2,edge_step,n_be", [(32, 25, 100, 4), (20, 20, 50, 4), (40, 20, 200, 2)])
def test_half_spectra_reproduce_every_candidate(n1, n2, edge_step, n_be):
    rng = np.random.default_rng(n1 * n2 + edge_step)
    nd, sub = n1 * n2, n1 * n2 // 2
    x = rng.standard_normal(nd) + 1j * rng.standard_normal(nd)
    pats = [(1.0, 1.0), (1.0, -1.0)]
    for p, (s0, s1) in enumerate(pats):
        inv = 0 if s0 == s1 else 1   # the parity whose power is the same for every edge
        ref0 = None
        for e in range(n_be):
            o = e * edge_step
            b0 = np.zeros(nd, complex)
            b1 = np.zeros(nd, complex)
            b0[:sub] = x[(o + np.arange(sub)) % nd]
            b1[:sub] = x[(o + sub + np.arange(sub)) % nd]
            ref = np.abs(s0 * np.fft.fft(b0) + s1 * np.fft.fft(b1)) ** 2
            f = s0 * x[(o + np.arange(sub)) % nd] + s1 * x[(o + sub + np.arange(sub)) % nd]
            got = np.abs(_half_spectrum(f, n1, n2, 0) + _half_spectrum(f, n1, n2, 1)) ** 2
            assert np.max(np.abs(got - ref)) <= 1e-12 * ref.max()
            if ref0 is None:
                ref0 = ref
            else:
                assert np.max(np.abs(ref[inv::2] - ref0[inv::2])) <= 1e-12 * ref0.max()


def test_invariant_halves_on_the_oracle_stage():
    # the oracle's own stage (FP64) on a 40 ms, four-edge plan: the even bins of pattern 0 and the
    # odd bins of pattern 1 have the same power at every edge
    plan = O.plan_acquire(G.GPSL1CA, 5e6, [3], min_doppler_coverage=5000.0, num_coherently_integrated_code_periods=40,
                          bit_edge_search_steps=4, precision="f64")
    assert plan.num_doppler_bins == 800 and plan.num_data_bits == 2
    rng = np.random.default_rng(7)
    cim = rng.standard_normal((800, 16)) + 1j * rng.standard_normal((800, 16))
    rec = {}
    O.sign_search_stage(cim, plan, 3, np.arange(16), record=rec)
    n_pat = 2
    for p, parity in ((0, 0), (1, 1)):
        base = rec[0 * n_pat + p]
        for e in range(1, 4):
            other = rec[e * n_pat + p]
            assert np.max(np.abs(other[parity::2] - base[parity::2])) <= 1e-12 * base.max()
        # and the other parity does change with the edge
        assert np.max(np.abs(rec[1 * n_pat + p][1 - parity::2] - base[1 - parity::2])) > 1e-6 * base.max()
