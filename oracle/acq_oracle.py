"""Oracle (test infrastructure only): CPU restatement of Acquisition.jl's FM-DBZP path.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import this module, and only as the
checker or the timed CPU baseline, never as the product. The product path is the
CUDA library under ``acquisition.jl_gb300/`` and it never routes through here.

Every function cites the reference file:line it restates (paths inside
JuliaGNSS/Acquisition.jl v2.6.4). The reference cannot run in this environment
(no Julia, FFTW or GNSSSignals), so the restatement is pinned by the reference's
own known-answer tests and its single numeric golden vector
(``tests/test_oracle_golden.py``).

Two precisions:

* ``precision="f32"`` keeps the reference's ComplexF32/Float32 data path and its
  FP32 op order where it changes results (IF phase, 1/fft_size scaling, parabolic
  interpolation in Float32). FFTs are pocketfft single precision (the reference uses
  FFTW single precision; both differ from exact by FP32 rounding only).
* ``precision="f64"`` runs the same algorithm in float64/complex128 and is the
  error reference for every FP32 result. It keeps the reference's FP32 *phase
  argument* of the IF wipe-off (a defined input quantisation of the algorithm) but
  evaluates everything after it in FP64.

Additions over the reference (it discards them): the sign pattern and bit edge
that win the max at every cell (strict ``>``, the earlier candidate keeps ties,
``src/noncoherent_integration.jl:99-112,278-293``) are tracked and reported at the
peak cell.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft
from scipy.special import gammainccinv

from . import gnss_codes
from .gnss_codes import System, gen_code

BATCH_FFT_THRESHOLD = 320   # src/plan.jl:7 (only selects FFTW plan shape there)


class ArgumentError(ValueError):
    """Mirror of Julia's ArgumentError."""


# --------------------------------------------------------------------------------------
# small numeric helpers
# --------------------------------------------------------------------------------------
def nextprod_2357(n: int) -> int:
    """Smallest 7-smooth integer >= n (Julia ``nextprod((2,3,5,7), n)``)."""
    m = max(int(n), 1)
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def fmdbzp_column_to_tau(col0: int, num_blocks: int, block_size: int) -> int:
    """src/plot.jl:16-20."""
    block_row = col0 // block_size
    within = col0 % block_size
    return ((num_blocks - block_row) % num_blocks) * block_size + within


def cfar_threshold(pfa: float, num_cells: int, num_noncoherent_integrations: int = 1) -> float:
    """src/cfar.jl:64-85 (gamma_inc_inv -> scipy gammainccinv on the upper tail)."""
    if not (0 < pfa < 1):
        raise ArgumentError(f"pfa must be in (0, 1), got {pfa}")
    if not num_cells > 0:
        raise ArgumentError(f"num_cells must be positive, got {num_cells}")
    if not num_noncoherent_integrations > 0:
        raise ArgumentError("num_noncoherent_integrations must be positive")
    pfa_per_cell = 1 - (1 - pfa) ** (1 / num_cells)
    a = float(num_noncoherent_integrations)
    x = gammainccinv(a, pfa_per_cell)
    return float(x / a)


def parabolic_interp(left, peak, right):
    """src/acquire.jl:9-13 in Float32 (returns python 0.0 when the denominator is 0)."""
    left, peak, right = np.float32(left), np.float32(peak), np.float32(right)
    denom = np.float32(2) * (np.float32(2) * peak - left - right)
    if denom == 0:
        return 0.0
    return np.float32((right - left) / denom)


# --------------------------------------------------------------------------------------
# sign patterns, src/sign_patterns.jl
# --------------------------------------------------------------------------------------
def sign_patterns(system: System | None, prn: int, num_data_bits: int, num_secondary_rotations: int,
                  num_coh_periods: int, use_secondary_code: bool) -> np.ndarray:
    """src/sign_patterns.jl:23-47 -> (num_coh_periods, num_patterns) float32."""
    num_data_combos = 1 << (num_data_bits - 1)
    sec_active = use_secondary_code and num_secondary_rotations > 1
    num_sec = num_secondary_rotations if sec_active else 1
    coh_per_bit = num_coh_periods // num_data_bits
    L = num_secondary_rotations if sec_active else 1
    pat = np.empty((num_coh_periods, num_data_combos * num_sec), dtype=np.float32)
    col = 0
    for r in range(num_sec):
        for d in range(num_data_combos):
            for k in range(num_coh_periods):
                bit_idx = k // coh_per_bit
                data_sign = 1.0 if bit_idx == 0 else (1.0 if ((d >> (bit_idx - 1)) & 1) == 0 else -1.0)
                sec_sign = float(system.secondary_value(prn, (k + r) % L)) if sec_active else 1.0
                pat[k, col] = data_sign * sec_sign
            col += 1
    return pat


def combined_phase_patterns(patterns: np.ndarray, num_coh_periods: int, dtype=np.complex64) -> np.ndarray:
    """src/sign_patterns.jl:80-93 -> out[p, q, s] = patterns[p, q] * exp(-2 pi i p s / N)."""
    if patterns.shape[0] != num_coh_periods:
        raise ArgumentError("patterns rows must equal num_coh_periods")
    p = np.arange(num_coh_periods)[:, None, None]
    s = np.arange(num_coh_periods)[None, None, :]
    phase = np.exp(-2j * np.pi * (p * s) / num_coh_periods)
    return (patterns[:, :, None].astype(np.float64) * phase).astype(dtype)


def tile_phase_patterns(combined: np.ndarray, num_doppler_bins: int) -> np.ndarray:
    """src/sign_patterns.jl:114-129 -> tiled[w, p, q] = combined[p, q, w mod N]."""
    n = combined.shape[0]
    if num_doppler_bins % n != 0:
        raise ArgumentError("num_doppler_bins must be a multiple of num_coh_periods")
    s = np.arange(num_doppler_bins) % n
    return np.transpose(combined[:, :, s], (2, 0, 1)).copy()


# --------------------------------------------------------------------------------------
# plan, src/plan.jl:312-697
# --------------------------------------------------------------------------------------
@dataclass
class Plan:
    system: System
    sampling_freq: float
    samples_per_code: int
    samples_per_code_eff: int
    num_blocks: int
    block_size: int
    fft_size: int
    num_coherently_integrated_code_periods: int
    num_data_bits: int
    bit_edge_search_steps: int
    num_noncoherent_accumulations: int
    num_doppler_bins: int
    doppler_freqs: np.ndarray
    doppler_step: float
    avail_prns: list
    noise_estimator: str
    use_secondary_code: bool
    max_secondary_code_rotations: int
    num_secondary_rotations: int
    precision: str
    codes: dict = field(default_factory=dict)
    prn_conj_ffts: dict = field(default_factory=dict)
    sign_patterns_by_prn: dict = field(default_factory=dict)
    tiled_by_prn: dict = field(default_factory=dict)

    @property
    def rotation_active(self) -> bool:
        return self.num_secondary_rotations > 1 and self.num_coherently_integrated_code_periods > 1

    @property
    def simple_path(self) -> bool:
        return self.num_data_bits == 1 and self.bit_edge_search_steps == 1 and not self.rotation_active

    @property
    def cdt(self):
        return np.complex64 if self.precision == "f32" else np.complex128

    @property
    def rdt(self):
        return np.float32 if self.precision == "f32" else np.float64


def plan_geometry(system: System, fs: float, min_doppler_coverage: float = 7000.0,
                  n_coh: int = 1, n_be: int = 1, n_nc: int = 1, use_secondary_code: bool = True,
                  max_secondary_code_rotations: int = 32) -> dict:
    """Validation + geometry, src/plan.jl:325-465 and :493-525."""
    if n_nc < 1:
        raise ArgumentError(f"num_noncoherent_accumulations must be >= 1, got {n_nc}")
    if n_coh < 1:
        raise ArgumentError("num_coherently_integrated_code_periods must be >= 1")
    if n_be < 1:
        raise ArgumentError(f"bit_edge_search_steps must be >= 1, got {n_be}")
    if n_coh == 1 and n_be > 1:
        raise ArgumentError("bit_edge_search_steps must be 1 when num_coherently_integrated_code_periods == 1 "
                            f"(sub-bit mode; no bit boundary search applies), got {n_be}")
    L = system.secondary_code_length
    if use_secondary_code and L > 1 and n_coh > 1 and L > max_secondary_code_rotations:
        raise ArgumentError(
            f"Secondary-code rotation search size exceeds the per-plan cap for {system.name}: "
            f"get_secondary_code_length(system)={L} > max_secondary_code_rotations={max_secondary_code_rotations} "
            f"at num_coherently_integrated_code_periods={n_coh}. Remedies (in order): "
            "(1) reduce num_coherently_integrated_code_periods; "
            f"(2) raise max_secondary_code_rotations to at least {L}; or "
            "(3) set use_secondary_code = false to opt out of the rotation search.")
    if use_secondary_code and L > 1 and n_coh > 1 and n_coh % L != 0:
        raise ArgumentError(
            "Secondary-code rotation search requires num_coherently_integrated_code_periods to be a whole "
            f"multiple of the secondary-code length L={L}, got num_coherently_integrated_code_periods={n_coh}. "
            "A partial secondary-code period makes the rotation search produce a +-Doppler sign ambiguity "
            "(issue #68). Remedies (in order): (1) set num_coherently_integrated_code_periods to a multiple "
            f"of {L}; (2) set num_coherently_integrated_code_periods = 1 and raise "
            "num_noncoherent_accumulations; or (3) set use_secondary_code = false.")
    spc = math.ceil(system.code_length / system.code_freq * fs)
    has_data = math.isfinite(system.data_freq) and system.data_freq > 0
    if has_data:
        bit_samples = math.ceil(fs / system.data_freq)
        bit_period_codes = bit_samples // spc
    else:
        bit_period_codes = n_coh
    bin_width = fs / spc
    min_num_blocks = math.ceil(2 * min_doppler_coverage / bin_width + 2 / n_coh)
    nb = None
    for cand in range(max(min_num_blocks, 1), spc + 1):
        if spc % cand == 0:
            nb = cand
            break
    if nb is None or min_num_blocks > spc:
        raise ArgumentError(f"No valid num_blocks found: samples_per_code={spc} has no divisor "
                            f">= min_num_blocks={min_num_blocks}.")
    if has_data and n_coh >= bit_period_codes:
        if n_coh % bit_period_codes != 0:
            raise ArgumentError(f"num_coherently_integrated_code_periods={n_coh} must be divisible by "
                                f"bit_period_codes={bit_period_codes} (code periods per data bit).")
        if bit_period_codes % n_be != 0:
            raise ArgumentError(f"bit_edge_search_steps={n_be} must divide bit_period_codes={bit_period_codes}.")
    bs = spc // nb
    F = nextprod_2357(2 * bs)
    ndb = n_coh // bit_period_codes if (has_data and n_coh >= bit_period_codes) else 1
    ndop = n_coh * nb
    cov = nb * fs / spc
    step = cov / ndop
    freqs = -cov / 2 + np.arange(ndop) * step
    rot = use_secondary_code and L > 1 and n_coh > 1
    R = L if rot else 1
    return dict(spc=spc, spc_eff=spc * R, nb=nb, bs=bs, F=F, ndb=ndb, ndop=ndop, freqs=freqs,
                step=step, R=R, bit_period_codes=bit_period_codes)


# threads per FFT call (-1: all cores); a process pool that spreads PRNs over cores sets 1
FFT_WORKERS = -1


def _fft(x, axis, prec):
    return sfft.fft(x, axis=axis, workers=FFT_WORKERS)


def _bfft(x, axis, prec):
    return sfft.ifft(x, axis=axis, norm="forward", workers=FFT_WORKERS)


def plan_acquire(system: System, sampling_freq: float, prns, *, min_doppler_coverage: float = 7000.0,
                 num_coherently_integrated_code_periods: int = 1, bit_edge_search_steps: int = 1,
                 num_noncoherent_accumulations: int = 1, noise_estimator: str = "opposite_row",
                 use_secondary_code: bool = True, max_secondary_code_rotations: int = 32,
                 precision: str = "f32", codes: dict | None = None) -> Plan:
    """src/plan.jl:312-697 (geometry, conj code-block spectra, patterns)."""
    g = plan_geometry(system, sampling_freq, min_doppler_coverage, num_coherently_integrated_code_periods,
                      bit_edge_search_steps, num_noncoherent_accumulations, use_secondary_code,
                      max_secondary_code_rotations)
    plan = Plan(system, float(sampling_freq), g["spc"], g["spc_eff"], g["nb"], g["bs"], g["F"],
                num_coherently_integrated_code_periods, g["ndb"], bit_edge_search_steps,
                num_noncoherent_accumulations, g["ndop"], g["freqs"], g["step"], [int(p) for p in prns],
                noise_estimator, use_secondary_code, max_secondary_code_rotations, g["R"], precision)
    cdt = plan.cdt
    for prn in plan.avail_prns:
        # src/plan.jl:230-251
        code = gen_code(plan.samples_per_code, system, prn, sampling_freq) if codes is None else codes[prn]
        plan.codes[prn] = np.asarray(code, dtype=np.int8)
        blocks = np.zeros((plan.num_blocks, plan.fft_size), dtype=cdt)
        blocks[:, :plan.block_size] = plan.codes[prn].reshape(plan.num_blocks, plan.block_size)
        plan.prn_conj_ffts[prn] = np.conj(_fft(blocks, 1, precision)).astype(cdt)
    sign_active = plan.num_data_bits > 1 or bit_edge_search_steps > 1 or plan.rotation_active
    if sign_active:
        for prn in plan.avail_prns:
            p = sign_patterns(system, prn, plan.num_data_bits, plan.num_secondary_rotations,
                              num_coherently_integrated_code_periods, use_secondary_code)
            plan.sign_patterns_by_prn[prn] = p
            if plan.rotation_active:
                comb = combined_phase_patterns(p, num_coherently_integrated_code_periods, cdt)
                plan.tiled_by_prn[prn] = tile_phase_patterns(comb, plan.num_doppler_bins)
    return plan


# --------------------------------------------------------------------------------------
# front end, src/acquire.jl:92-104 and src/coherent_integration.jl:12-56
# --------------------------------------------------------------------------------------
def if_phase_f32(seg_start0: int, n: int, interm_freq_hz: float, fs: float) -> np.ndarray:
    """FP32 phase argument of src/acquire.jl:96-99."""
    step = np.float32(-2 * math.pi * interm_freq_hz / fs)
    offset = np.float32(np.float32(seg_start0) * step)
    i = np.arange(n).astype(np.float32)
    return (offset + (i * step).astype(np.float32)).astype(np.float32)


def downconvert(signal, seg_start0: int, seg_len: int, interm_freq_hz: float, fs: float, prec: str):
    """src/acquire.jl:92-104: ComplexF32(x) (no scaling), then IF wipe-off."""
    x = np.asarray(signal[seg_start0:seg_start0 + seg_len]).astype(np.complex64)
    if prec == "f64":
        x = x.astype(np.complex128)
    if interm_freq_hz == 0:
        return x
    ph = if_phase_f32(seg_start0, seg_len, interm_freq_hz, fs)
    if prec == "f32":
        rot = (np.cos(ph) + 1j * np.sin(ph)).astype(np.complex64)
        return (x * rot).astype(np.complex64)
    ph = ph.astype(np.float64)
    return x * (np.cos(ph) + 1j * np.sin(ph))


def signal_block_ffts(seg, plan: Plan) -> np.ndarray:
    """src/coherent_integration.jl:12-56: FFT of each wrapped double block -> (G, F)."""
    G = plan.num_coherently_integrated_code_periods * plan.num_blocks
    seg_len = len(seg)
    bs = plan.block_size
    idx = (np.arange(G)[:, None] * bs + np.arange(2 * bs)[None, :]) % seg_len
    blocks = np.zeros((G, plan.fft_size), dtype=plan.cdt)
    blocks[:, :2 * bs] = seg[idx]
    return _fft(blocks, 1, plan.precision).astype(plan.cdt)


def coherent_matrix(S: np.ndarray, conj_fft: np.ndarray, plan: Plan) -> np.ndarray:
    """src/coherent_integration.jl:90-171: the (G, spc) coherent integration matrix.

    Row g = p*nb + k of column block r is (1/F) * IFFT(S_g * C*_{(k+r) mod nb})[0:bs).
    """
    G = S.shape[0]
    nb, bs, F = plan.num_blocks, plan.block_size, plan.fft_size
    cim = np.empty((G, nb * bs), dtype=plan.cdt)
    if plan.precision == "f32":
        inv = np.float32(1) / np.float32(F)
    else:
        inv = 1.0 / F
    k = np.arange(G) % nb
    for r in range(nb):
        prod = (S * conj_fft[(k + r) % nb]).astype(plan.cdt)
        corr = _bfft(prod, 1, plan.precision)[:, :bs]
        cim[:, r * bs:(r + 1) * bs] = (corr * inv).astype(plan.cdt)
    return cim


# --------------------------------------------------------------------------------------
# column stages
# --------------------------------------------------------------------------------------
def abs2(z):
    return (z.real * z.real + z.imag * z.imag)


def simple_column_power(cim: np.ndarray, plan: Plan) -> np.ndarray:
    """src/acquire.jl:265-292 + :335-385: FFT_ndop per column, |X|^2, fftshift -> sorted rows."""
    X = _fft(cim, 0, plan.precision).astype(plan.cdt)
    P = abs2(X).astype(plan.rdt)
    return np.fft.fftshift(P, axes=0)


def _half_swap_rows(ndop: int) -> np.ndarray:
    """Destination row for each raw bin in the sign/rotation kernels (top/bottom swap, quirk
    for odd ndop kept), src/noncoherent_integration.jl:92-113 and :267-293."""
    half = ndop // 2
    w = np.arange(ndop)
    return np.where(w < half, w + half, w - half)


def sign_search_stage(cim: np.ndarray, plan: Plan, prn: int, cp_cols: np.ndarray, record: dict | None = None):
    """Data-bit / bit-edge search for each column of ``cim``.

    src/noncoherent_integration.jl:60-115 (``_sign_search_column!``) driven by
    :654-686 (``_fill_sign_stage_column!``). Returns (stage (ndop, ncols), winner (ndop, ncols))
    where winner = edge * num_patterns + pattern of the first strict max (0 if never beaten).
    """
    ndop = plan.num_doppler_bins
    ndb = plan.num_data_bits
    pats = plan.sign_patterns_by_prn[prn]
    num_pat = pats.shape[1]
    coh_per_bit = pats.shape[0] // ndb
    sub_len = ndop // ndb
    bpc_k = plan.num_coherently_integrated_code_periods // ndb
    edge_step = bpc_k * plan.num_blocks // plan.bit_edge_search_steps
    ncols = cim.shape[1]
    stage = np.zeros((ndop, ncols), dtype=plan.rdt)
    winner = np.zeros((ndop, ncols), dtype=np.int32)
    dst_of = _half_swap_rows(ndop)
    half = ndop // 2
    for e in range(plan.bit_edge_search_steps):
        row_offset = e * edge_step
        subs = []
        for b in range(ndb):
            rows = (row_offset + b * sub_len + np.arange(sub_len)) % ndop
            buf = np.zeros((ndop, ncols), dtype=plan.cdt)
            buf[:sub_len] = cim[rows]
            subs.append(_fft(buf, 0, plan.precision).astype(plan.cdt))
        for p in range(num_pat):
            comb = np.zeros((ndop, ncols), dtype=plan.cdt)
            for b in range(ndb):
                comb = (comb + plan.rdt(pats[b * coh_per_bit, p]) * subs[b]).astype(plan.cdt)
            pw = abs2(comb).astype(plan.rdt)
            if record is not None:   # raw-bin power of candidate (e, p), keyed by its winner code
                record[e * num_pat + p] = pw
            # first half-loop (w < half) then second half-loop; strict > per cell
            for sel in (slice(0, half), slice(half, ndop)):
                w = np.arange(ndop)[sel]
                d = dst_of[sel]
                cand = pw[w]
                better = cand > stage[d]
                stage[d] = np.where(better, cand, stage[d])
                winner[d] = np.where(better, e * num_pat + p, winner[d])
    return stage, winner


def rotation_stage(cim: np.ndarray, plan: Plan, prn: int, cp_cols: np.ndarray, chunk: int = 2048,
                   record: dict | None = None):
    """Secondary-code rotation search for each column.

    src/noncoherent_integration.jl:183-297 (``_rotation_column!``) driven by :654-686.
    Returns (stage (R, ndop, ncols), winner (R, ndop, ncols)) with winner = edge*combos + combo.
    """
    ndop, nb, bs = plan.num_doppler_bins, plan.num_blocks, plan.block_size
    n_coh = plan.num_coherently_integrated_code_periods
    combos = 1 << (plan.num_data_bits - 1)
    R = plan.num_secondary_rotations
    tiled = plan.tiled_by_prn[prn]                  # (ndop, P, Q)
    Q = tiled.shape[2]
    bpc_k = n_coh // plan.num_data_bits
    edge_step = bpc_k * nb // plan.bit_edge_search_steps
    use_max = combos > 1 or plan.bit_edge_search_steps > 1
    ncols = cim.shape[1]
    stage = np.zeros((R, ndop, ncols), dtype=plan.rdt)
    winner = np.zeros((R, ndop, ncols), dtype=np.int32)
    dst_of = _half_swap_rows(ndop)
    half = ndop // 2
    pc = np.asarray(cp_cols, dtype=np.int64)
    wrap = ((nb - pc // bs) % nb) * bs + (pc % bs)
    col_row_offset = ((wrap + (bs >> 1)) // bs) % nb
    for c0 in range(0, ncols, chunk):
        c1 = min(ncols, c0 + chunk)
        cols = np.arange(c0, c1)
        for e in range(plan.bit_edge_search_steps):
            eff = (e * edge_step + col_row_offset[c0:c1]) % ndop          # (nc,)
            subs = np.zeros((n_coh, ndop, c1 - c0), dtype=plan.cdt)
            for k in range(n_coh):
                buf = np.zeros((ndop, c1 - c0), dtype=plan.cdt)
                rows = (eff[None, :] + k * nb + np.arange(nb)[:, None]) % ndop   # (nb, nc)
                buf[:nb] = cim[rows, cols[None, :]]
                subs[k] = _fft(buf, 0, plan.precision)
            # combine[q, w, c] = sum_p tiled[w, p, q] * subs[p, w, c]
            comb = np.einsum("wpq,pwc->qwc", tiled, subs, optimize=True).astype(plan.cdt)
            pw = abs2(comb).astype(plan.rdt)
            if record is not None:   # (rotation slice, winner code) -> raw-bin power (one chunk)
                for q in range(Q):
                    record[(q // combos, e * combos + q % combos)] = pw[q]
            for q in range(Q):
                ri = q // combos
                if not use_max:
                    stage[ri, dst_of, c0:c1] = pw[q]
                    winner[ri, dst_of, c0:c1] = e * combos + (q % combos)
                    continue
                for sel in (slice(0, half), slice(half, ndop)):
                    d = dst_of[sel]
                    cand = pw[q, sel]
                    cur = stage[ri, d, c0:c1]
                    better = cand > cur
                    stage[ri, d, c0:c1] = np.where(better, cand, cur)
                    winner[ri, d, c0:c1] = np.where(better, e * combos + (q % combos), winner[ri, d, c0:c1])
    return stage, winner


def code_drift_shifts(plan: Plan, step_idx: int) -> np.ndarray:
    """src/noncoherent_integration.jl:600-619 -> shifts in [0, spc) per sorted row."""
    if step_idx == 0:
        return np.zeros(plan.num_doppler_bins, dtype=np.int64)
    fs = plan.sampling_freq
    fcar = plan.system.center_freq
    dur = plan.num_coherently_integrated_code_periods * plan.samples_per_code / fs
    out = np.empty(plan.num_doppler_bins, dtype=np.int64)
    for r in range(plan.num_doppler_bins):
        raw = round(float(plan.doppler_freqs[r]) * step_idx * dur * fs / fcar)
        out[r] = raw % plan.samples_per_code
    return out


# --------------------------------------------------------------------------------------
# per-PRN surface
# --------------------------------------------------------------------------------------
@dataclass
class PrnSurface:
    power: np.ndarray          # (ndop, spc_eff) sorted Doppler rows
    winner: np.ndarray         # (ndop, spc_eff) int32 (edge*patterns + pattern), 0 on simple path
    order: str                 # "streamed" (N_nc == 1) or "materialised"


def prn_surface(plan: Plan, seg_ffts: list, prn: int) -> PrnSurface:
    """Surface of one PRN over all accumulation steps.

    N_nc == 1: src/acquire.jl:242-327; N_nc > 1: src/acquire.jl:114-163 with
    src/noncoherent_integration.jl:760-812 (drift keyed by destination sorted row).
    """
    ndop, spc, R = plan.num_doppler_bins, plan.samples_per_code, plan.num_secondary_rotations
    acc = np.zeros((ndop, plan.samples_per_code_eff), dtype=plan.rdt)
    win = np.zeros((ndop, plan.samples_per_code_eff), dtype=np.int32)
    cp = np.arange(spc)
    for m, S in enumerate(seg_ffts):
        cim = coherent_matrix(S, plan.prn_conj_ffts[prn], plan)
        shifts = code_drift_shifts(plan, m)
        dst_c = (cp[None, :] + shifts[:, None]) % spc            # (ndop, spc)
        rows = np.arange(ndop)[:, None]
        if plan.simple_path:
            P = simple_column_power(cim, plan)
            acc[rows, dst_c] += P
        elif plan.rotation_active:
            st, wn = rotation_stage(cim, plan, prn, cp)
            for s in range(R):
                acc[rows, s * spc + dst_c] += st[s]
                win[rows, s * spc + dst_c] = wn[s]
        else:
            st, wn = sign_search_stage(cim, plan, prn, cp)
            acc[rows, dst_c] += st
            win[rows, dst_c] = wn
    return PrnSurface(acc, win, "streamed" if plan.num_noncoherent_accumulations == 1 else "materialised")


def find_peak(surf: PrnSurface, plan: Plan):
    """Argmax with the reference tie-break.

    Materialised (src/est_signal_noise_power.jl:109-135): lowest effective column, then
    lowest sorted row. Streamed (src/acquire.jl:306-324,335-424): processing order
    (cp column, rotation slice, row) under strict >.
    """
    P = surf.power
    ndop = P.shape[0]
    if surf.order == "streamed" and plan.num_secondary_rotations > 1:
        spc, R = plan.samples_per_code, plan.num_secondary_rotations
        arr = P.reshape(ndop, R, spc).transpose(2, 1, 0).reshape(-1)   # (cp, s, row)
        i = int(np.argmax(arr))
        cpc, rem = divmod(i, R * ndop)
        s, row = divmod(rem, ndop)
        return float(arr[i]), row, s * spc + cpc
    arr = P.T.reshape(-1)
    i = int(np.argmax(arr))
    col, row = divmod(i, ndop)
    return float(arr[i]), row, col


def noise_power(surf: PrnSurface, plan: Plan, peak_row: int, peak_col: int) -> float:
    """OppositeRow (src/est_signal_noise_power.jl:211-227, src/acquire.jl:692-695) or
    GlobalMean (src/est_signal_noise_power.jl:150-170,229-243); summed in float64."""
    P = surf.power.astype(np.float64)
    ndop, ncols = P.shape
    if plan.noise_estimator == "global_mean":
        spchip = math.floor(plan.sampling_freq / plan.system.code_freq)
        lo = max(0, peak_col - spchip)
        hi = min(ncols - 1, peak_col + spchip)
        colsum = P.sum(axis=0)
        total = colsum.sum()
        excl = colsum[lo:hi + 1].sum()
        return (total - excl) / ((ncols - (hi - lo + 1)) * ndop)
    opp = (peak_row + ndop // 2) % ndop
    return P[opp].sum() / ncols


# --------------------------------------------------------------------------------------
# secondary-code phase, src/acquire.jl:503-538
# --------------------------------------------------------------------------------------
def candidate_powers(plan: Plan, signal, prn: int, row: int, col: int, interm_freq_hz: float = 0.0) -> dict:
    """Power of every data-bit / bit-edge candidate at surface cell (row, col) in the last
    accumulation step, keyed by the winner code the surface records there (edge * patterns +
    pattern; edge * combinations + combination within the rotation slice of `col`). The stage
    keeps the first strict maximum of these (src/noncoherent_integration.jl:99-112,278-293);
    candidates tied in exact arithmetic are broken by rounding. Test helper for the sign and
    rotation paths."""
    segs = all_segment_ffts(plan, signal, interm_freq_hz)
    m = len(segs) - 1
    cim = coherent_matrix(segs[m], plan.prn_conj_ffts[prn], plan)
    spc = plan.samples_per_code
    s_slice, c = divmod(col, spc)
    src = (c - int(code_drift_shifts(plan, m)[row])) % spc
    raw = np.where(_half_swap_rows(plan.num_doppler_bins) == row)[0]
    rec: dict = {}
    if plan.rotation_active:
        rotation_stage(cim[:, [src]], plan, prn, np.array([src]), record=rec)
        return {k[1]: float(max(v[w, 0] for w in raw)) for k, v in rec.items() if k[0] == s_slice}
    sign_search_stage(cim[:, [src]], plan, prn, np.array([src]), record=rec)
    return {k: float(max(v[w, 0] for w in raw)) for k, v in rec.items()}


def estimate_secondary_code_phase(plan: Plan, prn: int, signal, interm_freq_hz: float,
                                  code_phase: float, doppler_hz: float) -> int:
    system = plan.system
    L = plan.num_secondary_rotations
    spc = plan.samples_per_code
    fs = plan.sampling_freq
    code = gen_code(spc, system, prn, fs, system.code_freq, code_phase).astype(np.float64)
    phase_step = -2.0 * math.pi * (interm_freq_hz + doppler_hz) / fs
    n = np.arange(spc)
    zs = np.empty(L, dtype=np.complex128)
    sig = np.asarray(signal)
    for k in range(L):
        base = k * spc
        carr = np.exp(1j * (phase_step * base + phase_step * n))
        zs[k] = np.sum(sig[base:base + spc].astype(np.complex128) * carr * code)
    best_r, best_mag = 0, -1.0
    for r in range(L):
        s = sum(system.secondary_value(prn, (k + r) % L) * zs[k] for k in range(L))
        mag = abs(s) ** 2
        if mag > best_mag:
            best_mag, best_r = mag, r
    return best_r


# --------------------------------------------------------------------------------------
# acquire!, src/acquire.jl:54-89, :544-671, :681-781
# --------------------------------------------------------------------------------------
@dataclass
class Result:
    system: System
    prn: int
    sampling_frequency: float
    carrier_doppler: float
    code_phase: float
    secondary_code_phase: int | None
    CN0: float
    noise_power: float
    peak_to_noise_ratio: float
    num_noncoherent_integrations: int
    power_bins: np.ndarray | None
    dopplers: np.ndarray
    num_blocks: int
    block_size: int
    num_secondary_rotations: int
    # additions (not in the reference result):
    peak_power: float = 0.0
    peak_doppler_bin: int = 0        # 0-based sorted row
    peak_code_bin: int = 0           # 0-based effective column
    sign_pattern: int = -1           # data-bit combination index at the peak (-1 off the sign path)
    bit_edge: int = -1               # bit-edge alignment index at the peak (-1 off the sign path)


def get_num_cells(r: Result) -> int:
    """src/Acquisition.jl:124-126."""
    return len(r.dopplers) * r.num_blocks * r.block_size * r.num_secondary_rotations


def is_detected(r: Result, pfa: float = 0.01) -> bool:
    """src/Acquisition.jl:135-142."""
    return r.peak_to_noise_ratio > cfar_threshold(pfa, get_num_cells(r), r.num_noncoherent_integrations)


def all_segment_ffts(plan: Plan, signal, interm_freq_hz: float) -> list:
    seg_len = plan.num_coherently_integrated_code_periods * plan.samples_per_code
    return [signal_block_ffts(downconvert(signal, m * seg_len, seg_len, interm_freq_hz,
                                          plan.sampling_freq, plan.precision), plan)
            for m in range(plan.num_noncoherent_accumulations)]


def extract_result(plan: Plan, prn: int, surf: PrnSurface, signal, interm_freq_hz: float,
                   subsample_interpolation: bool, store_power_bins: bool) -> Result:
    """src/acquire.jl:544-671 / :681-781."""
    system = plan.system
    fs = plan.sampling_freq
    fc = system.code_freq
    code_length = system.code_length
    ndop = plan.num_doppler_bins
    spc = plan.samples_per_code
    peak, prow, pcol = find_peak(surf, plan)
    f32 = np.float32
    noise = f32(noise_power(surf, plan, prow, pcol))
    peak32 = f32(peak)
    signal_power = f32(peak32 - noise)
    pnr = f32((signal_power + noise) / noise)
    t_coh = plan.num_coherently_integrated_code_periods * (code_length / fc)
    with np.errstate(invalid="ignore", divide="ignore"):
        cn0 = 10 * math.log10(float(signal_power) / float(noise) / t_coh) if signal_power > 0 else float("nan")
    rotation_block = pcol // spc
    scrambled = pcol % spc
    delay = fmdbzp_column_to_tau(scrambled, plan.num_blocks, plan.block_size)
    code_phase = (-delay * fc / fs) % code_length
    doppler = float(plan.doppler_freqs[prow])
    P = surf.power
    if subsample_interpolation:
        col_l = (scrambled - 1) % spc + rotation_block * spc
        col_r = (scrambled + 1) % spc + rotation_block * spc
        row_l = ndop - 1 if prow == 0 else prow - 1
        row_r = 0 if prow == ndop - 1 else prow + 1
        pl, pr = f32(P[prow, col_l]), f32(P[prow, col_r])
        dl, dr = f32(P[row_l, pcol]), f32(P[row_r, pcol])
        sq = f32(np.sqrt(noise))
        if max(pl, pr) > sq:
            frac = parabolic_interp(pl, peak32, pr)
            d_int = float(delay) if isinstance(frac, float) else float(f32(f32(delay) + frac))
            code_phase = (-d_int * fc / fs) % code_length
        if max(dl, dr) > sq:
            frac = parabolic_interp(dl, peak32, dr)
            doppler = doppler + float(frac) * plan.doppler_step
    sec_phase = None
    if plan.num_secondary_rotations > 1:
        num_cells = ndop * spc * plan.num_secondary_rotations
        thr = cfar_threshold(0.01, num_cells, plan.num_noncoherent_accumulations)
        if float(pnr) > thr:
            sec_phase = estimate_secondary_code_phase(plan, prn, signal, interm_freq_hz, code_phase, doppler)
    sign_pattern = bit_edge = -1
    if not plan.simple_path:
        w = int(surf.winner[prow, pcol])
        if plan.rotation_active:
            combos = 1 << (plan.num_data_bits - 1)
            bit_edge, sign_pattern = divmod(w, combos)
        else:
            npat = plan.sign_patterns_by_prn[prn].shape[1]
            bit_edge, sign_pattern = divmod(w, npat)
    return Result(system, prn, fs, doppler, float(code_phase), sec_phase, float(cn0), float(noise), float(pnr),
                  plan.num_noncoherent_accumulations, P.astype(np.float32).copy() if store_power_bins else None,
                  plan.doppler_freqs, plan.num_blocks, plan.block_size, plan.num_secondary_rotations,
                  peak_power=float(peak32), peak_doppler_bin=prow, peak_code_bin=pcol,
                  sign_pattern=sign_pattern, bit_edge=bit_edge)


def acquire_b(plan: Plan, signal, prns, *, interm_freq: float = 0.0, subsample_interpolation: bool = False,
              store_power_bins: bool = False, return_surfaces: bool = False):
    """``acquire!`` (src/acquire.jl:54-89)."""
    prns = [int(p) for p in np.atleast_1d(prns)]
    if not all(p in plan.avail_prns for p in prns):
        raise ArgumentError(f"All requested PRNs must be in plan.avail_prns. Got: {prns}, "
                            f"available: {plan.avail_prns}")
    seg_len = plan.num_coherently_integrated_code_periods * plan.samples_per_code
    nseg = len(signal) // seg_len
    if nseg < plan.num_noncoherent_accumulations:
        raise ArgumentError(f"Signal has {len(signal)} samples -> {nseg} full segments of {seg_len}, but "
                            f"plan.num_noncoherent_accumulations={plan.num_noncoherent_accumulations}. "
                            "Provide a longer signal.")
    seg_ffts = all_segment_ffts(plan, signal, interm_freq)
    out, surfs = [], []
    for prn in prns:
        surf = prn_surface(plan, seg_ffts, prn)
        out.append(extract_result(plan, prn, surf, signal, interm_freq, subsample_interpolation,
                                  store_power_bins))
        surfs.append(surf)
    return (out, surfs) if return_surfaces else out


# --------------------------------------------------------------------------------------
# chip-sorted surface, src/plot.jl:16-20,35-57
# --------------------------------------------------------------------------------------
def fmdbzp_column_to_tau(c: int, num_blocks: int, block_size: int) -> int:
    """src/plot.jl:16-20."""
    return ((num_blocks - c // block_size) % num_blocks) * block_size + c % block_size


def _julia_fmod(x: float, y: float) -> float:
    r = math.fmod(x, y)
    if r == 0.0:
        return math.copysign(0.0, y)
    return r + y if (r > 0) != (y > 0) else r


def fmdbzp_sort_by_chip(power_bins: np.ndarray, num_blocks: int, block_size: int, code_freq: float,
                        fs: float):
    """src/plot.jl:35-57 -> (chip_axis, chip_sorted_power_bins, chip_order)."""
    width = power_bins.shape[1]
    code_length = width * code_freq / fs
    chip = np.array([_julia_fmod(-fmdbzp_column_to_tau(c, num_blocks, block_size) * code_freq / fs, code_length)
                     for c in range(width)])
    order = np.argsort(chip, kind="stable")
    return chip[order], power_bins[:, order], order


# --------------------------------------------------------------------------------------
# signal model, src/generate_test_signal.jl:45-68 (code Doppler, carrier, AWGN)
# --------------------------------------------------------------------------------------
def clean_signal(system: System, prn: int, n: int, fs: float, doppler: float, code_phase: float,
                 interm_freq: float = 0.0, phase_offset: float = math.pi / 8, amplitude: float = 1.0):
    fc = system.code_freq + doppler * system.code_freq / system.center_freq
    code = gen_code(n, system, prn, fs, fc, code_phase).astype(np.float64)
    t = np.arange(n)
    carrier = np.exp(1j * (2 * math.pi * t * (interm_freq + doppler) / fs + phase_offset))
    return amplitude * code * carrier
