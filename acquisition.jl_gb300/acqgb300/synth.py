"""Seeded synthetic GNSS recordings (host, numpy) following the reference's signal model.

Model (src/generate_test_signal.jl:45-68): per satellite, the code sampled at the Doppler-
shifted code rate f_code + f_d * f_code / f_carrier with GNSSSignals ``gen_code`` semantics,
times the carrier exp(i(2 pi (IF + f_d) t + phi0)), times +-1 data bits; plus complex white
Gaussian noise with the statistics of Julia's ``randn(ComplexF64)`` (unit total variance).

Scaling: noise has unit total power; a satellite at C/N0 (dB-Hz) has amplitude
sqrt(10^(CN0/10) / fs) — the reference's ``unit_noise_power = true`` convention.

Quantisers: ``to_ci16`` (x * 2^10, round, saturate) and ``to_ci8_3bit`` (3-bit, levels
+-1..+-7 at 0.5 sigma per component). Codes come from the C++ generator of libacqgb300.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .api import GNSSSystem


@dataclass
class Satellite:
    prn: int
    cn0: float                   # dB-Hz
    doppler: float               # Hz
    code_phase: float            # chips
    phase: float = math.pi / 8   # carrier phase offset, rad
    data_bits: bool = True       # +-1 data bits at the system's data rate
    bit_offset: float = 0.0      # seconds into the first data bit at sample 0


@dataclass
class Recording:
    system: GNSSSystem
    fs: float
    samples: np.ndarray           # complex64 (or quantised, see `quantised`)
    sats: list = field(default_factory=list)
    interm_freq: float = 0.0


def synth(system: GNSSSystem, fs: float, n: int, sats, seed: int, interm_freq: float = 0.0,
          noise: bool = True) -> np.ndarray:
    """complex128 samples of the model above."""
    rng = np.random.default_rng(seed)
    t = np.arange(n, dtype=np.float64)
    out = np.zeros(n, dtype=np.complex128)
    for s in sats:
        fc = system.code_frequency + s.doppler * system.code_frequency / system.center_frequency
        code = system.gen_code(n, s.prn, fs, fc, s.code_phase).astype(np.float64)
        carrier = np.exp(1j * (2 * math.pi * t * (interm_freq + s.doppler) / fs + s.phase))
        amp = math.sqrt(10 ** (s.cn0 / 10) / fs)
        x = amp * code * carrier
        if s.data_bits and math.isfinite(system.data_frequency) and system.data_frequency > 0:
            bit_idx = np.floor((t / fs + s.bit_offset) * system.data_frequency).astype(np.int64)
            nb = int(bit_idx[-1]) + 1
            bits = rng.choice(np.array([-1.0, 1.0]), size=nb)
            x = x * bits[bit_idx]
        out += x
    if noise:
        out += (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
    return out


def to_ci16(x: np.ndarray, scale: float = 2.0 ** 10) -> np.ndarray:
    """Interleaved int16 (n, 2): round(x * scale), saturated."""
    re = np.clip(np.rint(x.real * scale), -32768, 32767)
    im = np.clip(np.rint(x.imag * scale), -32768, 32767)
    return np.stack([re, im], axis=-1).astype(np.int16)


def to_ci8_3bit(x: np.ndarray) -> np.ndarray:
    """Interleaved int8 (n, 2): 3-bit quantiser, odd levels -7..7, step 0.5 sigma per component."""
    sigma = math.sqrt(0.5)

    def q(v):
        k = np.floor(v / (0.5 * sigma))
        return np.clip(2 * k + 1, -7, 7)

    return np.stack([q(x.real), q(x.imag)], axis=-1).astype(np.int8)


def random_sats(rng: np.random.Generator, prns, cn0_range, doppler_max, code_length, bit_period_s=0.0):
    out = []
    for prn in prns:
        out.append(Satellite(int(prn), float(rng.uniform(*cn0_range)), float(rng.uniform(-doppler_max, doppler_max)),
                             float(rng.uniform(0, code_length)), float(rng.uniform(0, 2 * math.pi)), True,
                             float(rng.uniform(0, bit_period_s)) if bit_period_s > 0 else 0.0))
    return out


def ragged_batch(seed: int = 3, n_recordings: int = 64, n_antennas: int = 4, max_nnc: int = 8):
    """Seeded ragged batch: recordings of uneven length (2-80 ms) from several antennas mixing
    GPS L1 C/A (5 MHz), Galileo E1B (12 MHz, synthetic codes) and GPS L5I (25 MHz, NH10).

    Returns a list of dicts: system, fs, samples (complex64), prns, n_coh, n_nc, cov, sats, antenna.
    8-32 PRNs per recording, 0-6 present at C/N0 30-48 dB-Hz, Doppler +-8 kHz. Coherent periods:
    1 for L1 C/A and E1B; 10 for L5I recordings of >= 20 ms (secondary-code search), else 1.
    Accumulations: floor(length / coherent time), capped at ``max_nnc``.
    """
    from .api import GalileoE1B, GPSL1CA, GPSL5I
    rng = np.random.default_rng(seed)
    kinds = [("GPSL1CA", GPSL1CA(), 5e6, 32), ("GalileoE1B", GalileoE1B(), 12e6, 36), ("GPSL5I", GPSL5I(), 25e6, 32)]
    # one satellite geometry per (antenna, system): same PRNs/Dopplers, per-antenna phases
    geo = {}
    for a in range(n_antennas):
        for name, sysm, _, maxprn in kinds:
            npres = int(rng.integers(0, 7))
            present = rng.choice(np.arange(1, maxprn + 1), size=npres, replace=False).tolist()
            geo[(a, name)] = [(int(p), float(rng.uniform(30, 48)), float(rng.uniform(-8000, 8000)),
                               float(rng.uniform(0, sysm.code_length))) for p in present]
    out = []
    for i in range(n_recordings):
        name, sysm, fs, maxprn = kinds[i % 3]
        ant = (i // 3) % n_antennas
        length_ms = float(rng.uniform(2.0, 80.0))
        t_code_ms = 1000.0 * sysm.code_length / sysm.code_frequency
        n_coh = 10 if (name == "GPSL5I" and length_ms >= 20.0) else 1
        t_coh = n_coh * t_code_ms
        n_nc = int(max(1, min(max_nnc, math.floor(length_ms / t_coh))))
        spc = int(math.ceil(sysm.code_length / sysm.code_frequency * fs))
        n = max(int(length_ms * 1e-3 * fs), n_nc * n_coh * spc)
        sats = [Satellite(p, c, d, cp, float(rng.uniform(0, 2 * math.pi)), True, 0.0) for (p, c, d, cp) in geo[(ant, name)]]
        x = synth(sysm, fs, n, sats, seed * 1000 + i).astype(np.complex64)
        n_prn = int(rng.integers(8, 33))
        searched = set(rng.choice(np.arange(1, maxprn + 1), size=min(n_prn, maxprn), replace=False).tolist())
        searched |= {s.prn for s in sats}
        out.append(dict(system=sysm, fs=fs, samples=x, prns=sorted(int(p) for p in searched), n_coh=n_coh,
                        n_nc=n_nc, cov=8000.0, sats=sats, antenna=ant, length_ms=length_ms))
    return out


def synth_device(system: GNSSSystem, fs: float, n: int, sats, seed: int, *, interm_freq: float = 0.0,
                 noise: bool = True, dtype: str = "cf32", out=None, stream: int = 0):
    """The same signal model generated on the GPU (``acq_synth_signal``) into a CUDA tensor (or
    ``out``: a device pointer or tensor). Data bits and noise come from a counter-based generator
    (not numpy's stream); the code and carrier match :func:`synth`."""
    import ctypes as C
    import torch
    from . import _lib as L
    from .api import _check
    code = {"cf32": L.ACQ_CF32, "ci16": L.ACQ_CI16, "ci8": L.ACQ_CI8, "cf64": L.ACQ_CF64}[dtype]
    arr = (L.SynthSat * max(1, len(sats)))()
    for i, s in enumerate(sats):
        arr[i] = L.SynthSat(int(s.prn), 1 if s.data_bits else 0, float(s.cn0), float(s.doppler), float(s.code_phase),
                            float(s.phase), float(s.bit_offset))
    if out is None:
        out = {"cf32": lambda: torch.empty(n, dtype=torch.complex64, device="cuda"),
               "cf64": lambda: torch.empty(n, dtype=torch.complex128, device="cuda"),
               "ci16": lambda: torch.empty((n, 2), dtype=torch.int16, device="cuda"),
               "ci8": lambda: torch.empty((n, 2), dtype=torch.int8, device="cuda")}[dtype]()
    ptr = out.data_ptr() if hasattr(out, "data_ptr") else int(out)
    _check(L.load().acq_synth_signal(system.sid, float(fs), int(n), arr, len(sats), float(interm_freq),
                                     int(seed) & 0xFFFFFFFFFFFFFFFF, 1 if noise else 0, code, C.c_void_p(ptr),
                                     C.c_void_p(stream)))
    return out
