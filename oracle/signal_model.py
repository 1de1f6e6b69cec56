"""Seeded synthetic recordings for the CPU legs of the benchmark (test infrastructure only).

The signal model of src/generate_test_signal.jl:45-68, restated on the oracle's own code
generator (oracle/gnss_codes.py) so that the CPU baseline never touches the product library:
per satellite the code sampled at the Doppler-shifted code rate f_code + f_d f_code / f_carrier,
the carrier exp(i(2 pi (IF + f_d) t + phi0)), +-1 data bits at the system's data rate; plus
complex white Gaussian noise of unit total power. A satellite at C/N0 (dB-Hz) has amplitude
sqrt(10^(CN0/10) / fs).

The random streams (satellite draws, data bits, noise) are consumed in the same order as the
product's host generator, so the same seed gives byte-identical recordings; a CPU test pins
that equality for every benchmark workload.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .gnss_codes import System, gen_code


@dataclass
class Sat:
    prn: int
    cn0: float
    doppler: float
    code_phase: float
    phase: float = math.pi / 8
    data_bits: bool = True
    bit_offset: float = 0.0


def random_sats(rng: np.random.Generator, prns, cn0_range, doppler_max, code_length, bit_period_s=0.0):
    """Satellites with C/N0, Doppler, code phase, carrier phase and bit offset drawn in order."""
    out = []
    for prn in prns:
        out.append(Sat(int(prn), float(rng.uniform(*cn0_range)), float(rng.uniform(-doppler_max, doppler_max)),
                       float(rng.uniform(0, code_length)), float(rng.uniform(0, 2 * math.pi)), True,
                       float(rng.uniform(0, bit_period_s)) if bit_period_s > 0 else 0.0))
    return out


def synth(system: System, fs: float, n: int, sats, seed: int, interm_freq: float = 0.0) -> np.ndarray:
    """complex128 samples: the satellites' signals plus unit-power complex white noise."""
    rng = np.random.default_rng(seed)
    t = np.arange(n, dtype=np.float64)
    out = np.zeros(n, dtype=np.complex128)
    for s in sats:
        fc = system.code_freq + s.doppler * system.code_freq / system.center_freq
        code = gen_code(n, system, s.prn, fs, fc, s.code_phase).astype(np.float64)
        carrier = np.exp(1j * (2 * math.pi * t * (interm_freq + s.doppler) / fs + s.phase))
        x = math.sqrt(10 ** (s.cn0 / 10) / fs) * code * carrier
        if s.data_bits and math.isfinite(system.data_freq) and system.data_freq > 0:
            bit_idx = np.floor((t / fs + s.bit_offset) * system.data_freq).astype(np.int64)
            bits = rng.choice(np.array([-1.0, 1.0]), size=int(bit_idx[-1]) + 1)
            x = x * bits[bit_idx]
        out += x
    out += (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
    return out


def to_ci16(x: np.ndarray, scale: float = 2.0 ** 10) -> np.ndarray:
    """Interleaved int16 (n, 2): round(x * scale), saturated."""
    re = np.clip(np.rint(x.real * scale), -32768, 32767)
    im = np.clip(np.rint(x.imag * scale), -32768, 32767)
    return np.stack([re, im], axis=-1).astype(np.int16)


def to_ci8_3bit(x: np.ndarray) -> np.ndarray:
    """Interleaved int8 (n, 2): 3-bit quantiser, odd levels -7..7, step 0.5 sigma per component."""
    step = 0.5 * math.sqrt(0.5)
    q = lambda v: np.clip(2 * np.floor(v / step) + 1, -7, 7)  # noqa: E731
    return np.stack([q(x.real), q(x.imag)], axis=-1).astype(np.int8)
