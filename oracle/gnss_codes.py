"""Oracle (test infrastructure only): CPU restatement of the GNSS code generators.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this module. It is the checker, never the product: the
product generates codes in C++ inside the C-ABI library.

The reference obtains codes from GNSSSignals.jl (compat "3, 4", not vendored and
not pinned by a Manifest). Its call sites are ``src/plan.jl:241`` (plan-time
replica), ``src/acquire.jl:509`` (secondary-code despread replica) and
``src/generate_test_signal.jl:47-54`` (test signals). This file restates the
published algorithms those packages implement:

* GPS L1 C/A Gold codes (IS-GPS-200): G1 = 1 + x^3 + x^10,
  G2 = 1 + x^2 + x^3 + x^6 + x^8 + x^9 + x^10, both seeded with ones, chip =
  G1[10] xor G2[s1] xor G2[s2] with the PRN's phase-selector taps. Pinned here by
  the ICD's first-10-chip octal values (``tests/test_oracle_golden.py``).
* GPS L5I (IS-GPS-705): XA = 1 + x^9 + x^10 + x^12 + x^13 (ones, short-cycled
  after 8190 chips), XB = 1 + x + x^3 + x^4 + x^6 + x^7 + x^8 + x^12 + x^13
  seeded with the all-ones state advanced by the PRN's XB code advance.
  The NH10 secondary code is pinned by ``test/sign_patterns.jl:45-46`` and is
  baked into the sampled code across primary periods, as GNSSSignals does
  (``test/secondary_code_search.jl:8-9``). PRN 1 is pinned end-to-end by the
  numeric golden vector of ``test/secondary_code_search.jl:119-130``.
* Galileo E1B: the ICD memory codes are not available here. Seeded synthetic
  +-1 memory codes (splitmix64 of prn<<32|chip) with a BOC(1,1) sub-carrier stand
  in for them and are labelled synthetic. Parity is unaffected because oracle and
  product share the same definition.

Sampling (GNSSSignals ``gen_code``): sample i takes chip
floor(start_phase + i*fc/fs) modulo the full (primary x secondary) length. When
fc and fs are whole Hz and start_phase is 0 the floor is taken exactly in integer
arithmetic; otherwise in float64 as ``start_phase + i * (fc / fs)``. GNSSSignals
uses a fixed-point phase accumulator whose rounding is not available here, so
samples where i*fc/fs is an exact integer other than 0 are "parity unpinned".
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# IS-GPS-200 phase-selector taps for PRN 1..32 (G2 stages, 1-based).
_L1CA_TAPS = [(2, 6), (3, 7), (4, 8), (5, 9), (1, 9), (2, 10), (1, 8), (2, 9), (3, 10), (2, 3),
              (3, 4), (5, 6), (6, 7), (7, 8), (8, 9), (9, 10), (1, 4), (2, 5), (3, 6), (4, 7),
              (5, 8), (6, 9), (1, 3), (4, 6), (5, 7), (6, 8), (7, 9), (8, 10), (1, 6), (2, 7),
              (3, 8), (4, 9)]

# IS-GPS-705 XB code advance (chips) for the I5 code of PRN 1..37.
_L5I_XB_ADVANCE = [266, 365, 804, 1138, 1509, 1559, 1756, 2084, 2170, 2303, 2527, 2687, 2930,
                   3471, 3940, 4132, 4332, 4924, 5343, 5443, 5641, 5816, 5898, 5918, 5955, 6243,
                   6345, 6477, 6518, 6875, 7168, 7187, 7329, 7577, 7720, 7777, 8057]

# NH10 as +-1 (bits 0000110101, 0 -> +1), test/sign_patterns.jl:45-46.
NH10 = np.array([1, 1, 1, 1, -1, -1, 1, -1, 1, -1], dtype=np.int8)


def _bits_to_pm1(bits) -> np.ndarray:
    return (1 - 2 * np.asarray(bits, dtype=np.int16)).astype(np.int8)


def l1ca_chips(prn: int) -> np.ndarray:
    if not 1 <= prn <= 32:
        raise ValueError(f"GPS L1 C/A PRN must be in 1:32, got {prn}")
    s1, s2 = _L1CA_TAPS[prn - 1]
    g1 = [1] * 10
    g2 = [1] * 10
    out = np.empty(1023, dtype=np.int16)
    for i in range(1023):
        out[i] = g1[9] ^ g2[s1 - 1] ^ g2[s2 - 1]
        f1 = g1[2] ^ g1[9]
        f2 = g2[1] ^ g2[2] ^ g2[5] ^ g2[7] ^ g2[8] ^ g2[9]
        g1 = [f1] + g1[:9]
        g2 = [f2] + g2[:9]
    return _bits_to_pm1(out)


def _l5_xa_step(r):
    return [r[8] ^ r[9] ^ r[11] ^ r[12]] + r[:12]


def _l5_xb_step(r):
    return [r[0] ^ r[2] ^ r[3] ^ r[5] ^ r[6] ^ r[7] ^ r[11] ^ r[12]] + r[:12]


def l5i_primary_chips(prn: int) -> np.ndarray:
    if not 1 <= prn <= len(_L5I_XB_ADVANCE):
        raise ValueError(f"GPS L5I PRN must be in 1:{len(_L5I_XB_ADVANCE)}, got {prn}")
    xb = [1] * 13
    for _ in range(_L5I_XB_ADVANCE[prn - 1]):
        xb = _l5_xb_step(xb)
    xa = [1] * 13
    out = np.empty(10230, dtype=np.int16)
    for i in range(10230):
        if i == 8190:  # XA short cycle: restart after 8190 chips
            xa = [1] * 13
        out[i] = xa[12] ^ xb[12]
        xa = _l5_xa_step(xa)
        xb = _l5_xb_step(xb)
    return _bits_to_pm1(out)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def e1b_synthetic_chips(prn: int) -> np.ndarray:
    """Seeded synthetic E1B memory code (NOT the ICD code; labelled synthetic)."""
    if not 1 <= prn <= 50:
        raise ValueError(f"Galileo E1B PRN must be in 1:50, got {prn}")
    with np.errstate(over="ignore"):
        k = (np.uint64(prn) << np.uint64(32)) | np.arange(4092, dtype=np.uint64)
        h = _splitmix64(k)
    return np.where((h >> np.uint64(63)) == 1, -1, 1).astype(np.int8)


@dataclass(frozen=True)
class System:
    name: str
    code_length: int            # primary chips
    code_freq: float            # Hz
    center_freq: float          # Hz
    data_freq: float            # Hz (0 or inf for pilots)
    secondary: np.ndarray | None = field(default=None, compare=False)
    boc11: bool = False

    @property
    def secondary_code_length(self) -> int:
        return 1 if self.secondary is None else len(self.secondary)

    def primary_chips(self, prn: int) -> np.ndarray:
        if self.name == "GPSL1CA":
            return l1ca_chips(prn)
        if self.name == "GPSL5I":
            return l5i_primary_chips(prn)
        if self.name == "GalileoE1B":
            return e1b_synthetic_chips(prn)
        raise ValueError(self.name)

    def full_chips(self, prn: int) -> np.ndarray:
        """Primary code with the secondary code baked across periods."""
        p = self.primary_chips(prn).astype(np.int8)
        if self.secondary is None:
            return p
        return (np.tile(p, len(self.secondary)).reshape(len(self.secondary), -1)
                * self.secondary[:, None]).reshape(-1).astype(np.int8)

    def secondary_value(self, prn: int, i: int) -> int:
        return 1 if self.secondary is None else int(self.secondary[i % len(self.secondary)])


GPSL1CA = System("GPSL1CA", 1023, 1.023e6, 1575.42e6, 50.0)
GPSL5I = System("GPSL5I", 10230, 10.23e6, 1176.45e6, 100.0, secondary=NH10)
GalileoE1B = System("GalileoE1B", 4092, 1.023e6, 1575.42e6, 250.0, boc11=True)

SYSTEMS = {s.name: s for s in (GPSL1CA, GPSL5I, GalileoE1B)}


def _is_whole(x: float) -> bool:
    return float(x).is_integer() and abs(x) < 2**52


def code_phase_indices(n: int, fs: float, fc: float, start_phase: float = 0.0):
    """Integer chip index and fractional chip phase of samples 0..n-1."""
    i = np.arange(n, dtype=np.int64)
    if start_phase == 0.0 and _is_whole(fs) and _is_whole(fc):
        fsi, fci = int(fs), int(fc)
        num = i * fci
        idx = num // fsi
        frac2 = 2 * (num - idx * fsi) >= fsi     # frac >= 0.5 (BOC half)
        return idx, frac2
    ph = start_phase + i.astype(np.float64) * (fc / fs)
    idx = np.floor(ph).astype(np.int64)
    frac2 = (ph - idx) >= 0.5
    return idx, frac2


def gen_code(n: int, system: System, prn: int, fs: float, fc: float | None = None,
             start_phase: float = 0.0) -> np.ndarray:
    """Sampled +-1 code (int8), GNSSSignals ``gen_code`` semantics."""
    if fc is None:
        fc = system.code_freq
    chips = system.full_chips(prn)
    L = len(chips)
    sp = math.fmod(start_phase, L)
    if sp < 0:
        sp += L
    idx, frac2 = code_phase_indices(n, fs, fc, sp)
    out = chips[np.mod(idx, L)].astype(np.int8)
    if system.boc11:
        out = np.where(frac2, -out, out).astype(np.int8)
    return out
