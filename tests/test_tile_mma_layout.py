"""Operand layout of the tensor-core coherent tile (csrc/acq_tile_mma.cuh), checked on the CPU.

k_tile_stubs stores, per row, the blocks Q_s[d][e] = u[8 s + d + e] (8 rows of 16 bytes); the
MMA reads the Hankel matrix H[j, b] = u[j + b] through a K-major no-swizzle descriptor whose
leading and stride byte offsets are both 128, and the code rows through one with stride
KCH * 128. This model follows the kernels' index arithmetic (stub row order, descriptor address
formula, TMEM column map, drain offsets) and checks that the product equals the FFT form of the
tile, (1/F) IFFT(FFT(u) * conj(FFT(c_m)))[0:bs), for block sizes with one and two lag halves.
"""
import numpy as np
import pytest


def ks(bs):
    return (bs + 15) // 16


def nh(bs):
    return (bs + 127) // 128


def n_stubs(bs):
    return 2 * ks(bs) + 16 * nh(bs) - 1


def stub_rows(u, bs):
    """Element-addressed image of one operand's Q_s blocks, as k_tile_stubs writes them."""
    nst = n_stubs(bs)
    span = 8 * nst + 8
    x = np.zeros(span, dtype=u.dtype)
    x[: min(len(u), span)] = u[:span]
    mem = np.zeros(nst * 64, dtype=u.dtype)
    for idx in range(nst * 8):            # 16-byte rows: Q_s row d = x[8 s + d : 8 s + d + 8]
        base = (idx >> 3) * 8 + (idx & 7)
        mem[idx * 8: idx * 8 + 8] = x[base: base + 8]
    return mem


def read_operand(mem, start_elem, lbo, sbo, rows, kdim=16):
    """rows x kdim operand through a K-major no-swizzle descriptor (byte offsets / 2 = elements)."""
    r = np.arange(rows)[:, None]
    k = np.arange(kdim)[None, :]
    addr = start_elem * 2 + (r >> 3) * sbo + (k >> 3) * lbo + (r & 7) * 16 + (k & 7) * 2
    return mem[addr // 2]


def code_rows(codes, bs, nb, n, chunk):
    """Element image of the B operand (128 code rows of one block, K-major, KCH 16-byte chunks)."""
    kch = 2 * ks(bs)
    mem = np.zeros(128 * kch * 8)
    for row in range(128):
        gr = chunk * 128 + row
        pi, m = divmod(gr, nb)
        for kc in range(kch):
            for e in range(8):
                b = kc * 8 + e
                v = codes[pi, m * bs + b] if (pi < n and b < bs) else 0.0
                mem[((row >> 3) * (kch * 128) + kc * 128 + (row & 7) * 16) // 2 + e] = v
    return mem


@pytest.mark.parametrize("bs,nb,n", [(40, 4, 3), (125, 4, 2), (200, 2, 1)])
def test_hankel_descriptor_product_equals_the_fft_tile(bs, nb, n):
    rng = np.random.default_rng(bs)
    spc = nb * bs
    F = 1 << int(np.ceil(np.log2(2 * bs)))
    codes = rng.choice([-1.0, 1.0], size=(n, spc))
    rows = [(rng.standard_normal(2 * bs) + 1j * rng.standard_normal(2 * bs)) for _ in range(nb)]
    kch, nst = 2 * ks(bs), n_stubs(bs)
    for g, u in enumerate(rows):
        k = g % nb
        # the four operands of the row (the split into hi + lo is exact here: lo = 0)
        ops = [stub_rows(u.real, bs), stub_rows(u.real * 0, bs), stub_rows(u.imag, bs), stub_rows(u.imag * 0, bs)]
        for chunk in range((n * nb + 127) // 128):
            bmem = code_rows(codes, bs, nb, n, chunk)
            # tensor memory: lag half h, Re at columns 256 h + col, Im at 256 h + 128 + col
            D = np.zeros((128, 512))
            for h in range(nh(bs)):
                for c in range(2):
                    acc = np.zeros((128, 128))
                    for kstep in range(ks(bs)):
                        B = read_operand(bmem, kstep * 128, 128, kch * 128, 128)
                        for part in range(2):
                            A = read_operand(ops[2 * c + part], 64 * (16 * h + 2 * kstep), 128, 128, 128)
                            acc += A @ B.T
                    D[:, h * 256 + c * 128: h * 256 + c * 128 + 128] = acc
            for col in range(128):
                gr = chunk * 128 + col
                pi, m = divmod(gr, nb)
                if pi >= n:
                    continue
                r = (m - k) % nb            # the drain's column block for code block m
                got = np.array([D[j % 128, (j // 128) * 256 + col] + 1j * D[j % 128, (j // 128) * 256 + 128 + col]
                                for j in range(bs)])
                cm = np.zeros(F)
                cm[:bs] = codes[pi, ((k + r) % nb) * bs: ((k + r) % nb + 1) * bs]
                ref = np.fft.ifft(np.fft.fft(u, F) * np.conj(np.fft.fft(cm)))[:bs]
                assert np.abs(got - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), (g, pi, m)


def test_stub_rows_cover_every_lag_and_k_block():
    # the largest Q_s index the MMAs read is the last stub: (2 KS - 1) + 15 + 16 (NH - 1)
    for bs in (16, 100, 128, 129, 250, 256):
        last = (2 * ks(bs) - 1) + 15 + 16 * (nh(bs) - 1)
        assert last == n_stubs(bs) - 1
        # every lag j < bs and tap b < bs lands inside the span the stub rows copy
        assert (bs - 1) + (bs - 1) < 8 * n_stubs(bs) + 8
