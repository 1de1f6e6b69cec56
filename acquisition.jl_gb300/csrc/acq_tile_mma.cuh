// acq_tile_mma.cuh — the coherent tile as a correlation GEMM on the 5th-generation tensor cores.
//
// The tile (src/coherent_integration.jl:136-171) is, per row g and code block m,
//   T[g, r bs + j] = (1/F) IFFT(U_g .* C*_m)[j],   m = (k + r) mod nb,  k = g mod nb,  j < bs,
// and because F >= 2 bs the circular correlation never wraps on the kept lags, so in the time
// domain it is the direct correlation of the double block u_g (2 bs samples) with the code block:
//   T[g, r bs + j] = sum_{b < bs} c_m[b] u_g[j + b].
// For one row g and all requested PRNs this is the real GEMM
//   D[j, (PRN, m)] = sum_b H_g[j, b] C[(PRN, m), b],   H_g[j, b] = u_g[j + b],  C = code samples,
// once for Re u_g and once for Im u_g. Code samples are small integers (exact in FP16); u_g is
// scaled by a power of two per row and split into FP16 hi + lo (hi + lo = u_g to 22 significant
// bits), so D = A (B_hi + B_lo) is the FP32-accumulated correlation to FP32-class accuracy.
//
// H_g is a Hankel matrix. In the K-major no-swizzle operand layout (8-row x 16-byte core
// matrices) its core matrix at (row block c, K block a) is Q_{a+c}, Q_s[d][e] = u_g[8 s + d + e],
// so one copy of the Q_s per row (8 x the samples instead of bs x) with a descriptor whose
// leading and stride byte offsets are both 128 presents the whole matrix to the MMA.
//
// k_tile_stubs builds, per (step, row), the Q_s of the four operands (Re hi, Re lo, Im hi, Im lo)
// from the input samples (IF wipe-off as k_frontend) after the first Doppler pass (the direct
// n_coh-point DFT of k_doppler_prepass, applied to the time-domain blocks: the map is linear and
// acts on rows only). k_tile_mma keeps one 128-row block of code rows resident per CTA and loops
// over rows g: a bulk copy brings the row's Q_s, one thread issues the MMAs into tensor memory,
// and the drain warps move D (times the row's inverse scale) to the tile with tcgen05.ld.
#pragma once

#include "acq_mma.cuh"

namespace acq {

constexpr int kTmmaRows = 128;      // code rows (PRN, block) per CTA: the MMA's M
constexpr int kTmmaDrainWarps = 16;
constexpr int kTmmaThreads = 32 * kTmmaDrainWarps + 64;   // drain warps, the issuing warp, the copy warp
// code rows one drain warp moves per lag half: the warps of a TMEM lane quarter split the 128
constexpr int kTmmaDrainRows = 4 * 128 / kTmmaDrainWarps;
static_assert(kTmmaDrainRows == 32 || kTmmaDrainRows == 64, "32 or 64 code rows per drain warp");
constexpr int kTmmaStubThreads = 256;

// geometry of the operands for a block size bs <= 256
__host__ __device__ constexpr int tmma_ks(int bs) { return (bs + 15) / 16; }     // K steps of 16
__host__ __device__ constexpr int tmma_nh(int bs) { return (bs + 127) / 128; }   // lag halves of 128 (MMA N)
__host__ __device__ constexpr int tmma_stubs(int bs) { return 2 * tmma_ks(bs) + 16 * tmma_nh(bs) - 1; }
__host__ __device__ constexpr int tmma_span(int bs) { return 8 * tmma_stubs(bs) + 8; }   // samples the Q_s read
__host__ __device__ constexpr int tmma_row_bytes(int bs) { return 4 * tmma_stubs(bs) * 128; }
__host__ __device__ constexpr int tmma_a_bytes(int bs) { return kTmmaRows * tmma_ks(bs) * 32; }
constexpr int kTmmaMaxBs = 256;
constexpr int kTmmaMaxSpan = tmma_span(kTmmaMaxBs);

// Per (step, row): the time-domain row after the first Doppler pass, its power-of-two scale and
// the Q_s of its four FP16 operands. Grid (G, n_nc), kTmmaStubThreads threads.
//   pre = 1: row k + nb k1 = W_ndop^{k k1} sum_q W_{n_coh}^{q k1} u_{k + nb q}   (k1 < n_coh)
//   pre = 0: row g = u_g
// u_g[t] = input[(g bs + t) mod seg_len] for t < 2 bs (IF wiped off as k_frontend), 0 beyond.
// The accumulator cells the Doppler-group column stage adds into atomically (H columns on each
// side of every column-block boundary), zeroed by this kernel's threads after the operand blocks
// when acc is set (the column stage runs after the tile, which runs after this kernel).
struct EdgeZero {
    float* acc;
    int64_t rows;
    int spc, spc_eff, W, H, n_bound;
};

__global__ void __launch_bounds__(kTmmaStubThreads) k_tile_stubs(const void* __restrict__ in, int dtype,
                                                                 int64_t seg_len, int G, int nb, int n_coh, int bs,
                                                                 int pre, int use_if, float if_step,
                                                                 const float* __restrict__ if_offset,
                                                                 const float2* __restrict__ twD,
                                                                 uint8_t* __restrict__ stubs,
                                                                 float* __restrict__ inv_scale, EdgeZero ez) {
    __shared__ __align__(16) uint16_t xh[4][kTmmaMaxSpan];
    __shared__ float red[kTmmaStubThreads / 32];
    pdl_trigger();
    const int rho = blockIdx.x, step = blockIdx.y;
    const int tid = threadIdx.x;
    const int64_t seg0 = static_cast<int64_t>(step) * seg_len;
    const float off = use_if ? if_offset[step] : 0.f;
    const int k = rho % nb, k1 = rho / nb;
    const int span = tmma_span(bs);
    // g < G and t < 2 bs, so g bs + t < seg_len + bs: one subtraction wraps it
    auto sample = [&](int g, int t) -> float2 {
        int64_t pos = static_cast<int64_t>(g) * bs + t;
        if (pos >= seg_len) pos -= seg_len;
        float2 v = load_sample(in, dtype, seg0 + pos);
        if (use_if) {
            const float ph = __fadd_rn(off, __fmul_rn(__ll2float_rn(pos), if_step));
            float s, c;
            sincosf(ph, &s, &c);
            v = make_float2(__fsub_rn(__fmul_rn(v.x, c), __fmul_rn(v.y, s)),
                            __fadd_rn(__fmul_rn(v.x, s), __fmul_rn(v.y, c)));
        }
        return v;
    };
    constexpr int kPer = (kTmmaMaxSpan + kTmmaStubThreads - 1) / kTmmaStubThreads;
    float2 x[kPer];
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int t = tid + i * kTmmaStubThreads;
        float2 acc = make_float2(0.f, 0.f);
        if (t < 2 * bs) {
            if (pre && n_coh > 1) {
                acc = sample(k, t);
                int e = 0;   // (q k1) mod n_coh
                for (int q = 1; q < n_coh; ++q) {
                    e += k1;
                    if (e >= n_coh) e -= n_coh;
                    const float2 v = sample(k + nb * q, t);
                    acc = c_add(acc, e ? c_mul(v, __ldg(twD + e * nb)) : v);
                }
                if (k * k1) acc = c_mul(acc, __ldg(twD + k * k1));
            } else {
                acc = sample(rho, t);
            }
        }
        x[i] = acc;
        mx = fmaxf(mx, fmaxf(fabsf(acc.x), fabsf(acc.y)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    mx = 0.f;
#pragma unroll
    for (int w = 0; w < kTmmaStubThreads / 32; ++w) mx = fmaxf(mx, red[w]);
    // |u s| < 2^15: hi stays inside FP16's range; lo = u s - hi carries the next 11 bits
    int ex = 0;
    if (mx > 0.f) frexpf(mx, &ex);
    ex = max(-100, min(100, ex));
    const float s = ldexpf(1.f, 15 - ex);
    if (tid == 0) ACQ_BC(&inv_scale[static_cast<int64_t>(step) * G + rho], 3)
        inv_scale[static_cast<int64_t>(step) * G + rho] = ldexpf(1.f, ex - 15);
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int t = tid + i * kTmmaStubThreads;
        if (t < span) {
            const float re = x[i].x * s, im = x[i].y * s;
            const __half rh = __float2half_rn(re), ih = __float2half_rn(im);
            xh[0][t] = __half_as_ushort(rh);
            xh[1][t] = __half_as_ushort(__float2half_rn(re - __half2float(rh)));
            xh[2][t] = __half_as_ushort(ih);
            xh[3][t] = __half_as_ushort(__float2half_rn(im - __half2float(ih)));
        }
    }
    __syncthreads();
    // Q_s rows: 16 bytes = 8 consecutive samples from 8 s + d, rows of all operands contiguous
    const int nst = tmma_stubs(bs);
    const int n_rows = 4 * nst * 8;
    uint4* out = reinterpret_cast<uint4*>(stubs + (static_cast<int64_t>(step) * G + rho) * tmma_row_bytes(bs));
    for (int idx = tid; idx < n_rows; idx += kTmmaStubThreads) {
        const int v = idx / (nst * 8);
        const int rem = idx - v * nst * 8;
        const int base = (rem >> 3) * 8 + (rem & 7);
        const uint16_t* src = xh[v] + base;
        uint4 w;
        w.x = static_cast<uint32_t>(src[0]) | (static_cast<uint32_t>(src[1]) << 16);
        w.y = static_cast<uint32_t>(src[2]) | (static_cast<uint32_t>(src[3]) << 16);
        w.z = static_cast<uint32_t>(src[4]) | (static_cast<uint32_t>(src[5]) << 16);
        w.w = static_cast<uint32_t>(src[6]) | (static_cast<uint32_t>(src[7]) << 16);
        ACQ_BC(&out[idx], 2) out[idx] = w;
    }
    if (ez.acc) {
        const int per_row = ez.n_bound * 2 * ez.H;
        const int64_t total = ez.rows * per_row;
        const int64_t nthr = static_cast<int64_t>(gridDim.x) * gridDim.y * blockDim.x;
        const bool narrow = total < (int64_t{1} << 31);   // 32-bit index arithmetic
        for (int64_t q = (static_cast<int64_t>(blockIdx.y) * gridDim.x + blockIdx.x) * blockDim.x + tid; q < total;
             q += nthr) {
            const int64_t r = narrow ? static_cast<int>(q) / per_row : q / per_row;
            const int e = static_cast<int>(q - r * per_row);
            const int jb = e / (2 * ez.H), o = e - jb * 2 * ez.H - ez.H;   // boundary jb, offset in [-H, H)
            const int b0 = jb == ez.n_bound - 1 ? ez.spc : jb * ez.W;
            int c = b0 + o;
            if (c < 0) c += ez.spc;
            if (c >= ez.spc) c -= ez.spc;
            ACQ_BC(&ez.acc[r * ez.spc_eff + c], 23) ez.acc[r * ez.spc_eff + c] = 0.f;
        }
    }
}

struct TileMmaParams {
    const uint8_t* stubs;      // (n_nc * G) rows of tmma_row_bytes(bs)
    const float* inv_scale;    // (n_nc * G)
    const int8_t* codes;       // (slots, spc)
    const int* slots;          // requested PRN -> code slot
    float2* T;                 // tile of all steps: [step][PRN][g][spc]
    int64_t t_step_stride;
    int n, G, nb, bs, spc;
    int n_chunks;              // ceil(n nb / 128) blocks of code rows
    int units;                 // n_nc * G rows
    int cpc;                   // CTAs per block of code rows
    int* err;
};

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// shared-memory bytes of k_tile_mma for a block size (plus 1 KB alignment slack)
__host__ __device__ constexpr int tmma_smem_bytes(int bs) {
    return 1024 + tmma_a_bytes(bs) + 2 * tmma_row_bytes(bs) + kTmmaRows * 12 + 128;
}

// Bounded mbarrier wait that also gives up when another warp has recorded an error (polled
// every 256 tries); on its own timeout it records error 6 and raises the block's abort flag.
__device__ __forceinline__ bool tmma_wait(uint64_t* bar, uint32_t parity, int* err, volatile int* abort_flag) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255u) == 255u && *abort_flag) return false;
    }
    atomicExch(err, 6);
    *abort_flag = 1;
    return false;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// GEMM roles: A = the row's Hankel operand (M = 128 lags of one half), B = the code rows
// (N = 128 (PRN, block) rows), so a tensor-memory lane holds one lag and its columns the code rows:
// a warp's tcgen05.ld gives 32 consecutive lags of 8 code rows, stored as 256 contiguous bytes
// per code row. Tensor memory: lag half h of Re D at columns 256 h .. + 127, of Im D at
// 256 h + 128 .. + 255.
// Warp roles: warp kTmmaDrainWarps + 1 (one elected thread) issues the bulk copies of the Q_s (two
// buffers), warp kTmmaDrainWarps (one elected thread) the MMAs, warps 0 .. kTmmaDrainWarps - 1
// move D to the tile. mbarriers:
//   sbar[b]   Q_s of buffer b landed (bulk-copy transaction count)
//   full[h]   MMAs of lag half h done (tcgen05.commit)
//   empty[h]  half h drained (one arrival per drain warp)
//   sfree[b]  MMAs reading buffer b done (tcgen05.commit), so the next copy may overwrite it
// Each barrier completes once per unit (per use of its buffer for sbar / sfree), and no wait can
// see two completions ahead, so every parity wait is unambiguous.
__global__ void __launch_bounds__(kTmmaThreads, 1) k_tile_mma(TileMmaParams p) {
    extern __shared__ uint8_t smraw_[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw_) + 1023) & ~uintptr_t(1023));
    const int KS = tmma_ks(p.bs), NH = tmma_nh(p.bs), NST = tmma_stubs(p.bs);
    const int KCH = 2 * KS;
    const uint32_t row_bytes = static_cast<uint32_t>(tmma_row_bytes(p.bs));
    uint8_t* Bc = sm;                                   // code rows, K-major
    uint8_t* stub0 = sm + tmma_a_bytes(p.bs);           // two Q_s buffers
    int64_t* col_off = reinterpret_cast<int64_t*>(stub0 + 2 * row_bytes);   // PRN row offset, -1: none
    int* col_m = reinterpret_cast<int*>(col_off + kTmmaRows);               // code block
    uint64_t* bars = reinterpret_cast<uint64_t*>(col_m + kTmmaRows);
    uint64_t* sbar = bars;        // [2]
    uint64_t* full = bars + 2;    // [2]
    uint64_t* empty = bars + 4;   // [2]
    uint64_t* sfree = bars + 6;   // [2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 8);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 9);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int chunk = blockIdx.x % p.n_chunks;
    const int q = blockIdx.x / p.n_chunks;
    const int u0 = static_cast<int>(static_cast<int64_t>(q) * p.units / p.cpc);
    const int u1 = static_cast<int>(static_cast<int64_t>(q + 1) * p.units / p.cpc);
    const int nu = u1 - u0;
    const uint32_t tcols = NH == 2 ? 512u : 256u;

    if (tid == 0) {
        for (int i = 0; i < 8; ++i) mbar_init(&bars[i], (i == 4 || i == 5) ? kTmmaDrainWarps : 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) tc_alloc(tslot, tcols);
    // B: code rows of this block, K-major, samples b >= bs zero (consecutive threads take
    // consecutive rows: eight 16-byte rows of a core matrix fill all banks)
    for (int i = tid; i < kTmmaRows * KCH; i += kTmmaThreads) {
        const int row = i % kTmmaRows, kc = i / kTmmaRows;
        const int gr = chunk * kTmmaRows + row;
        const int pi = gr / p.nb, m = gr - pi * p.nb;
        uint32_t w[4] = {0u, 0u, 0u, 0u};
        if (pi < p.n) {
            const int8_t* c = p.codes + static_cast<int64_t>(p.slots[pi]) * p.spc + static_cast<int64_t>(m) * p.bs;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int b = kc * 8 + e;
                uint32_t h = 0u;
                if (b < p.bs) ACQ_BC(&c[b], 5) h = __half_as_ushort(__int2half_rn(c[b]));
                w[e >> 1] |= h << ((e & 1) * 16);
            }
        }
        *reinterpret_cast<uint4*>(Bc + (row >> 3) * (KCH * 128) + kc * 128 + (row & 7) * 16) =
            make_uint4(w[0], w[1], w[2], w[3]);
    }
    if (tid < kTmmaRows) {
        const int gr = chunk * kTmmaRows + tid;
        const int pi = gr / p.nb;
        col_off[tid] = pi < p.n ? static_cast<int64_t>(pi) * p.G * p.spc : -1;
        col_m[tid] = gr - pi * p.nb;
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    pdl_wait();   // the operand blocks and their scales (code rows and slots are already in place)

    if (warp == kTmmaDrainWarps + 1) {
        // copy warp: unit u's operand blocks into buffer u & 1 as soon as the MMAs of unit u - 2
        // are done with it (one unit ahead of the MMAs)
        if (lane == 0) {
            uint32_t n_s[2] = {0u, 0u};   // copies issued per buffer, for the bounded drain on an error
            bool ok = true;
            for (int u = 0; u < nu; ++u) {
                const int b = u & 1;
                if (u >= 2 && !(ok = tmma_wait(&sfree[b], ((u - 2) >> 1) & 1, p.err, abort_flag))) break;
                ++n_s[b];
#ifdef ACQ_BOUNDS_CHECK
                if (!bc_ok(p.stubs + static_cast<int64_t>(u0 + u) * row_bytes, row_bytes, 4)) {
                    mbar_expect_tx(&sbar[b], 0u);   // completes the phase without a copy
                    continue;
                }
#endif
                mbar_expect_tx(&sbar[b], row_bytes);
                bulk_load(stub0 + b * row_bytes, p.stubs + static_cast<int64_t>(u0 + u) * row_bytes, row_bytes,
                          &sbar[b]);
            }
            if (!ok) {   // let every copy in flight land before the block's memory is released
                for (int i = 0; i < 2; ++i)
                    if (n_s[i]) mbar_wait_bounded(&sbar[i], (n_s[i] - 1) & 1, p.err, 6, 1u << 20);
            }
        }
    } else if (warp == kTmmaDrainWarps) {
        // issuing thread: per unit, wait for its operand blocks, then per lag half wait until the
        // drain has emptied that half, issue its MMAs and commit them to full[h]; sfree[b] tells
        // the copy warp when buffer b may be overwritten
        if (lane == 0) {
            // completions asked of each barrier, for the bounded drain on an error
            uint32_t n_full[2] = {0u, 0u}, n_free[2] = {0u, 0u};
            const uint32_t idesc = tc_idesc_f16(0, 128, kTmmaRows);
            // descriptors differ only in the start-address field (byte address / 16, < 2^14)
            const uint64_t a0 = tc_desc(stub0, 128, 128);
            const uint64_t b0 = tc_desc(Bc, 128, KCH * 128);
            bool ok = true;
            for (int u = 0; u < nu && ok; ++u) {
                const int b = u & 1;
                if (!(ok = tmma_wait(&sbar[b], (u >> 1) & 1, p.err, abort_flag))) break;
                for (int h = 0; h < NH && ok; ++h) {
                    if (!(ok = tmma_wait(&empty[h], (u & 1) ^ 1, p.err, abort_flag))) break;
                    tc_fence_after();
#pragma unroll 1
                    for (int c = 0; c < 2; ++c) {
                        const uint32_t d = tmem + h * 256 + c * 128;
#pragma unroll 1
                        for (int ks = 0; ks < KS; ++ks) {
                            const uint64_t bd = b0 + static_cast<uint64_t>(ks * 16);
                            const uint32_t aoff = (b * row_bytes + (2 * c) * NST * 128 + 128 * (16 * h + 2 * ks)) >> 4;
                            tc_mma_f16(d, a0 + aoff, bd, idesc, ks > 0);
                            tc_mma_f16(d, a0 + aoff + (NST * 128 >> 4), bd, idesc, true);
                        }
                    }
                    tc_commit(&full[h]);
                    ++n_full[h];
                }
                if (!ok) break;
                tc_commit(&sfree[b]);
                ++n_free[b];
            }
            if (!ok) {
                // let every MMA still in flight land before the block's memory is released
                for (int i = 0; i < 2; ++i) {
                    if (n_full[i]) mbar_wait_bounded(&full[i], (n_full[i] - 1) & 1, p.err, 6, 1u << 20);
                    if (n_free[i]) mbar_wait_bounded(&sfree[i], (n_free[i] - 1) & 1, p.err, 6, 1u << 20);
                }
            }
        }
    } else {
        // drain warps: warp w reads lags 128 h + 32 (w % 4) + lane (its TMEM lane quarter) and code
        // rows R (w / 4) .. + R - 1, R = kTmmaDrainRows; lane l holds the tile offsets of code rows
        // R (w / 4) + l (and + 32 + l when R = 64) for the current unit.
        // The next 16 columns' tcgen05.ld is in flight while the current ones are stored; the
        // stores stream (evict-first): the tile is read once, by the Doppler stage, much later.
        const int sp = warp & 3, cbase = (warp >> 2) * kTmmaDrainRows;
        const int64_t my_off = col_off[cbase + lane];
        const int64_t my_off2 = kTmmaDrainRows == 64 ? col_off[cbase + 32 + lane] : -1;
        const int my_m = col_m[cbase + lane], my_m2 = kTmmaDrainRows == 64 ? col_m[cbase + 32 + lane] : 0;
        for (int u = 0; u < nu; ++u) {
            const int gu = u0 + u;
            const int step = gu / p.G, rho = gu - (gu / p.G) * p.G;
            int r = my_m - rho % p.nb;
            if (r < 0) r += p.nb;
            int r2 = my_m2 - rho % p.nb;
            if (r2 < 0) r2 += p.nb;
            // cell offsets within the step (the host keeps a step's tile under 2^31 cells), shuffled
            // as one 32-bit value per code row; the step's base is added once
            const int64_t sbase = step * p.t_step_stride;
            const int rowb = rho * p.spc;
            const int off_l = my_off < 0 ? -1 : rowb + static_cast<int>(my_off) + r * p.bs;
            const int off_l2 = my_off2 < 0 ? -1 : rowb + static_cast<int>(my_off2) + r2 * p.bs;
            const float isc = p.inv_scale[gu];
            bool ok = true;
            for (int h = 0; h < NH; ++h) {
                if (!(ok = tmma_wait(&full[h], u & 1, p.err, abort_flag))) break;
                tc_fence_after();
                const int j = h * 128 + sp * 32 + lane;
                const bool jok = j < p.bs;
                float2* base = p.T + sbase + j;
                const uint32_t tb = tmem + (static_cast<uint32_t>(sp * 32) << 16) + h * 256 + cbase;
                float re[2][16], im[2][16];
                tc_ld8(tb + 0, re[0]);
                tc_ld8(tb + 8, re[0] + 8);
                tc_ld8(tb + 128, im[0]);
                tc_ld8(tb + 128 + 8, im[0] + 8);
                tc_wait_ld();
#pragma unroll
                for (int i = 0; i < kTmmaDrainRows; i += 16) {
                    const int cb = (i >> 4) & 1;
                    if (i + 16 < kTmmaDrainRows) {
                        tc_ld8(tb + i + 16, re[cb ^ 1]);
                        tc_ld8(tb + i + 24, re[cb ^ 1] + 8);
                        tc_ld8(tb + 128 + i + 16, im[cb ^ 1]);
                        tc_ld8(tb + 128 + i + 24, im[cb ^ 1] + 8);
                    }
                    const int ol = i < 32 ? off_l : off_l2;
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        const int off = __shfl_sync(0xffffffffu, ol, (i & 31) + e);
                        if (off >= 0 && jok)
                            ACQ_BC(base + off, 6) __stcs(base + off, make_float2(re[cb][e] * isc, im[cb][e] * isc));
                    }
                    tc_wait_ld();
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[h]);
            }
            if (!ok) break;
        }
    }
    // the next kernel's blocks may be scheduled once every block here has finished its work (an
    // earlier trigger would let them take shared memory beside blocks that still drain)
    pdl_trigger();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tc_dealloc(tmem, tcols);
    }
}

}  // namespace acq
