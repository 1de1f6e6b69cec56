// acq_mma.cuh — secondary-code rotation search with the candidate combine on the 5th-generation
// tensor cores (tcgen05.mma, FP16 or BF16 operands, FP32 accumulation in tensor memory).
//
// The rotation search (src/noncoherent_integration.jl:183-297) transforms, for every code-phase
// column and every candidate q = (rotation, data-bit combination), the alignment-rotated column
// weighted per sub-block by the candidate's +-1 pattern s_q[p] (src/sign_patterns.jl:23-47,
// 80-129). Split the ndop-point transform as ndop = NC x NB (NC sub-blocks of NB rows):
//   X_q[k1 + NC k2] = sum_p s_q[p] G_p[k1, k2],
//   G_p[k1, k2]     = FFT_NB over n2 of  x[(base + n2 + NB p) mod ndop] w_ndop^((n2 + NB p) k1),
// i.e. the sub-block spectra G (candidate-independent, FP32 FFTs on the CUDA cores) times the
// pattern matrix (exact in FP16/BF16). Per k1 the combine is one GEMM
//   D[m = (k2, column), n = (re|im, q)] = sum_k A[m, k = (p, re|im)] B[n, k]
// with B[q, 2p] = B[Qp + q, 2p + 1] = s_q[p] and zeros elsewhere, so that one tensor-memory lane
// holds Re and Im of X_q for one output bin. A is G rounded to FP16/BF16 (one operand) or split
// into hi + lo = G exactly to 2 x 11 (FP16) or 2 x 8 (BF16) significant bits (two MMAs into the
// same accumulator). The epilogue reads D with tcgen05.ld, forms |X_q|^2, keeps the max over data
// combinations per rotation (strict '>', earlier candidate wins) and scatters like the FP32 path.
//
// Operand layout in shared memory: K-major, no swizzle, 8-row x 16-byte core matrices;
// adjacent core matrices along K are 128 B apart (leading byte offset), along M/N KCH x 128 B
// apart (stride byte offset). Waits on the MMA-completion mbarrier are bounded; on timeout the
// block records an error, waits (bounded) again, frees its tensor memory and returns.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "acq_kernels_fs.cuh"

namespace acq {

constexpr int kRotMmaW = 8;   // code-phase columns per block

struct RotMmaParams {
    const float2* T;
    int spc, spc_eff, bs, R, combos, use_max, first;
    const float2* twD;
    const float* pats;
    const int* slots;
    const int* drift;
    float* acc;
    uint16_t* win;
    float scale;      // power of two applied to G before rounding (FP16 range)
    int* err;
};

// ---- tcgen05 helpers (PTX ISA, sm_100a family) ----
__device__ __forceinline__ void tc_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: start, leading byte offset (K direction), stride byte offset
// (M/N direction), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(const void* p, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = (smem_u32(p) >> 4) & 0x3FFFull;
    return a | (static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16) | (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, A/B format (0 FP16, 1 BF16), K-major
// A and B, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t tc_idesc_f16(int fmt, int m, int n) {
    return (1u << 4) | (static_cast<uint32_t>(fmt) << 7) | (static_cast<uint32_t>(fmt) << 10) |
           (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                           bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 32 lanes x 8 consecutive 32-bit columns
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__host__ __device__ constexpr int tc_tmem_cols(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512; }

template <int FMT>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    if (FMT == 0) {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
template <int FMT>
__device__ __forceinline__ float2 unpack2(uint32_t u) {
    if (FMT == 0) return __half22float2(*reinterpret_cast<const __half2*>(&u));
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u));
}
template <int FMT>
__device__ __forceinline__ uint16_t to16(float a) {
    if (FMT == 0) return __half_as_ushort(__float2half_rn(a));
    return __bfloat16_as_ushort(__float2bfloat16_rn(a));
}

// byte offset of element (row, k) of a K-major no-swizzle operand with KCH 16-byte chunks per row
template <int KCH>
__device__ __forceinline__ int op_offset(int row, int k) {
    return (row >> 3) * (KCH * 128) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

template <int NC, int NB, int QP>
struct RotMmaShape {
    static constexpr int W = kRotMmaW;
    static constexpr int ND = NC * NB;
    static constexpr int KP = (2 * NC + 15) / 16 * 16;     // K: (p, re|im), padded to MMA K steps
    static constexpr int KCH = KP / 8;
    static constexpr int N = 2 * QP;                        // re outputs then im outputs
    static constexpr int MROWS = NB * W;                    // (k2, column) rows per k1
    static constexpr int MT = (MROWS + 127) / 128;
    static constexpr int TILE_BYTES = 16 * KCH * 128;       // 128 rows
    static constexpr int B_BYTES = (N / 8) * KCH * 128;
    static constexpr int TCOLS = tc_tmem_cols(MT * 64);     // one 64-column slot per M tile
    __host__ __device__ static constexpr int off_b(int nsplit) { return nsplit * MT * TILE_BYTES; }
    __host__ __device__ static constexpr int off_tile(int nsplit) { return off_b(nsplit) + B_BYTES; }
    __host__ __device__ static constexpr int off_tws(int nsplit) { return off_tile(nsplit) + ND * W * 8; }
    __host__ __device__ static constexpr int off_cro(int nsplit) { return off_tws(nsplit) + ND * 8; }
    __host__ __device__ static constexpr int off_psm(int nsplit) { return off_cro(nsplit) + W * 4; }
    __host__ __device__ static constexpr int off_bar(int nsplit) { return (off_psm(nsplit) + 32 * NC * 4 + 15) / 16 * 16; }
    __host__ __device__ static constexpr int smem_bytes(int nsplit) { return off_bar(nsplit) + 16 + 1024; }   // + alignment slack
};

template <int NC, int NB, int QP, int CB, int FMT, int NSPLIT>
__global__ void __launch_bounds__(256, 2) k_rot_mma(RotMmaParams p) {
    static_assert(CB == 1 || CB == 2 || CB == 4 || CB == 8, "data-bit combinations per rotation");
    using S = RotMmaShape<NC, NB, QP>;
    constexpr int W = S::W, ND = S::ND, KCH = S::KCH, MT = S::MT;
    extern __shared__ uint8_t smraw_[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw_) + 1023) & ~uintptr_t(1023));
    uint8_t* A = sm;
    uint8_t* Bm = sm + S::off_b(NSPLIT);
    float2* tile = reinterpret_cast<float2*>(sm + S::off_tile(NSPLIT));
    float2* tws = reinterpret_cast<float2*>(sm + S::off_tws(NSPLIT));
    int* cro = reinterpret_cast<int*>(sm + S::off_cro(NSPLIT));
    float* psm = reinterpret_cast<float*>(sm + S::off_psm(NSPLIT));
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S::off_bar(NSPLIT));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int pi = blockIdx.y;
    const int slot = p.slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, p.spc - c0);
    const int n_pat = p.R * p.combos;

    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) tc_alloc(tslot, S::TCOLS);
    // operands: zero (padding rows / K stay zero), then the pattern matrix B
    {
        int4* a4 = reinterpret_cast<int4*>(A);
        const int n16 = (S::off_tile(NSPLIT)) / 16;
        for (int i = tid; i < n16; i += blockDim.x) a4[i] = make_int4(0, 0, 0, 0);
    }
    const float2* tp = p.T + static_cast<int64_t>(pi) * ND * p.spc;
    for (int w = tid; w < ND * W; w += blockDim.x) {
        const int e = w / W, t = w - (w / W) * W;
        float2 v = make_float2(0.f, 0.f);
        if (t < wv) ACQ_BC(&tp[static_cast<int64_t>(e) * p.spc + c0 + t], 50) v = tp[static_cast<int64_t>(e) * p.spc + c0 + t];
        tile[w] = v;
    }
    for (int i = tid; i < ND; i += blockDim.x) tws[i] = p.twD[i];
    if (tid < W) {
        const int pc = c0 + tid;
        const int wrap = ((NB - pc / p.bs) % NB) * p.bs + pc % p.bs;   // src/noncoherent_integration.jl:212-214
        cro[tid] = ((wrap + (p.bs >> 1)) / p.bs) % NB;
    }
    const float* pp = p.pats + static_cast<int64_t>(slot) * n_pat * NC;
    for (int i = tid; i < n_pat * NC; i += blockDim.x) psm[i] = pp[i];
    __syncthreads();
    for (int i = tid; i < S::N * NC; i += blockDim.x) {
        const int n = i / NC, pq = i - (i / NC) * NC;
        const int q = n < QP ? n : n - QP, c = n < QP ? 0 : 1;
        const float v = q < n_pat ? psm[q * NC + pq] : 0.f;
        *reinterpret_cast<uint16_t*>(Bm + op_offset<KCH>(n, 2 * pq + c)) = to16<FMT>(v);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    // phase-A role: sub-block pa of column ta (rows base .. base + NB - 1, cyclic)
    const bool has_a = tid < NC * W;
    const int pa = tid / W, ta = tid - (tid / W) * W;
    const int abase = has_a ? cro[ta] + NB * pa : 0;
    const uint32_t idesc = tc_idesc_f16(FMT, 128, S::N);
    const float inv_s2 = 1.0f / (p.scale * p.scale);
    float* ap = p.acc + static_cast<int64_t>(pi) * ND * p.spc_eff;
    uint16_t* wp = p.win + static_cast<int64_t>(pi) * ND * p.spc_eff;
    uint32_t phase = 0;
    bool ok = true;
    for (int k1 = 0; k1 < NC && ok; ++k1) {
        if (has_a) {
            // w_ND^((n2 + NB pa) k1), index reduced mod ND incrementally
            int ti = (NB * pa * k1) % ND;
            float2 v[NB];
#pragma unroll
            for (int n2 = 0; n2 < NB; ++n2) {
                const int row = abase + n2 >= ND ? abase + n2 - ND : abase + n2;
                v[n2] = c_mul(tile[row * W + ta], tws[ti]);
                ti += k1;
                ti = ti >= ND ? ti - ND : ti;
            }
            RegFFT<NB, false>::run(v);
            static_for<0, NB>([&](auto kc) {
                constexpr int k2 = decltype(kc)::value;
                const float2 g = v[reg_perm(NB, k2)];
                const float gr = g.x * p.scale, gi = g.y * p.scale;
                const int m = k2 * W + ta;
                const int off = (m >> 7) * S::TILE_BYTES + op_offset<KCH>(m & 127, 2 * pa);
                const uint32_t hi = pack2<FMT>(gr, gi);
                *reinterpret_cast<uint32_t*>(A + off) = hi;
                if (NSPLIT == 2) {
                    const float2 h = unpack2<FMT>(hi);
                    *reinterpret_cast<uint32_t*>(A + MT * S::TILE_BYTES + off) = pack2<FMT>(gr - h.x, gi - h.y);
                }
            });
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
#pragma unroll
                for (int s = 0; s < NSPLIT; ++s)
#pragma unroll
                    for (int ks = 0; ks < S::KP / 16; ++ks) {
                        const uint64_t ad = tc_desc(A + (s * MT + mt) * S::TILE_BYTES + ks * 256, 128, KCH * 128);
                        const uint64_t bd = tc_desc(Bm + ks * 256, 128, KCH * 128);
                        tc_mma_f16(tmem + mt * 64, ad, bd, idesc, s > 0 || ks > 0);
                    }
            tc_commit(bar);
        }
        const bool mine = mbar_wait_bounded(bar, phase, p.err, 3);
        phase ^= 1;
        ok = __syncthreads_or(mine ? 0 : 1) == 0;   // one decision for the whole block
        tc_fence_after();
        if (ok) {
            // epilogue: warp w reads lanes 32 (w % 4) .. of M tiles w / 4, w / 4 + 2, ...
            const int sp = warp & 3;
            for (int mt = warp >> 2; mt < MT; mt += 2) {
                const int m = mt * 128 + sp * 32 + lane;
                const bool valid = m < S::MROWS && (m % W) < wv;
                const int k2 = m / W, t = m % W;
                const int om = k1 + NC * k2;
                const int row = om < ND / 2 ? om + ND / 2 : om - ND / 2;
                int dc = 0;
                if (valid) {
                    dc = c0 + t + p.drift[row];
                    dc = dc >= p.spc ? dc - p.spc : dc;
                }
                const uint32_t tb = tmem + (static_cast<uint32_t>(sp * 32) << 16) + mt * 64;
                const int64_t rbase = static_cast<int64_t>(row) * p.spc_eff + dc;
                float best = 0.f;
                int bw = 0;
#pragma unroll
                for (int j = 0; j < QP / 8; ++j) {
                    float re[8], im[8];
                    tc_ld8(tb + 8 * j, re);
                    tc_ld8(tb + QP + 8 * j, im);
                    tc_wait_ld();
                    // max over each group of CB data-bit combinations (CB divides 8)
                    float bestv[8];
                    int bwv[8];
                    bool keep[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int q = 8 * j + i;
                        const int d = q & (CB - 1);
                        const float pw = __fadd_rn(__fmul_rn(re[i], re[i]), __fmul_rn(im[i], im[i])) * inv_s2;
                        if (d == 0) {
                            best = 0.f;
                            bw = 0;
                        }
                        if (!p.use_max || pw > best) {
                            best = pw;
                            bw = d;
                        }
                        bestv[i] = best;
                        bwv[i] = bw;
                        keep[i] = valid && d == CB - 1 && q / CB < p.R;
                    }
                    // accumulator read-modify-write: the chunk's loads first, then its stores
                    float old[8];
                    if (!(p.first & 1)) {
#pragma unroll
                        for (int i = 0; i < 8; ++i)
                            old[i] = keep[i] ? ap[rbase + ((8 * j + i) / CB) * p.spc] : 0.f;
                    }
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        if (keep[i]) {
                            const int64_t idx = rbase + ((8 * j + i) / CB) * p.spc;
                            ap[idx] = (p.first & 1) ? bestv[i] : old[i] + bestv[i];
                            if (p.first & 2) wp[idx] = static_cast<uint16_t>(bwv[i]);
                        }
                    }
                }
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    if (!ok) mbar_wait_bounded(bar, phase ^ 1, p.err, 4);   // let an MMA still in flight finish
    tc_fence_after();
    if (warp == 0) tc_dealloc(tmem, S::TCOLS);
}

}  // namespace acq

namespace acq {

// ------------------------------------------------------------------ Doppler DFT as a GEMM
// Simple-path column stage (src/acquire.jl:335-385, src/noncoherent_integration.jl:482-592)
// with the ndop-point Doppler DFT of every code column as one dense complex DFT-matrix GEMM on
// the tensor cores: for a block of 128 code columns,
//   D[m = column, n = (k, re|im)] = sum_{kk = (g, re|im)} A[m, kk] B[n, kk],
// A = the coherent tile (FP16/BF16, one operand or hi + lo), B = the real form of
// exp(-2 pi i g k / ndop) (hi + lo in the split variants: A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32
// accumulation in TMEM). The K dimension streams through shared memory in steps of 8 rows
// (16 real K): the block converts its tile rows while the tensor core works on the previous
// step (two buffers, one mbarrier each); the DFT-matrix chunks come from global memory by
// 16-byte cp.async. Epilogue: |X|^2, fftshift, destination-row drift, accumulation (loads of a
// batch before its stores). ndop <= 256 (TMEM: 2 ndop <= 512 FP32 columns).
constexpr int kDftCols = 128;       // code columns per block (MMA M)
constexpr int kDftThreads = 256;

struct DftMmaParams {
    const float2* T;                // (n, ndop, spc) coherent tile of one step
    int spc, nd, spc_eff, n_pad, ksteps, first, has_drift;
    const int* drift;               // (ndop) destination-row shifts
    float* acc;
    const uint8_t* B;               // [split][ksteps][n_pad x 16] canonical K-major chunks
    float scale;                    // power of two applied to the tile before rounding
    int* err;
};

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit_all() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_zero() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int FMT, int NSPLIT>
__global__ void __launch_bounds__(kDftThreads, 1) k_col_dft_mma(DftMmaParams p) {
    constexpr int A_BYTES = kDftCols * 32;   // 128 rows x 16 K x 2 B
    extern __shared__ uint8_t smraw_[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw_) + 1023) & ~uintptr_t(1023));
    const int b_bytes = p.n_pad * 32;
    uint8_t* Abuf = sm;                                        // [2][NSPLIT][A_BYTES]
    uint8_t* Bbuf = sm + 2 * NSPLIT * A_BYTES;                 // [2][NSPLIT][b_bytes]
    uint64_t* bar = reinterpret_cast<uint64_t*>(Bbuf + 2 * NSPLIT * b_bytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int pi = blockIdx.y;
    const int c0 = blockIdx.x * kDftCols;
    const int nt0 = p.n_pad < 256 ? p.n_pad : 256, nt1 = p.n_pad - nt0;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    if (warp == 0) tc_alloc(tslot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const float2* tp = p.T + static_cast<int64_t>(pi) * p.nd * p.spc;
    // producer role: column m = tid % 128, rows g = 8 ks + 4 (tid / 128) .. + 3
    const int m = tid & 127, half_rows = tid >> 7;
    const int c = c0 + m;
    uint32_t use[2] = {0, 0};
    bool ok = true;
    for (int ks = 0; ks < p.ksteps && ok; ++ks) {
        const int b = ks & 1;
        if (ks >= 2) {   // the MMAs of step ks-2 read this buffer
            const bool mine = mbar_wait_bounded(&bar[b], (use[b] - 1) & 1, p.err, 5);
            ok = __syncthreads_or(mine ? 0 : 1) == 0;
            if (!ok) break;
        }
        // B chunks (constant DFT matrix) by 16-byte asynchronous copies
        for (int s = 0; s < NSPLIT; ++s) {
            const uint8_t* src = p.B + (static_cast<int64_t>(s) * p.ksteps + ks) * b_bytes;
            uint8_t* dst = Bbuf + (b * NSPLIT + s) * b_bytes;
            for (int o = tid * 16; o < b_bytes; o += kDftThreads * 16) cp_async16(dst + o, src + o);
        }
        cp_async_commit_all();
        // A chunk: rows g = 8 ks + 4 half_rows + r of column c, K index 2 (g - 8 ks) + re|im
        float2 v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int g = 8 * ks + 4 * half_rows + r;
            v[r] = (g < p.nd && c < p.spc) ? tp[static_cast<int64_t>(g) * p.spc + c] : make_float2(0.f, 0.f);
            v[r].x *= p.scale;
            v[r].y *= p.scale;
        }
        // the 8 K values of this thread are one 16-byte core-matrix row: chunk kc = half_rows
        const int aoff = (m >> 3) * 256 + half_rows * 128 + (m & 7) * 16;
        uint4 hi, lo;
        uint32_t* hp = reinterpret_cast<uint32_t*>(&hi);
        uint32_t* lp = reinterpret_cast<uint32_t*>(&lo);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            hp[r] = pack2<FMT>(v[r].x, v[r].y);
            if (NSPLIT == 2) {
                const float2 h = unpack2<FMT>(hp[r]);
                lp[r] = pack2<FMT>(v[r].x - h.x, v[r].y - h.y);
            }
        }
        *reinterpret_cast<uint4*>(Abuf + (b * NSPLIT + 0) * A_BYTES + aoff) = hi;
        if (NSPLIT == 2) *reinterpret_cast<uint4*>(Abuf + (b * NSPLIT + 1) * A_BYTES + aoff) = lo;
        cp_async_wait_zero();
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            // products: hi*hi (+ hi*lo + lo*hi for the split variants)
            const int np = NSPLIT == 2 ? 3 : 1;
            for (int q = 0; q < np; ++q) {
                const int sa = q == 2 ? 1 : 0, sb = q == 1 ? 1 : 0;
                const uint8_t* Ab = Abuf + (b * NSPLIT + sa) * A_BYTES;
                const uint8_t* Bb = Bbuf + (b * NSPLIT + sb) * b_bytes;
                const uint64_t ad = tc_desc(Ab, 128, 256);
                const bool acc = ks > 0 || q > 0;
                tc_mma_f16(tmem, ad, tc_desc(Bb, 128, 256), tc_idesc_f16(FMT, 128, nt0), acc);
                if (nt1 > 0)
                    tc_mma_f16(tmem + 256, ad, tc_desc(Bb + (nt0 / 8) * 256, 128, 256), tc_idesc_f16(FMT, 128, nt1),
                               acc);
            }
            tc_commit(&bar[b]);
        }
        ++use[b];
    }
    // wait for the last steps' MMAs (bounded; on failure still wait for work in flight)
    for (int b = 0; b < 2 && ok; ++b)
        if (use[b] > 0) {
            const bool mine = mbar_wait_bounded(&bar[b], (use[b] - 1) & 1, p.err, 6);
            ok = __syncthreads_or(mine ? 0 : 1) == 0;
        }
    if (!ok) {
        for (int b = 0; b < 2; ++b)
            if (use[b] > 0) mbar_wait_bounded(&bar[b], (use[b] - 1) & 1, p.err, 7);
    }
    tc_fence_after();
    if (ok) {
        // epilogue: warp w reads lanes 32 (w % 4) ..; warps 0-3 the first half of the Doppler
        // bins, warps 4-7 the second
        const int sp = warp & 3, grp = warp >> 2;
        const int mrow = sp * 32 + lane;
        const int col = c0 + mrow;
        const bool valid = col < p.spc;
        const int kh = (p.nd + 1) / 2;
        const int kbeg = grp == 0 ? 0 : kh, kend = grp == 0 ? kh : p.nd;
        const float inv_s2 = 1.0f / (p.scale * p.scale);
        float* ap = p.acc + static_cast<int64_t>(pi) * p.nd * p.spc_eff;
        const int half = p.nd / 2;
        for (int k0 = kbeg & ~3; k0 < kend; k0 += 4) {
            float r8[8];
            tc_ld8(tmem + (static_cast<uint32_t>(sp * 32) << 16) + 2 * k0, r8);
            tc_wait_ld();
            int64_t idx[4];
            float pw[4];
            bool keep[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = k0 + j;
                keep[j] = valid && k >= kbeg && k < kend;
                pw[j] = __fadd_rn(__fmul_rn(r8[2 * j], r8[2 * j]), __fmul_rn(r8[2 * j + 1], r8[2 * j + 1])) * inv_s2;
                int row = k + half;
                row = row >= p.nd ? row - p.nd : row;
                int dc = col + (keep[j] && p.has_drift ? p.drift[row] : 0);
                dc = dc >= p.spc ? dc - p.spc : dc;
                idx[j] = static_cast<int64_t>(row) * p.spc_eff + dc;
            }
            float old[4];
            if (!p.first) {
#pragma unroll
                for (int j = 0; j < 4; ++j) old[j] = keep[j] ? ap[idx[j]] : 0.f;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (keep[j]) ap[idx[j]] = p.first ? pw[j] : __fadd_rn(old[j], pw[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tc_dealloc(tmem, 512);
}

// Real-form DFT matrix chunks for k_col_dft_mma: B[n = 2k + co][kk = 2g + ci] with
// (co, ci) = (re, re) cos, (re, im) sin, (im, re) -sin, (im, im) cos of 2 pi g k / ndop,
// rounded to FP16/BF16 (hi) and the rounding residual (lo), in the canonical K-major chunk
// layout of each 16-wide K step.
template <int FMT>
__global__ void k_dft_operand(int nd, int n_pad, int ksteps, int nsplit, uint8_t* __restrict__ out) {
    const int64_t total = static_cast<int64_t>(ksteps) * n_pad * 16;
    for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int ks = static_cast<int>(e / (n_pad * 16));
        const int rem = static_cast<int>(e - static_cast<int64_t>(ks) * n_pad * 16);
        const int n = rem / 16, kl = rem - (rem / 16) * 16;
        const int k = n >> 1, co = n & 1;
        const int g = 8 * ks + (kl >> 1), ci = kl & 1;
        double v = 0.0;
        if (k < nd && g < nd) {
            double sn, cs;
            sincospi(2.0 * static_cast<double>((static_cast<int64_t>(g) * k) % nd) / nd, &sn, &cs);
            v = co == ci ? cs : (co == 0 ? sn : -sn);
        }
        const int off = (n >> 3) * 256 + (kl >> 3) * 128 + (n & 7) * 16 + (kl & 7) * 2;
        const float vf = static_cast<float>(v);
        const uint16_t hi = to16<FMT>(vf);
        *reinterpret_cast<uint16_t*>(out + static_cast<int64_t>(ks) * n_pad * 32 + off) = hi;
        if (nsplit == 2) {
            const float h = FMT == 0 ? __half2float(__ushort_as_half(hi)) : __bfloat162float(__ushort_as_bfloat16(hi));
            const uint16_t lo = to16<FMT>(static_cast<float>(v - static_cast<double>(h)));
            *reinterpret_cast<uint16_t*>(out + (static_cast<int64_t>(ksteps) + ks) * n_pad * 32 + off) = lo;
        }
    }
}

}  // namespace acq
