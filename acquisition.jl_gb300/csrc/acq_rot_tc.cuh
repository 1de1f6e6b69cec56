// acq_rot_tc.cuh — secondary-code rotation search with the sign-weighted first FFT pass as a
// GEMM on the 5th-generation tensor cores and the second pass read straight from tensor memory.
//
// The rotation search (src/noncoherent_integration.jl:183-297) transforms, for every code-phase
// column and every candidate q = (rotation r, data-bit combination d), the alignment-rotated
// column x weighted per sub-block p by the candidate's +-1 pattern s_q[p] (src/sign_patterns.jl:
// 23-47). With the ndop = NC x NB split (element n2 + NB p lies in sub-block p):
//   X_q[k1 + NC k2] = sum_n2 W_NB^(n2 k2) W_ND^(n2 k1) Y_q[k1, n2],
//   Y_q[k1, n2]     = sum_p  M_q[k1, p] x[n2 + NB p],   M_q[k1, p] = W_NC^(p k1) s_q[p].
// The first line is the per-candidate second pass; the second is, for a block of W columns, one
// real GEMM
//   D[rho = (r, k1, d), n = (column, n2, re|im)] = sum_{k = (p, re|im)} A[rho, k] B[n, k]
// with A = (Re M, Im M) interleaved along K and B = (x_re, -x_im | x_im, x_re), so that one
// tensor-memory lane holds Y_q[k1, .] of one candidate for every column and n2. A (per PRN slot,
// built on the host) and B (per block of columns, built here from the tile) are split into FP16
// hi + lo; D = A_hi B_hi + A_hi B_lo + A_lo B_hi in FP32 (about 22 significant bits, FP32-class).
// The epilogue loads each lane's 2 NB values per column with tcgen05.ld, applies the twiddles,
// runs the NB-point FFT in registers, forms |X|^2, takes the max over the CB data-bit
// combinations of the lane group (strict '>', the earlier combination wins a tie), stages the
// rotation slices in shared memory and adds them to the accumulator with the destination-row
// drift, like k_col_rot_sb. One bit-edge step (the bit-edge search keeps the FP32 kernels).
//
// Persistent: one CTA per SM walks a contiguous range of (PRN, block of W columns) items. Waits on
// the MMA-completion mbarrier are bounded; on a timeout the block takes one decision, waits
// (bounded) for the MMAs in flight, frees its tensor memory and returns with the error recorded.
#pragma once

#include "acq_mma.cuh"

namespace acq {

constexpr int kRotTcW = 4;            // code-phase columns per item
constexpr int kRotTcThreads = 256;    // 8 warps: two per tensor-memory lane quarter
constexpr int kRotTcCols = 256;       // tensor-memory columns (D)

template <int NC, int NB, int CB>
struct RotTcShape {
    static constexpr int ND = NC * NB;
    static constexpr int W = kRotTcW;
    static constexpr int K1P = (2 * NC + 15) / 16 * 16;    // K = (p, re|im), padded to MMA K steps
    static constexpr int KCH = K1P / 8;
    static constexpr int NCOL = 2 * NB * W;                 // N = (column, n2, re|im)
    static constexpr int N1P = (NCOL + 15) / 16 * 16;
    static constexpr int TILE_BYTES = 16 * KCH * 128;      // 128 rows of A
    static constexpr int B_BYTES = (N1P / 8) * KCH * 128;   // one split of B
    static constexpr int NLD = (2 * NB + 7) / 8;            // tcgen05.ld x8 per column
    static constexpr int GT = 128 / CB;                     // lane groups (r, k1) per M tile
    static_assert(N1P <= 256 && N1P <= kRotTcCols, "N of one MMA");
    static_assert(2 * NB * (W - 1) + 8 * NLD <= kRotTcCols, "epilogue loads stay inside the allocation");
    __host__ __device__ static constexpr int rows(int R) { return R * NC * CB; }
    __host__ __device__ static constexpr int mt(int R) { return (rows(R) + 127) / 128; }
    __host__ __device__ static constexpr int a_bytes(int R) { return 2 * mt(R) * TILE_BYTES; }   // hi, lo
    __host__ __device__ static constexpr int off_b(int R) { return a_bytes(R); }
    __host__ __device__ static constexpr int off_stage(int R) { return off_b(R) + 2 * B_BYTES; }
    __host__ __device__ static constexpr int stage_bytes() { return GT * NB * W * 6; }
    __host__ __device__ static constexpr int off_tws(int R) { return (off_stage(R) + stage_bytes() + 15) / 16 * 16; }
    __host__ __device__ static constexpr int off_cro(int R) { return off_tws(R) + ND * 8; }
    __host__ __device__ static constexpr int off_bar(int R) { return (off_cro(R) + W * 4 + 15) / 16 * 16; }
    __host__ __device__ static constexpr int smem_bytes(int R) { return off_bar(R) + 16 + 1024; }   // + alignment
};

struct RotTcParams {
    const float2* T;          // (n, ndop, spc) coherent tile of one step
    int spc, spc_eff, bs, R, first, n_items, n_cblk;
    const float2* twD;        // ndop-point twiddles
    const uint8_t* A;         // per slot: the A operand, [hi | lo][M tile][128 rows x K]
    int a_bytes;              // bytes of one slot's A
    const int* slots;
    const int* drift;         // (ndop) destination-row shifts of this step
    float* acc;
    uint16_t* win;
    float scale;              // power of two applied to the tile before rounding to FP16
    int* err;
};

template <int NC, int NB, int CB>
__global__ void __launch_bounds__(kRotTcThreads, 1) k_rot_tc(RotTcParams p) {
    static_assert(CB == 1 || CB == 2 || CB == 4 || CB == 8, "data-bit combinations per rotation");
    using S = RotTcShape<NC, NB, CB>;
    constexpr int ND = S::ND, W = S::W, KCH = S::KCH, half = ND / 2;
    extern __shared__ uint8_t smraw_[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw_) + 1023) & ~uintptr_t(1023));
    const int MT = S::mt(p.R), nrows = S::rows(p.R);
    uint8_t* A = sm;
    uint8_t* Bo = sm + S::off_b(p.R);
    float* stg = reinterpret_cast<float*>(sm + S::off_stage(p.R));
    uint16_t* wst = reinterpret_cast<uint16_t*>(stg + S::GT * NB * W);
    float2* tws = reinterpret_cast<float2*>(sm + S::off_tws(p.R));
    int* cro = reinterpret_cast<int*>(sm + S::off_cro(p.R));
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S::off_bar(p.R));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int sp = warp & 3;                      // lane quarter of this warp
    const int cpair = (warp >> 2) * (W / 2);      // first of this warp's columns

    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    if (warp == 0) tc_alloc(tslot, kRotTcCols);
    {   // B: padding rows and K columns stay zero
        int4* b4 = reinterpret_cast<int4*>(Bo);
        for (int i = tid; i < 2 * S::B_BYTES / 16; i += blockDim.x) b4[i] = make_int4(0, 0, 0, 0);
    }
    for (int i = tid; i < ND; i += blockDim.x) tws[i] = p.twD[i];
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = tc_idesc_f16(0, 128, S::N1P);
    const float inv_s2 = 1.0f / (p.scale * p.scale);

    // a contiguous range of items (PRN-major), so the A operand changes at most a few times
    const int it0 = static_cast<int>(static_cast<int64_t>(blockIdx.x) * p.n_items / gridDim.x);
    const int it1 = static_cast<int>(static_cast<int64_t>(blockIdx.x + 1) * p.n_items / gridDim.x);
    int cur_slot = -1;
    uint32_t phase = 0;
    bool ok = true;
    for (int item = it0; item < it1 && ok; ++item) {
        const int pi = item / p.n_cblk, cb = item - (item / p.n_cblk) * p.n_cblk;
        const int c0 = cb * W;
        const int wv = min(W, p.spc - c0);
        const int slot = p.slots[pi];
        if (slot != cur_slot) {   // this PRN's A operand (the previous item's MMAs have completed)
            const int4* src = reinterpret_cast<const int4*>(p.A + static_cast<int64_t>(slot) * p.a_bytes);
            int4* dst = reinterpret_cast<int4*>(A);
            for (int i = tid; i < p.a_bytes / 16; i += blockDim.x) ACQ_BC(&src[i], 60) dst[i] = src[i];
            cur_slot = slot;
        }
        if (tid < W) {
            const int pc = min(c0 + tid, p.spc - 1);
            const int wrap = ((NB - pc / p.bs) % NB) * p.bs + pc % p.bs;   // src/noncoherent_integration.jl:212-214
            cro[tid] = ((wrap + (p.bs >> 1)) / p.bs) % NB;
        }
        __syncthreads();
        // B for this item: column c, element n2 + NB pp of its alignment-rotated column
        const float2* tp = p.T + static_cast<int64_t>(pi) * ND * p.spc;
        for (int task = tid; task < W * ND; task += blockDim.x) {
            const int c = task / ND, e = task - (task / ND) * ND;
            const int pp = e / NB, n2 = e - (e / NB) * NB;
            float2 x = make_float2(0.f, 0.f);
            if (c < wv) {
                int row = cro[c] + e;
                row = row >= ND ? row - ND : row;
                ACQ_BC(&tp[static_cast<int64_t>(row) * p.spc + c0 + c], 61) x = tp[static_cast<int64_t>(row) * p.spc + c0 + c];
            }
            const float xr = x.x * p.scale, xi = x.y * p.scale;
            const __half hr = __float2half_rn(xr), hi_ = __float2half_rn(xi);
            const __half lr = __float2half_rn(xr - __half2float(hr)), li = __float2half_rn(xi - __half2float(hi_));
            const int n_re = c * 2 * NB + 2 * n2, n_im = n_re + 1;
            const int k_r = 2 * pp, k_i = 2 * pp + 1;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                uint8_t* B = Bo + s * S::B_BYTES;
                const __half vr = s ? lr : hr, vi = s ? li : hi_;
                *reinterpret_cast<__half*>(B + op_offset<KCH>(n_re, k_r)) = vr;
                *reinterpret_cast<__half*>(B + op_offset<KCH>(n_re, k_i)) = __hneg(vi);
                *reinterpret_cast<__half*>(B + op_offset<KCH>(n_im, k_r)) = vi;
                *reinterpret_cast<__half*>(B + op_offset<KCH>(n_im, k_i)) = vr;
            }
        }
        fence_proxy_async();
        __syncthreads();
        float* ap = p.acc + static_cast<int64_t>(pi) * ND * p.spc_eff;
        uint16_t* wp = p.win + static_cast<int64_t>(pi) * ND * p.spc_eff;
        for (int t = 0; t < MT; ++t) {
            if (tid == 0) {
                tc_fence_after();
#pragma unroll
                for (int ks = 0; ks < S::K1P / 16; ++ks) {
                    const uint64_t ah = tc_desc(A + t * S::TILE_BYTES + ks * 256, 128, KCH * 128);
                    const uint64_t al = tc_desc(A + (MT + t) * S::TILE_BYTES + ks * 256, 128, KCH * 128);
                    const uint64_t bh = tc_desc(Bo + ks * 256, 128, KCH * 128);
                    const uint64_t bl = tc_desc(Bo + S::B_BYTES + ks * 256, 128, KCH * 128);
                    tc_mma_f16(tmem, ah, bh, idesc, ks > 0);
                    tc_mma_f16(tmem, ah, bl, idesc, true);
                    tc_mma_f16(tmem, al, bh, idesc, true);
                }
                tc_commit(bar);
            }
            const bool mine = mbar_wait_bounded(bar, phase, p.err, 7);
            phase ^= 1;
            ok = __syncthreads_or(mine ? 0 : 1) == 0;   // one decision for the whole block
            if (!ok) break;
            tc_fence_after();
            // epilogue: lane rho = t 128 + 32 sp + lane, group (r, k1) = rho / CB, combination d = rho % CB
            const int g0 = t * S::GT;
            if (t * 128 + sp * 32 < nrows) {   // warps whose lanes are all padding skip
                const int rho = t * 128 + sp * 32 + lane;
                const int grp = rho / CB, d = rho - (rho / CB) * CB;
                const int k1 = grp % NC;
                const uint32_t tb = tmem + (static_cast<uint32_t>(sp * 32) << 16);
#pragma unroll 1
                for (int cc = cpair; cc < cpair + W / 2; ++cc) {
                    float dv[8 * S::NLD];
#pragma unroll
                    for (int j = 0; j < S::NLD; ++j) tc_ld8(tb + cc * 2 * NB + 8 * j, dv + 8 * j);
                    tc_wait_ld();
                    float2 v[NB];
                    int ti = 0;   // n2 k1 < ND
#pragma unroll
                    for (int n2 = 0; n2 < NB; ++n2) {
                        const float2 y = make_float2(dv[2 * n2], dv[2 * n2 + 1]);
                        v[n2] = n2 ? c_mul(y, tws[ti]) : y;
                        ti += k1;
                    }
                    RegFFT<NB, false>::run(v);
                    static_for<0, NB>([&](auto kc) {
                        constexpr int k2 = decltype(kc)::value;
                        const float2 x = v[reg_perm(NB, k2)];
                        float best = __fmul_rn(__fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y)), inv_s2);
                        int bd = d;
#pragma unroll
                        for (int o = 1; o < CB; o <<= 1) {   // max over the group's combinations
                            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                            const int od = __shfl_xor_sync(0xffffffffu, bd, o);
                            if (ob > best || (ob == best && od < bd)) {
                                best = ob;
                                bd = od;
                            }
                        }
                        if (d == 0 && rho < nrows) {
                            const int s = ((grp - g0) * NB + k2) * W + cc;
                            stg[s] = best;
                            wst[s] = static_cast<uint16_t>(bd);
                        }
                    });
                }
            }
            tc_fence_before();
            __syncthreads();
            // the staged groups of this M tile into the accumulator (loads of a batch before its stores)
            const int n_grp = min(S::GT, nrows / CB - g0);
            const int n_el = n_grp * NB * W;
            for (int w0 = tid; w0 < n_el; w0 += 8 * blockDim.x) {
                int64_t idx[8];
                bool on[8];
                float old[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int w = w0 + u * blockDim.x;
                    const int gl = w / (NB * W), rem = w - (w / (NB * W)) * (NB * W);
                    const int k2 = rem / W, c = rem - (rem / W) * W;
                    on[u] = w < n_el && c < wv;
                    const int grp = g0 + gl;
                    const int r = grp / NC, k1 = grp - (grp / NC) * NC;
                    const int om = k1 + NC * k2;
                    const int row = om < half ? om + half : om - half;
                    int dr = 0;
                    if (on[u]) ACQ_BC(&p.drift[row], 62) dr = p.drift[row];
                    int dc = c0 + c + dr;
                    dc = dc >= p.spc ? dc - p.spc : dc;
                    idx[u] = static_cast<int64_t>(row) * p.spc_eff + static_cast<int64_t>(r) * p.spc + dc;
#ifdef ACQ_BOUNDS_CHECK
                    if (on[u]) on[u] = bc_ok(&ap[idx[u]], 4u, 63) && (!(p.first & 2) || bc_ok(&wp[idx[u]], 2u, 64));
#endif
                }
                if (!(p.first & 1)) {
#pragma unroll
                    for (int u = 0; u < 8; ++u) old[u] = on[u] ? ap[idx[u]] : 0.f;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (!on[u]) continue;
                    const int w = w0 + u * blockDim.x;
                    ap[idx[u]] = (p.first & 1) ? stg[w] : old[u] + stg[w];
                    if (p.first & 2) wp[idx[u]] = wst[w];
                }
            }
            __syncthreads();
        }
    }
    if (!ok) mbar_wait_bounded(bar, phase ^ 1, p.err, 8);   // let the MMAs still in flight finish
    tc_fence_after();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, kRotTcCols);
}

}  // namespace acq
