// acq_kernels_fs.cuh — FM-DBZP kernels specialised at compile time for hot sizes: the two-pass
// register FFT (acq_fft.cuh) replaces the generic Stockham stages. Instantiated in the
// acq_inst_*.cu translation units; each kernel cites the reference code it replaces (paths
// inside JuliaGNSS/Acquisition.jl v2.6.4).
#pragma once

#include <cooperative_groups.h>
#include <cuda.h>
#include <cstdint>

#include "acq_bounds.cuh"
#include "acq_fft.cuh"

namespace acq {

// Programmatic dependent launch (a kernel launched with programmatic stream serialisation may
// start while its predecessor in the stream finishes): pdl_trigger lets the next kernel's blocks
// be scheduled once every block of this grid has issued it; pdl_wait blocks until the preceding
// grid has completed and its memory operations are visible. Every kernel of such a chain waits
// before it exits, so the ordering stays transitive. Both are no-ops in a normal launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ------------------------------------------------------------------ specialised hot sizes
__host__ __device__ constexpr int tile_row_pitch(int n2) { return n2 % 2 == 0 ? n2 + 1 : n2; }

// Coherent tile with the two-pass register FFT (F = N1 * N2): same mathematics as k_tile,
// NF inverse FFTs per row and round; pass 1 forms S_g .* C*_m on the fly, pass 2 writes the
// first bs lags of each row straight to the tile. `twT` holds the pass-1 twiddles W_F^{n2 k1} at
// [k1 * N2 + n2]. A CTA transforms R rows g0, g0 + nb, ... that share g mod nb, so they use the
// code blocks in the same order: each code-spectrum value loaded in pass 1 serves R products, and
// each thread runs R independent FFTs. Every output value is computed by the same operations
// whatever R is.
template <int N1, int N2, int R>
__global__ void __launch_bounds__(256) k_tile_fs(const float2* __restrict__ S, const float2* __restrict__ C,
                                                 const int* __restrict__ slots, int G, int nb, int bs, int spc,
                                                 const float2* __restrict__ twT, int NF,
                                                 float2* __restrict__ T, int64_t t_step_stride, int FS) {
    constexpr int F = N1 * N2;
    // row pitch of the pass-1 output in a buffer: pass-2 thread k1 reads row k1, so an even N2
    // gets one element of padding (rows of a power-of-two length would share banks)
    constexpr int P2 = tile_row_pitch(N2);
    extern __shared__ float2 sm[];
    float2* sg = sm;            // R rows of S
    float2* buf = sm + R * F;   // R * NF buffers of stride FS >= N1 * P2 (padding staggers the banks of neighbouring FFTs)
    const int k = blockIdx.x % nb;
    const int g0 = (blockIdx.x / nb) * R * nb + k;
    const int nr = min(R, (G - g0 + nb - 1) / nb);   // rows of this CTA inside the plan's G
    const int pi = blockIdx.y;
    const int slot = slots[pi];
#pragma unroll
    for (int rho = 0; rho < R; ++rho) {
        const float2* Sg = S + (static_cast<int64_t>(blockIdx.z) * G + g0 + rho * nb) * F;
        for (int t = threadIdx.x; t < F; t += blockDim.x)
            sg[rho * F + t] = rho < nr ? Sg[t] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2* trow = T + blockIdx.z * t_step_stride + (static_cast<int64_t>(pi) * G + g0) * spc;
    for (int m0 = 0; m0 < nb; m0 += NF) {
        const int nf = min(NF, nb - m0);
        for (int task = threadIdx.x; task < nf * N2; task += blockDim.x) {
            // odd FFTs of the round take n2 in descending order: a half-warp spanning FFTs f and
            // f + 1 then reads one contiguous range of S positions (shared ones broadcast) instead
            // of two ranges that fall on the same banks
            const int f = task / N2, i = task - f * N2;
            const int n2 = (f & 1) ? N2 - 1 - i : i;
            const float2* Cm = C + (static_cast<int64_t>(slot) * nb + m0 + f) * F;
            float2 v[R][N1];
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) {
                const int n = n2 + N2 * n1;
                const float2 c = __ldg(Cm + n);
#pragma unroll
                for (int rho = 0; rho < R; ++rho) v[rho][n1] = c_mul(sg[rho * F + n], c);
            }
#pragma unroll
            for (int rho = 0; rho < R; ++rho) RegFFT<N1, true>::run(v[rho]);
            static_for<0, N1>([&](auto kc) {
                constexpr int k1 = decltype(kc)::value;
                constexpr int pr = reg_perm(N1, k1);
                const bool twd = k1 != 0 && n2 != 0;
                const float2 w = twd ? tw_load<true>(twT, k1 * N2 + n2) : make_float2(1.f, 0.f);
#pragma unroll
                for (int rho = 0; rho < R; ++rho) {
                    float2 y = v[rho][pr];
                    if (twd) y = c_mul(y, w);
                    buf[(rho * NF + f) * FS + n2 + P2 * k1] = y;
                }
            });
        }
        __syncthreads();
        for (int task = threadIdx.x; task < R * nf * N1; task += blockDim.x) {
            const int rho = task / (nf * N1);
            const int rem = task - rho * nf * N1;
            const int f = rem / N1, k1 = rem - f * N1;
            if (rho >= nr) continue;
            const float2* x = buf + (rho * NF + f) * FS;
            float2 v[N2];
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2) v[n2] = x[P2 * k1 + n2];
            RegFFT<N2, true>::run(v);
            int r = m0 + f - k;
            if (r < 0) r += nb;
            float2* dst = trow + static_cast<int64_t>(rho) * nb * spc + r * bs;
            static_for<0, N2>([&](auto kc) {
                constexpr int k2 = decltype(kc)::value;
                constexpr int pr = reg_perm(N2, k2);
                // F >= 2 bs: lags from F / 2 on are never kept, so the FFT outputs feeding only
                // them are dropped at compile time
                if constexpr (N1 * k2 < F / 2) {
                    const int j = k1 + N1 * k2;
                    if (j < bs) {
                        const float2 y = v[pr];
                        dst[j] = y;
                    }
                }
            });
        }
        __syncthreads();
    }
}

// Simple column stage with the two-pass register FFT (ndop = N1 * N2): in place in shared
// memory, |X|^2, fftshift and the destination-row drift scatter fused into pass 2.
template <int N1, int N2>
__global__ void __launch_bounds__(256) k_col_simple_fs(const float2* __restrict__ T, int spc, int W,
                                                       const float2* __restrict__ twD, const int* __restrict__ drift,
                                                       int first, int has_drift, float* __restrict__ acc, int spc_eff) {
    constexpr int ND = N1 * N2;
    extern __shared__ float2 sm[];
    int* dr = reinterpret_cast<int*>(sm + ND * W);
    const int pi = blockIdx.y;
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const float2* tp = T + static_cast<int64_t>(pi) * ND * spc;
    for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        float2 v = make_float2(0.f, 0.f);
        if (t < wv) ACQ_BC(&tp[static_cast<int64_t>(e) * spc + c0 + t], 40) v = tp[static_cast<int64_t>(e) * spc + c0 + t];
        sm[w] = v;
    }
    for (int i = threadIdx.x; i < ND; i += blockDim.x) dr[i] = has_drift ? drift[i] : 0;
    __syncthreads();
    for (int task = threadIdx.x; task < N2 * W; task += blockDim.x) {
        const int n2 = task / W, t = task - n2 * W;
        fourstep_pass1<N1, N2, false>(sm + t, W, n2, twD);
    }
    __syncthreads();
    constexpr int half = ND / 2;
    float* ap = acc + static_cast<int64_t>(pi) * ND * spc_eff;
    for (int task = threadIdx.x; task < N1 * W; task += blockDim.x) {
        const int k1 = task / W, t = task - k1 * W;
        if (t >= wv) continue;
        const int c = c0 + t;
        float2 v[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) v[n2] = sm[(N2 * k1 + n2) * W + t];
        RegFFT<N2, false>::run(v);
        // power in natural order, then the accumulator cells: loads batched ahead of the stores
        float p[N2];
        int64_t idx[N2];
        static_for<0, N2>([&](auto kc) {
            constexpr int k2 = decltype(kc)::value;
            constexpr int pr = reg_perm(N2, k2);
            const float2 x = v[pr];
            p[k2] = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
            int row = k1 + N1 * k2 + half;
            if (row >= ND) row -= ND;
            int dc = c + dr[row];
            if (dc >= spc) dc -= spc;
            idx[k2] = static_cast<int64_t>(row) * spc_eff + dc;
        });
        if (first) {
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) ap[idx[k2]] = p[k2];
        } else {
            float old[N2];
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) old[k2] = ap[idx[k2]];
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) ap[idx[k2]] = __fadd_rn(old[k2], p[k2]);
        }
    }
}

// ------------------------------------------------------------------ TMA-staged column stage
// mbarrier / bulk-tensor helpers (PTX ISA 8.x).
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// the same load with an L2 evict-first policy (data read once)
__device__ __forceinline__ void tma_load_2d_ef(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, "
        "%3}], [%4], %5;" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

// Bounded wait on an mbarrier phase: gives up after kWaitLimit polls, records `code` in *err.
constexpr uint32_t kWaitLimit = 1u << 24;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err, int code,
                                                  uint32_t limit = kWaitLimit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicExch(err, code);
    return false;
}

// Peak key with the reference tie-break: float bits above the complemented scan order, so the
// largest key is the largest value and, among equal values, the first in scan order.
__device__ __forceinline__ unsigned long long peak_key(float v, uint32_t order) {
    return (static_cast<unsigned long long>(__float_as_uint(v)) << 32) |
           static_cast<unsigned long long>(0xFFFFFFFFu - order);
}

struct ColTmaParams {
    int spc, spc_eff, n_nc, W, halo, box_rows, n_boxes, n_items, n_cblk, rows_per_step;
    int n1;                // pass-2 FFTs per column when the first pass was applied to the spectra
    // k_col_tma_k1 only, when non-null: per-item statistics for the extraction (FP64 row sums of
    // everything the item adds to a row; the peak key of the cells it stores), npk keys per PRN
    double* rowpart;
    unsigned long long* peakpart;
    int npk;
    const float2* twD;
    const int* drift;      // (n_nc, ndop) in [0, spc)
    float* acc;            // (n_req, ndop, spc_eff)
    int* err;
    // k_col_tma_k1: polls of each tile wait before the block gives up (kWaitLimit; a test sets
    // 0 to run the give-up path); the wait for copies still in flight keeps the full limit
    uint32_t wait_polls;
};

// Persistent column stage for all accumulation steps of the simple path. Work item = (requested
// PRN, block of W code-phase columns); for every step the (ndop x W) tile of the coherent
// matrix arrives by TMA into one of two shared buffers while the other is transformed. The
// Doppler FFT (four-step, in place), |X|^2, fftshift and the destination-row drift scatter go
// into a shared accumulator with an H-column halo; it is written once per work item (interior
// stored, halo/edge atomically added to the zeroed accumulator). Replaces the per-step column
// kernel and its accumulator read-modify-write (src/noncoherent_integration.jl:482-592).
//
// PRE: the first four-step pass (N1 = n_coh points over the coherent periods q of the rows
// k + nb q, times W_ndop^{k k1}) was applied to the signal spectra before the coherent tile
// (k_doppler_prepass), which is linear in them and uses the same code blocks for all q of a
// class k. The tile then holds row k + nb k1 = that pass's output, and this kernel runs only the
// nb-point pass (N2 = nb, p.n1 = n_coh tasks per column).
template <int N1, int N2, bool PRE>
__global__ void __launch_bounds__(256) k_col_tma(const __grid_constant__ CUtensorMap tmap, ColTmaParams p) {
    const int n1 = PRE ? p.n1 : N1;
    const int ND = n1 * N2;
    const int W = p.W, H = p.halo, AW = p.W + 2 * p.halo;
    // each tile buffer starts on a 128-byte boundary (TMA destination): stride rounded up to
    // 16 complex values
    const int BS = (ND * W + 15) & ~15;
    extern __shared__ __align__(128) unsigned char smraw[];
    float2* const buf0 = reinterpret_cast<float2*>(smraw);   // buffer b at buf0 + b * BS
    float* accs = reinterpret_cast<float*>(buf0 + 2 * BS);
    // offs[m * ND + f]: shared-accumulator offset of FFT output f in step m (fftshifted row,
    // row pitch, halo and that row's code drift), so pass 2 needs one load per output
    int* offs = reinterpret_cast<int*>(accs + ND * AW);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smraw) + ((2 * BS * 8 + ND * AW * 4 + p.n_nc * ND * 4 + 15) / 8);
    const uint32_t tile_bytes = static_cast<uint32_t>(ND) * W * 8;
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_fence_init();
    }
    const int half = ND / 2;
    for (int i = threadIdx.x; i < p.n_nc * ND; i += blockDim.x) {
        const int m = i / ND, f = i - m * ND;
        int row = f + half;
        if (row >= ND) row -= ND;
        int sh = p.drift[m * ND + row];
        if (sh > p.spc / 2) sh -= p.spc;
        offs[i] = row * AW + H + sh;
    }
    for (int i = threadIdx.x; i < ND * AW; i += blockDim.x) accs[i] = 0.f;
    __syncthreads();
    // this CTA's tile sequence: k -> (item = blockIdx.x + (k / n_nc) * gridDim.x, step = k % n_nc)
    const int my_items = p.n_items > static_cast<int>(blockIdx.x)
                             ? (p.n_items - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                             : 0;
    const int K = my_items * p.n_nc;
    auto issue = [&](int k) {
        const int item = blockIdx.x + (k / p.n_nc) * gridDim.x;
        const int m = k % p.n_nc;
        const int pi = item / p.n_cblk, cb = item - pi * p.n_cblk;
        const int b = k & 1;
        fence_proxy_async();
        mbar_expect_tx(&mbar[b], tile_bytes);
        const int row0 = m * p.rows_per_step + pi * ND;
        for (int rb = 0; rb < p.n_boxes; ++rb)
            tma_load_2d(buf0 + b * BS + rb * p.box_rows * W, &tmap, cb * W, row0 + rb * p.box_rows, &mbar[b]);
    };
    uint32_t phases = 0u;   // bit b: the parity to wait for on mbar[b]
    // task -> (row of the pass, column) decompositions, stepped by blockDim.x without dividing by W
    const int q0 = threadIdx.x / W, r0 = threadIdx.x - q0 * W;
    const int dq = blockDim.x / W, dr = blockDim.x - dq * W;
    if (threadIdx.x == 0 && K > 0) issue(0);
    for (int k = 0; k < K; ++k) {
        const int b = k & 1;
        if (threadIdx.x == 0 && k + 1 < K) issue(k + 1);
        if (!mbar_wait_bounded(&mbar[b], (phases >> b) & 1u, p.err, 1)) {
            // give the copies in flight a bounded chance to land, then leave
            mbar_wait_bounded(&mbar[b ^ 1], (phases >> (b ^ 1)) & 1u, p.err, 1);
            return;
        }
        phases ^= 1u << b;
        const int item = blockIdx.x + (k / p.n_nc) * gridDim.x;
        const int m = k % p.n_nc;
        const int pi = item / p.n_cblk, cb = item - pi * p.n_cblk;
        const int c0 = cb * W;
        const int wv = min(W, p.spc - c0);
        float2* tl = buf0 + b * BS;
        if constexpr (!PRE) {
            for (int task = threadIdx.x, n2 = q0, t = r0; task < N2 * W;
                 task += blockDim.x, n2 += dq + (t + dr >= W), t += t + dr >= W ? dr - W : dr)
                fourstep_pass1<N1, N2, false>(tl + t, W, n2, p.twD);
            __syncthreads();
        }
        for (int task = threadIdx.x, k1 = q0, t = r0; task < n1 * W;
             task += blockDim.x, k1 += dq + (t + dr >= W), t += t + dr >= W ? dr - W : dr) {
            if (t >= wv) continue;
            float2 v[N2];
#pragma unroll
            for (int n2 = 0; n2 < N2; ++n2) v[n2] = tl[(N2 * k1 + n2) * W + t];
            RegFFT<N2, false>::run(v);
            const int* om = offs + m * ND + k1;
            float* at = accs + t;
            static_for<0, N2>([&](auto kc) {
                constexpr int k2 = decltype(kc)::value;
                constexpr int pr = reg_perm(N2, k2);
                const float2 xv = v[pr];
                const float pw = __fadd_rn(__fmul_rn(xv.x, xv.x), __fmul_rn(xv.y, xv.y));
                float* cell = at + om[n1 * k2];
                *cell = __fadd_rn(*cell, pw);
            });
        }
        __syncthreads();
        if (m == p.n_nc - 1) {
            float* ap = p.acc + static_cast<int64_t>(pi) * ND * p.spc_eff;
            // one half-warp (span <= 16) or warp per row: no division by the runtime span
            const int span = wv + 2 * H;
            const int lpr = span <= 16 ? 16 : 32;
            const int rstep = (blockDim.x / 32) * (32 / lpr);
            const int lane = threadIdx.x & (lpr - 1);
            for (int row = threadIdx.x / lpr; row < ND; row += rstep)
            for (int j = lane; j < span; j += lpr) {
                const int lc = j - H;
                float* src = accs + row * AW + H + lc;
                const float v = *src;
                *src = 0.f;
                int c = c0 + lc;
                if (c < 0) c += p.spc;
                if (c >= p.spc) c -= p.spc;
                float* cell = ap + static_cast<int64_t>(row) * p.spc_eff + c;
                if (H == 0 || (lc >= H && lc < wv - H)) *cell = v;
                else if (v != 0.f) atomicAdd(cell, v);
            }
            __syncthreads();
        }
    }
}

// Row-sum slot of (requested PRN pi, column block cb) in the per-item statistics.
__device__ __forceinline__ double* rowpart_item(const ColTmaParams& p, int pi, int cb, int nd) {
    return p.rowpart + (static_cast<int64_t>(pi) * p.n_cblk + cb) * nd;
}

// PRE-mode column stage by Doppler group: output (k1, k2) of a column needs only the nb tile rows
// k1 * nb + k (k < nb), so a work item is (requested PRN, k1, block of W columns) and its tile is
// nb rows x W columns: each row segment is W * 8 contiguous bytes (1 KB at W = 128) instead of the
// narrow segments of all ndop rows. Per step: one TMA box into one of two shared buffers (the next
// step's box loads while this one is transformed), one nb-point FFT per column, |X|^2 into a shared
// accumulator of the item's nb output rows with an H-column halo (drift shift per row and step
// from a per-item table), written once per item (interior stored, halo/edge atomically added to
// the zeroed accumulator). Same mathematics as k_col_tma<1, nb, true>.
template <int N2>
__global__ void __launch_bounds__(128) k_col_tma_k1(const __grid_constant__ CUtensorMap tmap, ColTmaParams p) {
    const int n1 = p.n1, ND = n1 * N2, half = ND / 2;
    const int W = p.W, H = p.halo, AW = W + 2 * H;
    const int BS = (N2 * W + 15) & ~15;   // buffer stride (complex values), 128-byte aligned
    extern __shared__ __align__(128) unsigned char smraw[];
    float2* const buf0 = reinterpret_cast<float2*>(smraw);   // buffer b at buf0 + b * BS
    float* accs = reinterpret_cast<float*>(buf0 + 2 * BS);   // N2 x AW
    int* sht = reinterpret_cast<int*>(accs + N2 * AW);       // n_nc x N2: accumulator offset of output k2
    int* rowof = sht + p.n_nc * N2;                          // N2: destination row of output k2
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smraw) + ((2 * BS * 8 + N2 * AW * 4 + (p.n_nc + 1) * N2 * 4 + 15) / 8);
    const uint32_t tile_bytes = static_cast<uint32_t>(N2) * W * 8;
    pdl_trigger();
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_fence_init();
    }
    for (int i = threadIdx.x; i < N2 * AW; i += blockDim.x) accs[i] = 0.f;
    __syncthreads();
    pdl_wait();   // the tile and the zeroed accumulator edges
    const int n_items = p.n_items;   // = n_req * n1 * n_cblk, item = (pi * n1 + k1) * n_cblk + cb
    const int my_items = n_items > static_cast<int>(blockIdx.x)
                             ? (n_items - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                             : 0;
    const int K = my_items * p.n_nc;
    // the box of step m of the work item with group grp (= pi * n1 + k1) and column block cb
    auto issue = [&](int m, int grp, int cb, int b) {
        fence_proxy_async();
        mbar_expect_tx(&mbar[b], tile_bytes);
        tma_load_2d_ef(buf0 + b * BS, &tmap, cb * W, m * p.rows_per_step + grp * N2, &mbar[b]);
    };
    uint32_t phases = 0u;   // bit b: the parity to wait for on mbar[b]
    if (threadIdx.x == 0 && K > 0) {
        const int g0 = static_cast<int>(blockIdx.x) / p.n_cblk;
        issue(0, g0, static_cast<int>(blockIdx.x) - g0 * p.n_cblk, 0);
    }
    // step m of work item `item` (kept across iterations: the divisions run once per item)
    int m = 0, item = blockIdx.x;
    int grp = 0, cb = 0, k1 = 0, pi = 0;
    for (int k = 0; k < K; ++k, m = (m + 1 == p.n_nc) ? 0 : m + 1, item += (m == 0) ? gridDim.x : 0) {
        const int b = k & 1;
        if (m == 0) {
            grp = item / p.n_cblk;
            cb = item - grp * p.n_cblk;
            k1 = grp % n1;
            pi = grp / n1;
        }
        if (m == 0) {   // this item's output rows and per-step offsets (the epilogue synced before)
            for (int i = threadIdx.x; i < (p.n_nc + 1) * N2; i += blockDim.x) {
                const int mm = i / N2, k2 = i - mm * N2;
                int row = k1 + n1 * k2 + half;
                if (row >= ND) row -= ND;
                if (mm == p.n_nc) {
                    rowof[k2] = row;
                } else {
                    int sh = 0;
                    ACQ_BC(&p.drift[mm * ND + row], 30) sh = p.drift[mm * ND + row];
                    if (sh > p.spc / 2) sh -= p.spc;
                    sht[i] = k2 * AW + H + sh;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0 && k + 1 < K) {   // the next step's box (a new item: divide once)
            if (m + 1 < p.n_nc) {
                issue(m + 1, grp, cb, (k + 1) & 1);
            } else {
                const int itn = item + static_cast<int>(gridDim.x);
                const int gn = itn / p.n_cblk;
                issue(0, gn, itn - gn * p.n_cblk, (k + 1) & 1);
            }
        }
        const bool landed = mbar_wait_bounded(&mbar[b], (phases >> b) & 1u, p.err, 1, p.wait_polls);
        const uint32_t parity_b = (phases >> b) & 1u;
        if (landed) phases ^= 1u << b;
        const int c0 = cb * W;
        const int wv = landed ? min(W, p.spc - c0) : 0;
        const float2* tl = buf0 + b * BS;
        const int* om = sht + m * N2;
        for (int t = threadIdx.x; t < wv; t += blockDim.x) {
            float2 v[N2];
#pragma unroll
            for (int q = 0; q < N2; ++q) v[q] = tl[q * W + t];
            RegFFT<N2, false>::run(v);
            float* at = accs + t;
            static_for<0, N2>([&](auto kc) {
                constexpr int k2 = decltype(kc)::value;
                constexpr int pr = reg_perm(N2, k2);
                const float2 xv = v[pr];
                const float pw = __fadd_rn(__fmul_rn(xv.x, xv.x), __fmul_rn(xv.y, xv.y));
                float* cell = at + om[k2];
                *cell = __fadd_rn(*cell, pw);
            });
        }
        // one block-wide decision: if any thread's wait gave up, thread 0 (which issued every copy)
        // waits with the full limit for the copies still in flight into this block's buffers, then
        // the whole block leaves (the error word is already set)
        if (__syncthreads_or(!landed)) {
            if (threadIdx.x == 0) {
                if (!landed) mbar_wait_bounded(&mbar[b], parity_b, p.err, 1);
                if (k + 1 < K) mbar_wait_bounded(&mbar[b ^ 1], (phases >> (b ^ 1)) & 1u, p.err, 1);
            }
            __syncthreads();
            return;
        }
        if (m == p.n_nc - 1) {
            float* ap = p.acc + static_cast<int64_t>(pi) * ND * p.spc_eff;
            const int span = wv + 2 * H;
            const int lane = threadIdx.x & 31, warp = threadIdx.x / 32;
            // the largest stored value of this lane and its scan order (the smaller order wins a tie)
            float bv = -1.f;
            uint32_t bo = 0xFFFFFFFFu;
            for (int k2 = warp; k2 < N2; k2 += blockDim.x / 32) {
                const int row = rowof[k2];
                float* arow = ap + static_cast<int64_t>(row) * p.spc_eff;
                float rs = 0.f;
                for (int j = lane; j < span; j += 32) {
                    const int lc = j - H;
                    float* src = accs + k2 * AW + H + lc;
                    const float v = *src;
                    *src = 0.f;
                    rs += v;
                    int c = c0 + lc;
                    if (c < 0) c += p.spc;
                    if (c >= p.spc) c -= p.spc;
                    if (H == 0 || (lc >= H && lc < wv - H)) {
                        ACQ_BC(&arow[c], 31) arow[c] = v;
                        const uint32_t ord = static_cast<uint32_t>(c) * ND + row;
                        if (v > bv || (v == bv && ord < bo)) {
                            bv = v;
                            bo = ord;
                        }
                    } else if (v != 0.f) {
                        ACQ_BC(arow + c, 32) atomicAdd(arow + c, v);
                    }
                }
                if (p.rowpart) {   // FP32 across the warp, FP64 across column blocks (in the extraction)
                    for (int o = 16; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);
                    if (lane == 0) ACQ_BC(&rowpart_item(p, pi, cb, ND)[row], 33) rowpart_item(p, pi, cb, ND)[row] = static_cast<double>(rs);
                }
            }
            if (p.peakpart) {
                unsigned long long best = bv >= 0.f ? peak_key(bv, bo) : 0ULL;
                for (int o = 16; o > 0; o >>= 1) {
                    const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
                    best = other > best ? other : best;
                }
                unsigned long long* kred = reinterpret_cast<unsigned long long*>(accs);   // free until the next item
                __syncthreads();
                if (lane == 0) kred[warp] = best;
                __syncthreads();
                if (threadIdx.x == 0) {
                    unsigned long long b = kred[0];
                    for (int w = 1; w < static_cast<int>(blockDim.x / 32); ++w) b = kred[w] > b ? kred[w] : b;
                    ACQ_BC(&p.peakpart[static_cast<int64_t>(pi) * p.npk + k1 * p.n_cblk + cb], 34)
                        p.peakpart[static_cast<int64_t>(pi) * p.npk + k1 * p.n_cblk + cb] = b;
                }
                __syncthreads();
                if (threadIdx.x < blockDim.x / 32) kred[threadIdx.x] = 0ULL;   // the accumulator starts at zero
            }
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ fused simple path
// One thread-block cluster of CL CTAs per (requested PRN, column block r) runs every
// accumulation step of the simple path without touching HBM in between:
//   1. CTA q inverse-FFTs its rows g in [q*RPC, (q+1)*RPC) (F = N1F*N2F, S_g .* C*_{(k+r) mod nb})
//      and stores lag j of row g into the shared memory of the CTA that owns column j
//      (distributed shared memory, columns [q*CPC, (q+1)*CPC) belong to CTA q);
//   2. after a cluster barrier each CTA runs the Doppler FFT (ndop = N1D*N2D) down its CPC
//      columns and adds |X|^2 (fftshift, destination-row drift) into a shared-memory
//      accumulator with an H-column halo on each side;
//   3. after the last step interior columns are stored, halo/edge columns are atomically added
//      to the (zeroed) global accumulator.
// Same mathematics as k_tile + k_col_simple_fs; the per-cell step order of the sums is kept.
struct FusedParams {
    int G, nb, bs, spc, spc_eff, n_nc, rpc, cpc, nf, halo;
    const float2* S;       // (n_nc, G, F)
    const float2* C;       // (slots, nb, F)
    const int* slots;
    const float2* twF;
    const float2* twD;
    const int* drift;      // (n_nc, ndop) in [0, spc)
    float* acc;            // (n_req, ndop, spc_eff)
};

template <int N1F, int N2F, int N1D, int N2D>
__global__ void __launch_bounds__(256) k_fused_simple(FusedParams fp) {
    namespace cg = cooperative_groups;
    constexpr int F = N1F * N2F;
    constexpr int ND = N1D * N2D;
    constexpr int NW = 8;                       // warps per CTA (256 threads)
    cg::cluster_group cluster = cg::this_cluster();
    const int q = static_cast<int>(cluster.block_rank());
    const int CL = static_cast<int>(cluster.num_blocks());
    const int r = blockIdx.x / CL;
    const int pi = blockIdx.y;
    const int slot = fp.slots[pi];
    const int CPC = fp.cpc, H = fp.halo, AW = fp.cpc + 2 * fp.halo;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    extern __shared__ float2 sm[];
    float2* tile = sm;                                         // ND x CPC, written by every CTA of the cluster
    float2* wbuf = tile + ND * CPC + wid * F;                  // this warp's FFT buffer (NW x F)
    float* accl = reinterpret_cast<float*>(tile + ND * CPC + NW * F);   // ND x AW
    int* dr = reinterpret_cast<int*>(accl + ND * AW);          // this step's signed drift per sorted row
    const int g0 = q * fp.rpc, g1 = min(ND, g0 + fp.rpc);
    const int j0 = q * CPC;
    const int wv = max(0, min(CPC, fp.bs - j0));
    const int cpw = (CPC + NW - 1) / NW;                       // Doppler columns per warp
    for (int i = threadIdx.x; i < ND * AW; i += blockDim.x) accl[i] = 0.f;
    cluster.sync();   // every CTA of the cluster is running before any remote store
    constexpr int half = ND / 2;
    for (int m = 0; m < fp.n_nc; ++m) {
        const float2* Sm = fp.S + static_cast<int64_t>(m) * fp.G * F;
        for (int i = threadIdx.x; i < ND; i += blockDim.x) {
            int sh = fp.drift[m * ND + i];
            if (sh > fp.spc / 2) sh -= fp.spc;       // signed drift, |sh| <= H
            dr[i] = sh;
        }
        // ---- inverse FFTs: warp wid owns rows g0+wid, g0+wid+NW, ...; lags go to their owner CTA
        for (int g = g0 + wid; g < g1; g += NW) {
            const int cm = (g % fp.nb + r) % fp.nb;
            const float2* Sg = Sm + static_cast<int64_t>(g) * F;
            const float2* Cm = fp.C + (static_cast<int64_t>(slot) * fp.nb + cm) * F;
            for (int n2 = lane; n2 < N2F; n2 += 32) {
                float2 v[N1F];
#pragma unroll
                for (int n1 = 0; n1 < N1F; ++n1) {
                    const int n = n2 + N2F * n1;
                    v[n1] = c_mul(__ldg(Sg + n), __ldg(Cm + n));
                }
                RegFFT<N1F, true>::run(v);
                static_for<0, N1F>([&](auto kc) {
                    constexpr int k1 = decltype(kc)::value;
                    constexpr int pr = reg_perm(N1F, k1);
                    float2 y = v[pr];
                    if (k1 != 0 && n2 != 0) y = c_mul(y, tw_load<true>(fp.twF, n2 * k1));
                    wbuf[n2 + N2F * k1] = y;
                });
            }
            __syncwarp();
            for (int k1 = lane; k1 < N1F; k1 += 32) {
                float2 v[N2F];
#pragma unroll
                for (int n2 = 0; n2 < N2F; ++n2) v[n2] = wbuf[N2F * k1 + n2];
                RegFFT<N2F, true>::run(v);
                static_for<0, N2F>([&](auto kc) {
                    constexpr int k2 = decltype(kc)::value;
                    constexpr int pr = reg_perm(N2F, k2);
                    const int j = k1 + N1F * k2;
                    if (j < fp.bs) {
                        const int owner = j / CPC;
                        float2* dst = cluster.map_shared_rank(tile, owner);
                        const float2 y = v[pr];
                        dst[g * CPC + (j - owner * CPC)] = y;
                    }
                });
            }
            __syncwarp();
        }
        cluster.sync();
        // ---- Doppler FFT: warp wid owns columns [wid*cpw, (wid+1)*cpw); each destination cell gets
        // exactly one contribution per step (the drift scatter is a bijection per row)
        const int t0 = wid * cpw, t1 = min(wv, t0 + cpw);
        const int ncw = max(0, t1 - t0);
        for (int task = lane; task < N2D * ncw; task += 32) {
            const int n2 = task / ncw, t = t0 + (task - n2 * ncw);
            fourstep_pass1<N1D, N2D, false>(tile + t, CPC, n2, fp.twD);
        }
        __syncwarp();
        for (int task = lane; task < N1D * ncw; task += 32) {
            const int k1 = task / ncw, t = t0 + (task - k1 * ncw);
            float2 v[N2D];
#pragma unroll
            for (int n2 = 0; n2 < N2D; ++n2) v[n2] = tile[(N2D * k1 + n2) * CPC + t];
            RegFFT<N2D, false>::run(v);
            static_for<0, N2D>([&](auto kc) {
                constexpr int k2 = decltype(kc)::value;
                constexpr int pr = reg_perm(N2D, k2);
                const float2 xv = v[pr];
                const float p = __fadd_rn(__fmul_rn(xv.x, xv.x), __fmul_rn(xv.y, xv.y));
                int row = k1 + N1D * k2 + half;
                if (row >= ND) row -= ND;
                float* cell = accl + row * AW + H + t + dr[row];
                *cell = __fadd_rn(*cell, p);
            });
        }
        cluster.sync();   // every CTA is done with its tile (and dr) before the next step overwrites it
    }
    // ---- write back: interior columns are owned, halo/edge columns are shared with neighbours
    float* ap = fp.acc + static_cast<int64_t>(pi) * ND * fp.spc_eff;
    const int cbase = r * fp.bs + j0;
    const int lo = -H, hi = wv + H;
    const int span = hi - lo;
    for (int i = threadIdx.x; i < ND * span; i += blockDim.x) {
        const int row = i / span;
        const int lc = lo + (i - row * span);
        const float v = accl[row * AW + H + lc];
        int c = cbase + lc;
        if (c < 0) c += fp.spc;
        if (c >= fp.spc) c -= fp.spc;
        float* cell = ap + static_cast<int64_t>(row) * fp.spc_eff + c;
        if (H == 0 || (lc >= H && lc < wv - H)) *cell = v;
        else if (v != 0.f) atomicAdd(cell, v);
    }
}

// ------------------------------------------------------------------ specialised sign / rotation stages
// Even ndop = N1 * N2 only (the odd-ndop stage quirk stays on the generic kernels). For every
// candidate (bit edge, data-bit pattern or secondary-code rotation) the zero-padded / pattern-
// weighted column is transformed in place with the two-pass register FFT and max-reduced (or
// stored) into the stage in sorted-Doppler order, exactly as k_col_sign / k_col_rot.
// Scatter of a staged (rows x W) slice into the accumulator at column offset col0 with the
// destination-row drift: dc = (c0 + t + drift[row]) mod spc. Read-modify-writes are issued in
// batches of 8 (all loads, then all stores) so that their latencies overlap. `first`: bit 0 =
// store instead of add, bit 1 = also store the winning candidate.
__device__ __forceinline__ void scatter_rmw_rt(const float* __restrict__ stg, const uint16_t* __restrict__ wst,
                                               int n, int W, int tid, int nthr, int wv, int c0, int spc,
                                               int64_t spc_eff, int64_t col0, const int* __restrict__ drift,
                                               int first, float* __restrict__ ap, uint16_t* __restrict__ wp) {
    for (int w0 = tid; w0 < n; w0 += 8 * nthr) {
        int64_t idx[8];
        bool ok[8];
        float old[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int w = w0 + u * nthr;
            const int row = w / W, t = w - (w / W) * W;
            ok[u] = w < n && t < wv;
            int dr = 0;
            if (ok[u]) ACQ_BC(&drift[row], 42) dr = drift[row];
            int dc = c0 + t + dr;
            dc = dc >= spc ? dc - spc : dc;
            idx[u] = static_cast<int64_t>(row) * spc_eff + col0 + dc;
#ifdef ACQ_BOUNDS_CHECK
            if (ok[u]) ok[u] = bc_ok(&ap[idx[u]], 4u, 43) && (!(first & 2) || bc_ok(&wp[idx[u]], 2u, 44));
#endif
        }
        if (!(first & 1)) {
#pragma unroll
            for (int u = 0; u < 8; ++u) old[u] = ok[u] ? ap[idx[u]] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (!ok[u]) continue;
            const int w = w0 + u * nthr;
            ap[idx[u]] = (first & 1) ? stg[w] : old[u] + stg[w];
            if (first & 2) wp[idx[u]] = wst[w];
        }
    }
}
template <int W>
__device__ __forceinline__ void scatter_rmw(const float* __restrict__ stg, const uint16_t* __restrict__ wst, int n,
                                            int tid, int nthr, int wv, int c0, int spc, int64_t spc_eff,
                                            int64_t col0, const int* __restrict__ drift, int first,
                                            float* __restrict__ ap, uint16_t* __restrict__ wp) {
    scatter_rmw_rt(stg, wst, n, W, tid, nthr, wv, c0, spc, spc_eff, col0, drift, first, ap, wp);
}

template <int N1, int N2>
__device__ __forceinline__ void stage_pass2(float2* wk, int W, int k1, int t, const float2* __restrict__ twD,
                                            float* stage, uint16_t* wst, bool use_max, int cand) {
    constexpr int ND = N1 * N2;
    constexpr int half = ND / 2;
    float2 v[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = wk[(N2 * k1 + n2) * W + t];
    RegFFT<N2, false>::run(v);
    static_for<0, N2>([&](auto kc) {
        constexpr int k2 = decltype(kc)::value;
        constexpr int pr = reg_perm(N2, k2);
        const int om = k1 + N1 * k2;
        const int dst = om < half ? om + half : om - half;
        const float2 x = v[pr];
        const float pw = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
        float* sp = stage + dst * W + t;
        if (!use_max || pw > *sp) {
            *sp = pw;
            wst[dst * W + t] = static_cast<uint16_t>(cand);
        }
    });
    (void)twD;
}

template <int N1, int N2>
__global__ void __launch_bounds__(256) k_col_sign_fs(const float2* __restrict__ T, int spc, int W,
                                                     const float2* __restrict__ twD, const float* __restrict__ pats,
                                                     int n_pat, int n_coh, int ndb, int n_be, int edge_step,
                                                     const int* __restrict__ slots, const int* __restrict__ drift,
                                                     int first, float* __restrict__ acc, uint16_t* __restrict__ win,
                                                     int spc_eff) {
    constexpr int ND = N1 * N2;
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* wk = tile + ND * W;
    float* stage = reinterpret_cast<float*>(wk + ND * W);
    uint16_t* wst = reinterpret_cast<uint16_t*>(stage + ND * W);
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const float2* tp = T + static_cast<int64_t>(pi) * ND * spc;
    for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        float2 v = make_float2(0.f, 0.f);
        if (t < wv) ACQ_BC(&tp[static_cast<int64_t>(e) * spc + c0 + t], 41) v = tp[static_cast<int64_t>(e) * spc + c0 + t];
        tile[w] = v;
        stage[w] = 0.f;
        wst[w] = 0;
    }
    __syncthreads();
    const int sub_len = ND / ndb;
    const int coh_per_bit = n_coh / ndb;
    const float* pp = pats + static_cast<int64_t>(slot) * n_pat * n_coh;
    for (int e = 0; e < n_be; ++e) {
        const int row_offset = e * edge_step;
        for (int p = 0; p < n_pat; ++p) {
            for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
                const int i = w / W, t = w - i * W;
                float2 v = make_float2(0.f, 0.f);
                if (i < sub_len) {
                    for (int b = 0; b < ndb; ++b) {
                        const float sgn = pp[p * n_coh + b * coh_per_bit];
                        const float2 x = tile[((row_offset + b * sub_len + i) % ND) * W + t];
                        v = make_float2(v.x + sgn * x.x, v.y + sgn * x.y);
                    }
                }
                wk[w] = v;
            }
            __syncthreads();
            for (int task = threadIdx.x; task < N2 * W; task += blockDim.x) {
                const int n2 = task / W, t = task - n2 * W;
                fourstep_pass1<N1, N2, false>(wk + t, W, n2, twD);
            }
            __syncthreads();
            for (int task = threadIdx.x; task < N1 * W; task += blockDim.x) {
                const int k1 = task / W, t = task - k1 * W;
                stage_pass2<N1, N2>(wk, W, k1, t, twD, stage, wst, true, e * n_pat + p);
            }
            __syncthreads();
        }
    }
    float* ap = acc + static_cast<int64_t>(pi) * ND * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ND * spc_eff;
    scatter_rmw_rt(stage, wst, ND * W, W, threadIdx.x, blockDim.x, wv, c0, spc, spc_eff, 0, drift, first, ap, wp);
}

template <int N1, int N2>
__global__ void __launch_bounds__(256) k_col_rot_fs(const float2* __restrict__ T, int spc, int W,
                                                    const float2* __restrict__ twD, const float* __restrict__ pats,
                                                    int n_coh, int nb, int bs, int R, int combos, int n_be,
                                                    int edge_step, int use_max, const int* __restrict__ slots,
                                                    const int* __restrict__ drift, int first, float* __restrict__ acc,
                                                    uint16_t* __restrict__ win, int spc_eff) {
    constexpr int ND = N1 * N2;
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* wk = tile + ND * W;
    float* stage = reinterpret_cast<float*>(wk + ND * W);
    uint16_t* wst = reinterpret_cast<uint16_t*>(stage + ND * W);
    int* cro = reinterpret_cast<int*>(wst + ((ND * W + 1) & ~1));
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const int n_pat = R * combos;
    const float2* tp = T + static_cast<int64_t>(pi) * ND * spc;
    for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        float2 v = make_float2(0.f, 0.f);
        if (t < wv) ACQ_BC(&tp[static_cast<int64_t>(e) * spc + c0 + t], 41) v = tp[static_cast<int64_t>(e) * spc + c0 + t];
        tile[w] = v;
    }
    for (int t = threadIdx.x; t < W; t += blockDim.x) {
        const int pc = c0 + t;
        const int wrap = ((nb - pc / bs) % nb) * bs + pc % bs;   // src/noncoherent_integration.jl:212-214
        cro[t] = ((wrap + (bs >> 1)) / bs) % nb;
    }
    __syncthreads();
    const float* pp = pats + static_cast<int64_t>(slot) * n_pat * n_coh;
    float* ap = acc + static_cast<int64_t>(pi) * ND * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ND * spc_eff;
    for (int ri = 0; ri < R; ++ri) {
        for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
            stage[w] = 0.f;
            wst[w] = 0;
        }
        for (int e = 0; e < n_be; ++e) {
            for (int d = 0; d < combos; ++d) {
                const float* pq = pp + static_cast<int64_t>(ri * combos + d) * n_coh;
                __syncthreads();
                for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
                    const int i = w / W, t = w - i * W;
                    int row = (e * edge_step + cro[t]) % ND + i;
                    if (row >= ND) row -= ND;
                    const float sgn = pq[i / nb];
                    const float2 x = tile[row * W + t];
                    wk[w] = make_float2(sgn * x.x, sgn * x.y);
                }
                __syncthreads();
                for (int task = threadIdx.x; task < N2 * W; task += blockDim.x) {
                    const int n2 = task / W, t = task - n2 * W;
                    fourstep_pass1<N1, N2, false>(wk + t, W, n2, twD);
                }
                __syncthreads();
                for (int task = threadIdx.x; task < N1 * W; task += blockDim.x) {
                    const int k1 = task / W, t = task - k1 * W;
                    stage_pass2<N1, N2>(wk, W, k1, t, twD, stage, wst, use_max != 0, e * combos + d);
                }
            }
        }
        __syncthreads();
        for (int w = threadIdx.x; w < ND * W; w += blockDim.x) {
            const int row = w / W, t = w - row * W;
            if (t >= wv) continue;
            int dc = c0 + t + drift[row];
            if (dc >= spc) dc -= spc;
            const int64_t idx = static_cast<int64_t>(row) * spc_eff + ri * spc + dc;
            ap[idx] = first ? stage[w] : ap[idx] + stage[w];
            wp[idx] = wst[w];
        }
    }
}

// ------------------------------------------------------------------ rotation stage, sub-block split
// Rotation search with the FFT split ndop = NC x NB (NC = coherent periods = sub-blocks, NB =
// blocks per period): element n2 + NB * p of the column lies in sub-block p, so the pattern
// sign of sub-block p multiplies pass-1 register p and pass 1 reads the alignment-rotated column
// straight from the tile (no separate candidate vector). Pass-2 thread (k1, t) owns the NB output
// bins k1 + NC * k2 of column t for every candidate, so the max over data-bit combinations and
// bit edges (strict '>', earlier candidate wins) stays in registers and is scattered once per
// rotation. Same result as k_col_rot_fs. `first`: bit 0 = first accumulation step (store instead of
// add), bit 1 = store the winning candidate (only the last step's survives).
// Block size for k_col_rot_sb: every pass-2 task (k1, t) needs its own thread; pass 1 loops.
__host__ __device__ constexpr int rot_sb_block(int nc, int nb, int w) {
    return nb * w <= 256 ? ((nc > nb ? nc : nb) * w + 31) / 32 * 32 : (nc * w + 31) / 32 * 32;
}

template <int NC, int NB, int W>
__global__ void __launch_bounds__(rot_sb_block(NC, NB, W))
    k_col_rot_sb(const float2* __restrict__ T, int spc, const float2* __restrict__ twD, const float* __restrict__ pats,
                 int bs, int R, int combos, int n_be, int edge_step, int use_max, const int* __restrict__ slots,
                 const int* __restrict__ drift, int first, float* __restrict__ acc, uint16_t* __restrict__ win,
                 int spc_eff) {
    constexpr int ND = NC * NB;
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* wk = tile + ND * W;
    float2* tws = wk + ND * W;                              // ND-point twiddles
    int* cro = reinterpret_cast<int*>(tws + ND);
    float* psm = reinterpret_cast<float*>(cro + W);       // this slot's patterns (n_pat x NC)
    const int tid = threadIdx.x;
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const int n_pat = R * combos;
    const float2* tp = T + static_cast<int64_t>(pi) * ND * spc;
    {
        // the block's tile loads in flight together, then the shared-memory stores
        constexpr int NT = rot_sb_block(NC, NB, W), NL = (ND * W + NT - 1) / NT;
        float2 tv[NL];
#pragma unroll
        for (int u = 0; u < NL; ++u) {
            const int w = tid + u * NT;
            const int e = w / W, t = w - e * W;
            tv[u] = make_float2(0.f, 0.f);
            if (w < ND * W && t < wv)
                ACQ_BC(&tp[static_cast<int64_t>(e) * spc + c0 + t], 41) tv[u] = tp[static_cast<int64_t>(e) * spc + c0 + t];
        }
#pragma unroll
        for (int u = 0; u < NL; ++u)
            if (tid + u * NT < ND * W) tile[tid + u * NT] = tv[u];
    }
    for (int i = tid; i < ND; i += blockDim.x) tws[i] = twD[i];
    if (tid < W) {
        const int pc = c0 + tid;
        const int wrap = ((NB - pc / bs) % NB) * bs + pc % bs;   // src/noncoherent_integration.jl:212-214
        cro[tid] = ((wrap + (bs >> 1)) / bs) % NB;
    }
    const float* pp = pats + static_cast<int64_t>(slot) * n_pat * NC;
    for (int i = tid; i < n_pat * NC; i += blockDim.x) psm[i] = pp[i];
    __syncthreads();
    float* ap = acc + static_cast<int64_t>(pi) * ND * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ND * spc_eff;
    // pass-2 role (k1, t2) of this thread; pass-1 tasks (n2, t1) loop over the block
    const int k1 = tid / W, t2 = tid - (tid / W) * W;
    const bool p2 = tid < NC * W;
    for (int ri = 0; ri < R; ++ri) {
        float best[NB];
        int bwin[NB];
#pragma unroll
        for (int k2 = 0; k2 < NB; ++k2) {
            best[k2] = 0.f;
            bwin[k2] = 0;
        }
        for (int e = 0; e < n_be; ++e) {
            for (int d = 0; d < combos; ++d) {
                const float* pq = psm + (ri * combos + d) * NC;
                for (int task = tid; task < NB * W; task += blockDim.x) {
                    const int n2 = task / W, t1 = task - (task / W) * W;
                    int base = (e * edge_step + cro[t1]) % ND + n2;
                    if (base >= ND) base -= ND;
                    float2 v[NC];
#pragma unroll
                    for (int p = 0; p < NC; ++p) {
                        int row = base + NB * p;
                        if (row >= ND) row -= ND;
                        v[p] = c_scale(tile[row * W + t1], pq[p]);
                    }
                    RegFFT<NC, false>::run(v);
                    static_for<0, NC>([&](auto kc) {
                        constexpr int kk = decltype(kc)::value;
                        constexpr int pr = reg_perm(NC, kk);
                        float2 y = v[pr];
                        if (kk != 0) y = c_mul(y, tws[n2 * kk]);
                        wk[(n2 + NB * kk) * W + t1] = y;
                    });
                }
                __syncthreads();
                if (p2) {
                    const int cand = e * combos + d;
                    float2 v[NB];
#pragma unroll
                    for (int m = 0; m < NB; ++m) v[m] = wk[(NB * k1 + m) * W + t2];
                    RegFFT<NB, false>::run(v);
                    // block-uniform cases: a single candidate per rotation, or a max whose winners
                    // are kept only on the last step (the only winner map that survives)
                    if (!use_max) {
                        static_for<0, NB>([&](auto kc) {
                            constexpr int k2 = decltype(kc)::value;
                            const float2 x = v[reg_perm(NB, k2)];
                            best[k2] = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
                        });
                    } else if (!(first & 2)) {
                        static_for<0, NB>([&](auto kc) {
                            constexpr int k2 = decltype(kc)::value;
                            const float2 x = v[reg_perm(NB, k2)];
                            best[k2] = fmaxf(best[k2], __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y)));
                        });
                    } else {
                        static_for<0, NB>([&](auto kc) {
                            constexpr int k2 = decltype(kc)::value;
                            const float2 x = v[reg_perm(NB, k2)];
                            const float pw = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
                            const bool take = pw > best[k2];
                            best[k2] = take ? pw : best[k2];
                            bwin[k2] = take ? cand : bwin[k2];
                        });
                    }
                }
                __syncthreads();
            }
        }
        // stage the rotation slice through the (now free) work buffer, then scatter with every thread
        float* stg = reinterpret_cast<float*>(wk);
        uint16_t* wst = reinterpret_cast<uint16_t*>(stg + ND * W);
        if (p2) {
            constexpr int half = ND / 2;
#pragma unroll
            for (int k2 = 0; k2 < NB; ++k2) {
                const int om = k1 + NC * k2;
                const int row = om < half ? om + half : om - half;
                stg[row * W + t2] = best[k2];
                wst[row * W + t2] = static_cast<uint16_t>(bwin[k2]);
            }
        }
        __syncthreads();
        scatter_rmw<W>(stg, wst, ND * W, tid, blockDim.x, wv, c0, spc, spc_eff, ri * spc, drift, first, ap, wp);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ data-bit / bit-edge search, split
// Sign search (src/noncoherent_integration.jl:60-115) with the FFT split ndop = N1 x N2. For bit
// edge e every data-bit pattern p transforms v_p = sum_b s(p, b) x_b, x_b the b-th sub-block of
// the edge-shifted column zero-padded to ndop (src/sign_patterns.jl:23-47). By linearity pass 1
// transforms each sub-block once (its inputs are zero for n1 >= N1 / NDB, known at compile time)
// and pass 2 combines the sub-block results with each pattern's signs while loading. Pass-2
// thread (p, k1, t) keeps the running max over the edges for its pattern in registers; the NP
// patterns' maxima are merged at the end in candidate order (e, p) (strict '>', earlier wins).
// Same result as k_col_sign_fs. Block: NP * N1 * W threads.
template <int N1, int N2, int W, int NDB>
__global__ void __launch_bounds__((1 << (NDB - 1)) * N1 * W, ((1 << (NDB - 1)) * N1 * W <= 256) ? 2 : 1)
    k_col_sign_sb(const float2* __restrict__ T, int spc, const float2* __restrict__ twD, const float* __restrict__ pats,
                  int n_coh, int n_be, int edge_step, const int* __restrict__ slots, const int* __restrict__ drift,
                  int first, float* __restrict__ acc, uint16_t* __restrict__ win, int spc_eff) {
    constexpr int ND = N1 * N2, NP = 1 << (NDB - 1), SUB = ND / NDB, NZ = N1 / NDB;
    static_assert(N1 % NDB == 0, "sub-blocks must align with pass-1 rows");
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* wk = tile + ND * W;                 // NDB pass-1 results
    float2* tws = wk + NDB * ND * W;
    float* sgn = reinterpret_cast<float*>(tws + ND);   // s(p, b), NP x NDB
    const int tid = threadIdx.x;
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const float2* tp = T + static_cast<int64_t>(pi) * ND * spc;
    for (int w = tid; w < ND * W; w += blockDim.x) {
        const int e = w / W, t = w - (w / W) * W;
        float2 v = make_float2(0.f, 0.f);
        if (t < wv) ACQ_BC(&tp[static_cast<int64_t>(e) * spc + c0 + t], 41) v = tp[static_cast<int64_t>(e) * spc + c0 + t];
        tile[w] = v;
    }
    for (int i = tid; i < ND; i += blockDim.x) tws[i] = twD[i];
    if (tid < NP * NDB) {
        const int pp = tid / NDB, b = tid - (tid / NDB) * NDB;
        sgn[tid] = pats[(static_cast<int64_t>(slot) * NP + pp) * n_coh + b * (n_coh / NDB)];
    }
    __syncthreads();
    // pass-2 role
    const int p2 = tid / (N1 * W), r2 = tid - (tid / (N1 * W)) * (N1 * W);
    const int k1 = r2 / W, t2 = r2 - (r2 / W) * W;
    float best[N2];
    int bwin[N2];
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
        best[k2] = 0.f;
        bwin[k2] = 0;
    }
    for (int e = 0; e < n_be; ++e) {
        const int off = (e * edge_step) % ND;
        for (int task = tid; task < NDB * N2 * W; task += blockDim.x) {
            const int b = task / (N2 * W), r = task - (task / (N2 * W)) * (N2 * W);
            const int n2 = r / W, t = r - (r / W) * W;
            int base = off + b * SUB + n2;
            base = base >= ND ? base - ND : base;
            base = base >= ND ? base - ND : base;
            float2 v[N1];
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) {
                if (n1 < NZ) {
                    int row = base + N2 * n1;
                    row = row >= ND ? row - ND : row;
                    v[n1] = tile[row * W + t];
                } else {
                    v[n1] = make_float2(0.f, 0.f);
                }
            }
            RegFFT<N1, false>::run(v);
            float2* x = wk + b * ND * W;
            static_for<0, N1>([&](auto kc) {
                constexpr int kk = decltype(kc)::value;
                constexpr int pr = reg_perm(N1, kk);
                float2 y = v[pr];
                if (kk != 0) y = c_mul(y, tws[n2 * kk]);
                x[(n2 + N2 * kk) * W + t] = y;
            });
        }
        __syncthreads();
        {
            float s[NDB];
#pragma unroll
            for (int b = 0; b < NDB; ++b) s[b] = sgn[p2 * NDB + b];
            float2 v[N2];
#pragma unroll
            for (int m = 0; m < N2; ++m) {
                float2 a = make_float2(0.f, 0.f);
#pragma unroll
                for (int b = 0; b < NDB; ++b) {
                    const float2 y = wk[b * ND * W + (N2 * k1 + m) * W + t2];
                    a = b == 0 ? c_scale(y, s[0]) : c_axpy(s[b], y, a);
                }
                v[m] = a;
            }
            RegFFT<N2, false>::run(v);
            const int cand = e * NP + p2;
            if (first & 2) {   // the last step's winners are stored
                static_for<0, N2>([&](auto kc) {
                    constexpr int k2 = decltype(kc)::value;
                    const float2 x = v[reg_perm(N2, k2)];
                    const float pw = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
                    const bool take = pw > best[k2];
                    best[k2] = take ? pw : best[k2];
                    bwin[k2] = take ? cand : bwin[k2];
                });
            } else {           // earlier steps only add the maxima
                static_for<0, N2>([&](auto kc) {
                    constexpr int k2 = decltype(kc)::value;
                    const float2 x = v[reg_perm(N2, k2)];
                    best[k2] = fmaxf(best[k2], __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y)));
                });
            }
        }
        __syncthreads();
    }
    // merge the patterns' maxima (candidate order (e, p)), stage, scatter
    float* stg = reinterpret_cast<float*>(wk);
    uint16_t* wst = reinterpret_cast<uint16_t*>(stg + NP * ND * W);
    constexpr int half = ND / 2;
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
        const int om = k1 + N1 * k2;
        const int row = om < half ? om + half : om - half;
        stg[(p2 * ND + row) * W + t2] = best[k2];
        wst[(p2 * ND + row) * W + t2] = static_cast<uint16_t>(bwin[k2]);
    }
    __syncthreads();
    if (NP > 1) {
        for (int w = tid; w < ND * W; w += blockDim.x) {
            float bv = stg[w];
            int bw = wst[w];
            for (int q = 1; q < NP; ++q) {
                const float v = stg[q * ND * W + w];
                const int c = wst[q * ND * W + w];
                if (v > bv || (v == bv && c < bw)) {
                    bv = v;
                    bw = c;
                }
            }
            stg[w] = bv;
            wst[w] = static_cast<uint16_t>(bw);
        }
        __syncthreads();
    }
    float* ap = acc + static_cast<int64_t>(pi) * ND * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ND * spc_eff;
    scatter_rmw<W>(stg, wst, ND * W, tid, blockDim.x, wv, c0, spc, spc_eff, 0, drift, first, ap, wp);
}

// ------------------------------------------------------------------ bit-edge search by half spectra
// The search of k_col_sign_sb for two data bits (src/noncoherent_integration.jl:60-115 with the
// patterns of src/sign_patterns.jl:23-47, s(p, 1) = +-s(p, 0)), with less work. Candidate (e, p)
// of a column is |DFT_ND(f)|^2, f[i] = s(p, 0) x[o + i] + s(p, 1) x[o + SUB + i] for i < SUB =
// ND / 2 and 0 beyond, o = e * edge_step (each sub-block is placed at the start of its own
// zero-padded transform). From one edge to the next f moves by a cyclic shift when
// s(p, 0) = s(p, 1) and by a negacyclic one (the wrapped part negated) when s(p, 0) = -s(p, 1).
// The even bins are DFT_SUB(f), whose power a cyclic shift leaves unchanged; the odd bins are
// DFT_SUB(f W_ND^i), whose power a negacyclic shift leaves unchanged. So each pattern has one half
// spectrum that is the same for every edge (computed once, as edge 0: the first candidate wins
// exact ties) and one computed per edge: 2 (1 + n_be) half spectra per column instead of
// 4 n_be, 37.5 % fewer transform points at four edges.
// Half spectrum of parity q in the split n = n2 + N2 n1 (n1 < N1 / 2 nonzero), k = k1 + N1 k2,
// k1 = 2 j + q: pass 1 = DFT_{N1/2} over n1 of f[n2 + N2 n1] W_N1^(q n1), times W_ND^(n2 k1);
// pass 2 = DFT_N2 over n2 for each k1 of that parity.
// Thread (g, k1, t) owns bins k1 + N1 k2 of column t and takes units g, g + 2, ... of its
// parity's list [the edge-invariant half, edges 0 .. n_be - 1]; each round transforms two units of
// each parity. The two groups' maxima merge in candidate order (e, p), as in k_col_sign_sb.
template <int N1, int N2, int W>
__global__ void __launch_bounds__(2 * N1 * W, (2 * N1 * W <= 256) ? 2 : 1)
    k_col_sign_fold(const float2* __restrict__ T, int spc, const float2* __restrict__ twD,
                    const float* __restrict__ pats, int n_coh, int n_be, int edge_step, const int* __restrict__ slots,
                    const int* __restrict__ drift, int first, float* __restrict__ acc, uint16_t* __restrict__ win,
                    int spc_eff) {
    constexpr int ND = N1 * N2, SUB = ND / 2, H1 = N1 / 2, NP = 2;
    static_assert(N1 % 2 == 0, "the half spectra split the pass-1 length");
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* wk = tile + ND * W;                 // 4 slots (parity, group) of SUB x W pass-1 results
    float2* tws = wk + 2 * ND * W;
    float* sgn = reinterpret_cast<float*>(tws + ND);   // s(p, b), NP x 2
    const int tid = threadIdx.x;
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const float2* tp = T + static_cast<int64_t>(pi) * ND * spc;
    {
        // every load of the thread in flight at once, then the shared-memory stores
        constexpr int NT = 2 * N1 * W, NL = (ND * W + NT - 1) / NT;
        float2 tv[NL];
#pragma unroll
        for (int u = 0; u < NL; ++u) {
            const int w = tid + u * NT;
            const int e = w / W, t = w - (w / W) * W;
            tv[u] = make_float2(0.f, 0.f);
            if (w < ND * W && t < wv)
                ACQ_BC(&tp[static_cast<int64_t>(e) * spc + c0 + t], 45) tv[u] = tp[static_cast<int64_t>(e) * spc + c0 + t];
        }
#pragma unroll
        for (int u = 0; u < NL; ++u)
            if (tid + u * NT < ND * W) tile[tid + u * NT] = tv[u];
    }
    for (int i = tid; i < ND; i += blockDim.x) tws[i] = twD[i];
    if (tid < NP * 2) {
        const int pp = tid / 2, b = tid - (tid / 2) * 2;
        sgn[tid] = pats[(static_cast<int64_t>(slot) * NP + pp) * n_coh + b * (n_coh / 2)];
    }
    __syncthreads();
    const int g = tid / (N1 * W), r2 = tid - g * (N1 * W);
    const int k1 = r2 / W, t2 = r2 - (r2 / W) * W;
    const int par = k1 & 1, jj = k1 >> 1;
    const int p_cyc = sgn[0] == sgn[1] ? 0 : 1;   // the pattern whose even bins are edge-invariant
    // (edge, pattern) of unit u of parity q
    auto unit = [&](int q, int u, int& e, int& p) {
        const int pinv = q == 0 ? p_cyc : 1 - p_cyc;
        e = u == 0 ? 0 : u - 1;
        p = u == 0 ? pinv : 1 - pinv;
    };
    float best[N2];
    int bwin[N2];
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
        best[k2] = 0.f;
        bwin[k2] = 0;
    }
    const int nu = n_be + 1;
    for (int u0 = 0; u0 < nu; u0 += 2) {
        // pass 1: slot s = 2 q + h holds unit u0 + h of parity q
        for (int task = tid; task < 4 * N2 * W; task += blockDim.x) {
            const int s = task / (N2 * W), r = task - s * (N2 * W);
            const int q = s >> 1, u = u0 + (s & 1);
            if (u >= nu) continue;
            const int n2 = r / W, t = r - (r / W) * W;
            int e, p;
            unit(q, u, e, p);
            const float s0 = sgn[p * 2], s1 = sgn[p * 2 + 1];
            const int o = (e * edge_step) % ND;
            float2 v[H1];
#pragma unroll
            for (int n1 = 0; n1 < H1; ++n1) {
                int ra = o + n2 + N2 * n1;   // < ND + SUB
                ra = ra >= ND ? ra - ND : ra;
                int rb = ra + SUB;
                rb = rb >= ND ? rb - ND : rb;
                float2 y = c_axpy(s1, tile[rb * W + t], c_scale(tile[ra * W + t], s0));
                if (q && n1 != 0) y = c_mul(y, tws[n1 * N2]);   // W_N1^n1
                v[n1] = y;
            }
            RegFFT<H1, false>::run(v);
            float2* x = wk + s * SUB * W;
            static_for<0, H1>([&](auto kc) {
                constexpr int j = decltype(kc)::value;
                float2 y = v[reg_perm(H1, j)];
                const int kk = 2 * j + q;
                if (kk * n2 != 0) y = c_mul(y, tws[n2 * kk]);   // < ND
                x[(n2 + N2 * j) * W + t] = y;
            });
        }
        __syncthreads();
        const int u = u0 + g;
        if (u < nu) {
            int e, p;
            unit(par, u, e, p);
            const int cand = e * NP + p;
            const float2* x = wk + (2 * par + g) * SUB * W;
            float2 v[N2];
#pragma unroll
            for (int m = 0; m < N2; ++m) v[m] = x[(m + N2 * jj) * W + t2];
            RegFFT<N2, false>::run(v);
            if (first & 2) {   // the last step's winners are stored; equal powers: the earlier candidate
                static_for<0, N2>([&](auto kc) {
                    constexpr int k2 = decltype(kc)::value;
                    const float2 xv = v[reg_perm(N2, k2)];
                    const float pw = __fadd_rn(__fmul_rn(xv.x, xv.x), __fmul_rn(xv.y, xv.y));
                    const bool take = pw > best[k2] || (pw == best[k2] && cand < bwin[k2]);
                    best[k2] = take ? pw : best[k2];
                    bwin[k2] = take ? cand : bwin[k2];
                });
            } else {
                static_for<0, N2>([&](auto kc) {
                    constexpr int k2 = decltype(kc)::value;
                    const float2 xv = v[reg_perm(N2, k2)];
                    best[k2] = fmaxf(best[k2], __fadd_rn(__fmul_rn(xv.x, xv.x), __fmul_rn(xv.y, xv.y)));
                });
            }
        }
        __syncthreads();
    }
    // merge the two groups' maxima (candidate order (e, p)), stage, scatter
    float* stg = reinterpret_cast<float*>(wk);
    uint16_t* wst = reinterpret_cast<uint16_t*>(stg + 2 * ND * W);
    constexpr int half = ND / 2;
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
        const int om = k1 + N1 * k2;
        const int row = om < half ? om + half : om - half;
        stg[(g * ND + row) * W + t2] = best[k2];
        wst[(g * ND + row) * W + t2] = static_cast<uint16_t>(bwin[k2]);
    }
    __syncthreads();
    for (int w = tid; w < ND * W; w += blockDim.x) {
        float bv = stg[w];
        int bw = wst[w];
        const float v = stg[ND * W + w];
        const int c = wst[ND * W + w];
        if (v > bv || (v == bv && c < bw)) {
            bv = v;
            bw = c;
        }
        stg[w] = bv;
        wst[w] = static_cast<uint16_t>(bw);
    }
    __syncthreads();
    float* ap = acc + static_cast<int64_t>(pi) * ND * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ND * spc_eff;
    scatter_rmw<W>(stg, wst, ND * W, tid, blockDim.x, wv, c0, spc, spc_eff, 0, drift, first, ap, wp);
}

}  // namespace acq
