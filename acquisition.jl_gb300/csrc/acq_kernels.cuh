// acq_kernels.cuh — the FM-DBZP kernels (plain form). Each kernel cites the reference code
// it replaces (paths inside JuliaGNSS/Acquisition.jl v2.6.4).
#pragma once

#include <cstdint>

#include "acq_bounds.cuh"
#include "acq_fft.cuh"
#include "acq_kernels_fs.cuh"
#include "acqgb300.h"

namespace acq {

// ------------------------------------------------------------------ sample loading
// ComplexF32(x) with no scaling, src/acquire.jl:94,101.
__device__ __forceinline__ float2 load_sample(const void* p, int dtype, int64_t i) {
#ifdef ACQ_BOUNDS_CHECK
    {
        const unsigned sz = dtype == ACQ_CF32 ? 8u : dtype == ACQ_CI16 ? 4u : dtype == ACQ_CI8 ? 2u : 16u;
        if (!bc_ok(static_cast<const char*>(p) + i * sz, sz, 1)) return make_float2(0.f, 0.f);
    }
#endif
    switch (dtype) {
        case ACQ_CF32: return reinterpret_cast<const float2*>(p)[i];
        case ACQ_CI16: {
            short2 v = reinterpret_cast<const short2*>(p)[i];
            return make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
        }
        case ACQ_CI8: {
            char2 v = reinterpret_cast<const char2*>(p)[i];
            return make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
        }
        default: {
            double2 v = reinterpret_cast<const double2*>(p)[i];
            return make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
        }
    }
}

// ------------------------------------------------------------------ input upload
// Recordings in page-locked, device-mapped host memory (cudaHostAlloc, cudaHostRegister, pinned
// torch tensors) reach the device through this gather: every SM issues 16-byte loads across the
// host link, each byte is read once, and one launch moves up to kCopySegs recordings. Segment s
// copies vec[s + 1] - vec[s] 16-byte vectors, then tail[s] (< 16) bytes, from src[s] to dst[s];
// both addresses are 16-byte aligned. Vector i of the flattened list lies in the segment whose
// range holds it (binary search over the prefix in shared memory).
constexpr int kCopySegs = 64;
constexpr int kCopyThreads = 256;
constexpr int kCopyUnroll = 4;      // loads in flight per thread
struct CopyList {
    const unsigned char* src[kCopySegs];
    unsigned char* dst[kCopySegs];
    int64_t vec[kCopySegs + 1];     // prefix of 16-byte vectors
    int tail[kCopySegs];
    int n;
};

__global__ void __launch_bounds__(kCopyThreads) k_copy_in(CopyList L) {
    __shared__ int64_t pre[kCopySegs + 1];
    const int tid = threadIdx.x;
    const int n = L.n;
    for (int s = tid; s <= n; s += kCopyThreads) pre[s] = L.vec[s];
    __syncthreads();
    const int64_t total = pre[n];
    constexpr int kChunk = kCopyThreads * kCopyUnroll;
    for (int64_t c = static_cast<int64_t>(blockIdx.x) * kChunk; c < total; c += static_cast<int64_t>(gridDim.x) * kChunk) {
        uint4 v[kCopyUnroll];
        int seg[kCopyUnroll];
        int64_t off[kCopyUnroll];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u) {
            const int64_t i = c + u * kCopyThreads + tid;
            seg[u] = -1;
            if (i < total) {
                int lo = 0, hi = n - 1;   // the last s with pre[s] <= i
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (pre[mid] <= i) lo = mid;
                    else hi = mid - 1;
                }
                seg[u] = lo;
                off[u] = i - pre[lo];
                v[u] = reinterpret_cast<const uint4*>(L.src[lo])[off[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u)
            if (seg[u] >= 0) {
                uint4* d = reinterpret_cast<uint4*>(L.dst[seg[u]]) + off[u];
                ACQ_BC(d, 24) *d = v[u];
            }
    }
    if (blockIdx.x == 0)
        for (int s = 0; s < n; ++s)
            if (tid < L.tail[s]) {
                const int64_t b = (pre[s + 1] - pre[s]) * 16 + tid;
                ACQ_BC(L.dst[s] + b, 25) L.dst[s][b] = L.src[s][b];
            }
}

// ------------------------------------------------------------------ (a) front end
// Downconversion (src/acquire.jl:92-104) fused with the double-block FFT of every
// wrapped double block (src/coherent_integration.jl:12-56). One CTA per (step, block).
// IF phase in FP32 exactly as the reference: phase = offset + Float32(i) * step, no FMA.
__global__ void k_frontend(const void* __restrict__ in, int dtype, int64_t seg_len, int G, int bs, FftDesc fd,
                           float2* __restrict__ S, int use_if, float if_step, const float* __restrict__ if_offset) {
    extern __shared__ float2 sm[];
    const int F = fd.n;
    float2* a = sm;
    float2* b = sm + F;
    const int gi = blockIdx.x;
    const int step = gi / G;
    const int g = gi - step * G;
    const int64_t seg0 = static_cast<int64_t>(step) * seg_len;
    const float off = use_if ? if_offset[step] : 0.f;
    for (int t = threadIdx.x; t < F; t += blockDim.x) {
        float2 v = make_float2(0.f, 0.f);
        if (t < 2 * bs) {
            int64_t pos = (static_cast<int64_t>(g) * bs + t) % seg_len;
            v = load_sample(in, dtype, seg0 + pos);
            if (use_if) {
                float ph = __fadd_rn(off, __fmul_rn(__ll2float_rn(pos), if_step));
                float s, c;
                sincosf(ph, &s, &c);
                v = make_float2(__fsub_rn(__fmul_rn(v.x, c), __fmul_rn(v.y, s)),
                                __fadd_rn(__fmul_rn(v.x, s), __fmul_rn(v.y, c)));
            }
        }
        a[t] = v;
    }
    __syncthreads();
    float2* src = a;
    float2* dst = b;
    fft_block<false>(src, dst, fd, 1, F, 1, false);
    float2* out = S + static_cast<int64_t>(gi) * F;
    for (int t = threadIdx.x; t < F; t += blockDim.x) out[t] = src[t];
}

// ------------------------------------------------------------------ plan-time code spectra
// conj(FFT(code sub-block k zero-padded to fft_size)), src/plan.jl:230-251. One CTA per (slot, k).
__global__ void k_code_spectra(const int8_t* __restrict__ codes, int spc, int nb, int bs, FftDesc fd,
                               float2* __restrict__ C) {
    extern __shared__ float2 sm[];
    const int F = fd.n;
    float2* a = sm;
    float2* b = sm + F;
    const int slot = blockIdx.x / nb;
    const int k = blockIdx.x - slot * nb;
    const int8_t* code = codes + static_cast<int64_t>(slot) * spc + static_cast<int64_t>(k) * bs;
    for (int t = threadIdx.x; t < F; t += blockDim.x)
        a[t] = make_float2(t < bs ? static_cast<float>(code[t]) : 0.f, 0.f);
    __syncthreads();
    float2* src = a;
    float2* dst = b;
    fft_block<false>(src, dst, fd, 1, F, 1, false);
    // conjugated and scaled by 1/F, the inverse FFT's normalisation, so the tile kernels need no
    // per-output scaling
    float2* out = C + static_cast<int64_t>(blockIdx.x) * F;
    const float inv_F = 1.0f / static_cast<float>(F);
    for (int t = threadIdx.x; t < F; t += blockDim.x) out[t] = make_float2(src[t].x * inv_F, -src[t].y * inv_F);
}

// ------------------------------------------------------------------ (a) coherent tile
// Row g = p*nb + k, column block r of the coherent integration matrix:
// (1/F) * IFFT(S_g .* C*_{(k+r) mod nb})[0:bs), src/coherent_integration.jl:136-171 (the 1/F is
// carried by the stored code spectra).
// One CTA per (g, requested PRN); it reuses S_g for all nb code blocks, B IFFTs at a time.
__global__ void k_tile(const float2* __restrict__ S, const float2* __restrict__ C, const int* __restrict__ slots,
                       int G, int nb, int bs, int spc, FftDesc fd, int B, float2* __restrict__ T) {
    extern __shared__ float2 sm[];
    const int F = fd.n;
    float2* sg = sm;
    float2* A = sm + F;
    float2* Bb = A + B * F;
    const int g = blockIdx.x;
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int k = g % nb;
    const float2* Sg = S + static_cast<int64_t>(g) * F;
    for (int t = threadIdx.x; t < F; t += blockDim.x) sg[t] = Sg[t];
    __syncthreads();
    float2* trow = T + (static_cast<int64_t>(pi) * G + g) * spc;
    for (int m0 = 0; m0 < nb; m0 += B) {
        const int nbat = min(B, nb - m0);
        const float2* Cm = C + (static_cast<int64_t>(slot) * nb + m0) * F;
        for (int w = threadIdx.x; w < nbat * F; w += blockDim.x) {
            const int e = w % F;
            A[w] = c_mul(sg[e], __ldg(Cm + w));
        }
        __syncthreads();
        float2* src = A;
        float2* dst = Bb;
        fft_block<true>(src, dst, fd, nbat, F, 1, false);
        for (int w = threadIdx.x; w < nbat * bs; w += blockDim.x) {
            const int bb = w / bs;
            const int j = w - bb * bs;
            int r = m0 + bb - k;
            if (r < 0) r += nb;
            float2 v = src[bb * F + j];
            trow[r * bs + j] = v;
        }
        __syncthreads();
        if (src != A) {  // keep A as the product buffer for the next batch
            float2* t = A;
            A = Bb;
            Bb = t;
        }
    }
}

// ------------------------------------------------------------------ (b) simple column stage
// Doppler FFT down every column, |X|^2, fftshift fold and the drift scatter keyed by the
// destination sorted row: src/acquire.jl:265-292, :335-385 and the fused pilot kernels
// src/noncoherent_integration.jl:482-592. first != 0 writes instead of accumulating.
__global__ void k_col_simple(const float2* __restrict__ T, int ndop, int spc, int W, FftDesc fd,
                             const int* __restrict__ drift, int first, float* __restrict__ acc, int spc_eff) {
    extern __shared__ float2 sm[];
    float2* A = sm;
    float2* Bb = sm + ndop * W;
    const int pi = blockIdx.y;
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const float2* tp = T + static_cast<int64_t>(pi) * ndop * spc;
    for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        A[w] = t < wv ? tp[static_cast<int64_t>(e) * spc + c0 + t] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2* src = A;
    float2* dst = Bb;
    fft_block<false>(src, dst, fd, W, 1, W, true);
    const int half = ndop / 2;
    float* ap = acc + static_cast<int64_t>(pi) * ndop * spc_eff;
    for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        if (t >= wv) continue;
        const float2 x = src[w];
        const float p = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
        int row = e + half;
        if (row >= ndop) row -= ndop;
        int dc = c0 + t + drift[row];
        if (dc >= spc) dc -= spc;
        float* cell = ap + static_cast<int64_t>(row) * spc_eff + dc;
        *cell = first ? p : *cell + p;
    }
}

// Destination-row update of the sign/rotation stage (top/bottom half swap of
// src/noncoherent_integration.jl:92-113 and :267-293, including the odd-ndop quirk where raw
// bins 0 and ndop-1 both land on row ndop/2 and row ndop-1 is never written).
__device__ __forceinline__ void stage_update(float* stage, uint16_t* wst, const float2* X, int ndop, int W,
                                             int om, int t, bool use_max, int cand) {
    const int half = ndop / 2;
    const bool odd = (ndop & 1) != 0;
    if (odd && om == ndop - 1) return;
    int order_n = (odd && om == 0) ? 2 : 1;
    for (int u = 0; u < order_n; ++u) {
        const int o = u == 0 ? om : ndop - 1;
        const int dst = o < half ? o + half : o - half;
        const float2 x = X[o * W + t];
        const float p = __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y));
        float* s = stage + dst * W + t;
        if (!use_max || p > *s) {
            *s = p;
            wst[dst * W + t] = static_cast<uint16_t>(cand);
        }
    }
}

// ------------------------------------------------------------------ (c) data-bit / bit-edge search
// Per column: for every bit edge e and data-bit pattern p, the zero-padded length-ndop FFT of
// the sign-weighted sum of the ndb sub-blocks (linearity of the reference's
// sum_b sign_b * FFT(pad(sub_b)), src/noncoherent_integration.jl:60-115), |.|^2 and a strict
// max into the stage; then the drift scatter of src/noncoherent_integration.jl:695-746.
__global__ void k_col_sign(const float2* __restrict__ T, int ndop, int spc, int W, FftDesc fd,
                           const float* __restrict__ pats, int n_pat, int n_coh, int ndb, int n_be, int edge_step,
                           const int* __restrict__ slots, const int* __restrict__ drift, int first,
                           float* __restrict__ acc, uint16_t* __restrict__ win, int spc_eff) {
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* A = tile + ndop * W;
    float2* Bb = A + ndop * W;
    float* stage = reinterpret_cast<float*>(Bb + ndop * W);
    uint16_t* wst = reinterpret_cast<uint16_t*>(stage + ndop * W);
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const float2* tp = T + static_cast<int64_t>(pi) * ndop * spc;
    for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        tile[w] = t < wv ? tp[static_cast<int64_t>(e) * spc + c0 + t] : make_float2(0.f, 0.f);
        stage[w] = 0.f;
        wst[w] = 0;
    }
    __syncthreads();
    const int sub_len = ndop / ndb;
    const int coh_per_bit = n_coh / ndb;
    const float* pp = pats + static_cast<int64_t>(slot) * n_pat * n_coh;
    for (int e = 0; e < n_be; ++e) {
        const int row_offset = e * edge_step;
        for (int p = 0; p < n_pat; ++p) {
            for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
                const int i = w / W, t = w - i * W;
                float2 v = make_float2(0.f, 0.f);
                if (i < sub_len) {
                    for (int b = 0; b < ndb; ++b) {
                        const float sgn = pp[p * n_coh + b * coh_per_bit];
                        const float2 x = tile[((row_offset + b * sub_len + i) % ndop) * W + t];
                        v = make_float2(v.x + sgn * x.x, v.y + sgn * x.y);
                    }
                }
                A[w] = v;
            }
            __syncthreads();
            float2* src = A;
            float2* dst = Bb;
            fft_block<false>(src, dst, fd, W, 1, W, true);
            for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
                const int om = w / W, t = w - om * W;
                stage_update(stage, wst, src, ndop, W, om, t, true, e * n_pat + p);
            }
            __syncthreads();
        }
    }
    float* ap = acc + static_cast<int64_t>(pi) * ndop * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ndop * spc_eff;
    for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
        const int row = w / W, t = w - row * W;
        if (t >= wv) continue;
        int dc = c0 + t + drift[row];
        if (dc >= spc) dc -= spc;
        const int64_t idx = static_cast<int64_t>(row) * spc_eff + dc;
        ap[idx] = first ? stage[w] : ap[idx] + stage[w];
        wp[idx] = wst[w];
    }
}

// ------------------------------------------------------------------ (c) secondary-code rotation search
// Per column and rotation: for every bit edge and data-bit combination, the length-ndop FFT of
// the pattern-weighted column rotated by the per-column block-alignment snap. This equals the
// reference's sub-block FFTs combined with the phase-ramped patterns
// (FFT_N(x)[w] = sum_p e^{-2 pi i p s / N_coh} sub_p[w], src/sign_patterns.jl:62-68) of
// _rotation_column!, src/noncoherent_integration.jl:183-297; each rotation owns its
// spc-wide slice and the drift wraps inside the slice (src/noncoherent_integration.jl:729-736).
__global__ void k_col_rot(const float2* __restrict__ T, int ndop, int spc, int W, FftDesc fd,
                          const float* __restrict__ pats, int n_coh, int nb, int bs, int R, int combos, int n_be,
                          int edge_step, int use_max, const int* __restrict__ slots, const int* __restrict__ drift,
                          int first, float* __restrict__ acc, uint16_t* __restrict__ win, int spc_eff) {
    extern __shared__ float2 sm[];
    float2* tile = sm;
    float2* A = tile + ndop * W;
    float2* Bb = A + ndop * W;
    float* stage = reinterpret_cast<float*>(Bb + ndop * W);
    uint16_t* wst = reinterpret_cast<uint16_t*>(stage + ndop * W);
    int* cro = reinterpret_cast<int*>(wst + ((ndop * W + 1) & ~1));
    const int pi = blockIdx.y;
    const int slot = slots[pi];
    const int c0 = blockIdx.x * W;
    const int wv = min(W, spc - c0);
    const int n_pat = R * combos;
    const float2* tp = T + static_cast<int64_t>(pi) * ndop * spc;
    for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
        const int e = w / W, t = w - e * W;
        tile[w] = t < wv ? tp[static_cast<int64_t>(e) * spc + c0 + t] : make_float2(0.f, 0.f);
    }
    for (int t = threadIdx.x; t < W; t += blockDim.x) {
        const int pc = c0 + t;
        const int wrap = ((nb - pc / bs) % nb) * bs + pc % bs;   // src/noncoherent_integration.jl:212-214
        cro[t] = ((wrap + (bs >> 1)) / bs) % nb;
    }
    __syncthreads();
    const float* pp = pats + static_cast<int64_t>(slot) * n_pat * n_coh;
    float* ap = acc + static_cast<int64_t>(pi) * ndop * spc_eff;
    uint16_t* wp = win + static_cast<int64_t>(pi) * ndop * spc_eff;
    for (int ri = 0; ri < R; ++ri) {
        for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
            stage[w] = 0.f;
            wst[w] = 0;
        }
        __syncthreads();
        for (int e = 0; e < n_be; ++e) {
            for (int d = 0; d < combos; ++d) {
                const int q = ri * combos + d;
                const float* pq = pp + static_cast<int64_t>(q) * n_coh;
                for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
                    const int i = w / W, t = w - i * W;
                    int eff = (e * edge_step + cro[t]) % ndop;
                    int row = eff + i;
                    if (row >= ndop) row -= ndop;
                    const float sgn = pq[i / nb];
                    const float2 x = tile[row * W + t];
                    A[w] = make_float2(sgn * x.x, sgn * x.y);
                }
                __syncthreads();
                float2* src = A;
                float2* dst = Bb;
                fft_block<false>(src, dst, fd, W, 1, W, true);
                for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
                    const int om = w / W, t = w - om * W;
                    stage_update(stage, wst, src, ndop, W, om, t, use_max != 0, e * combos + d);
                }
                __syncthreads();
            }
        }
        for (int w = threadIdx.x; w < ndop * W; w += blockDim.x) {
            const int row = w / W, t = w - row * W;
            if (t >= wv) continue;
            int dc = c0 + t + drift[row];
            if (dc >= spc) dc -= spc;
            const int64_t idx = static_cast<int64_t>(row) * spc_eff + ri * spc + dc;
            ap[idx] = first ? stage[w] : ap[idx] + stage[w];
            wp[idx] = wst[w];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ (c) reduction
// Peak with the reference tie-break, FP64 noise sums. Materialised order (lowest effective
// column, then lowest row: src/est_signal_noise_power.jl:109-135); streamed rotation order
// (code-phase column, rotation slice, row: src/acquire.jl:306-324).

constexpr int kStatsCols = 256;  // columns per stats CTA

__global__ void k_stats(const float* __restrict__ acc, int ndop, int ncols, int spc, int R, int streamed_rot,
                        double* __restrict__ rowpart, double* __restrict__ colsum,
                        unsigned long long* __restrict__ peakpart) {
    __shared__ float colred[8][kStatsCols];
    __shared__ unsigned long long keyred[8];
    // per-lane FP32 row partials of a chunk of 32 rows; one thread per row sums its 32 partials
    // in FP64 (instead of an FP64 shuffle tree run by every lane)
    __shared__ float rowred[32][33];
    const int pi = blockIdx.y;
    const int nct = gridDim.x;
    const int c0 = blockIdx.x * kStatsCols;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const float* ap = acc + static_cast<int64_t>(pi) * ndop * ncols;
    float cpart[kStatsCols / 32];
#pragma unroll
    for (int i = 0; i < kStatsCols / 32; ++i) cpart[i] = 0.f;
    unsigned long long best = 0ULL;
    double* rp = rowpart + (static_cast<int64_t>(pi) * nct + blockIdx.x) * ndop;
    for (int e0 = 0; e0 < ndop; e0 += 32) {
        // rows e0 + wp, e0 + wp + 8, ... of this chunk
        for (int e = e0 + wp; e < min(e0 + 32, ndop); e += 8) {
            float rs = 0.f;
            const float* rowp = ap + static_cast<int64_t>(e) * ncols;
#pragma unroll
            for (int i = 0; i < kStatsCols / 32; ++i) {
                const int c = c0 + lane + 32 * i;
                if (c < ncols) {
                    const float v = rowp[c];
                    cpart[i] += v;
                    rs += v;
                    uint32_t order;
                    if (streamed_rot) {
                        const int s = c / spc, cp = c - s * spc;
                        order = (static_cast<uint32_t>(cp) * R + s) * static_cast<uint32_t>(ndop) + e;
                    } else {
                        order = static_cast<uint32_t>(c) * ndop + e;
                    }
                    const unsigned long long key = peak_key(v, order);
                    best = key > best ? key : best;
                }
            }
            rowred[e - e0][lane] = rs;
        }
        __syncthreads();
        if (threadIdx.x < 32 && e0 + static_cast<int>(threadIdx.x) < ndop) {
            double rsd = 0.0;
            for (int l = 0; l < 32; ++l) rsd += static_cast<double>(rowred[threadIdx.x][l]);
            rp[e0 + threadIdx.x] = rsd;
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < kStatsCols / 32; ++i) colred[wp][lane + 32 * i] = cpart[i];
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other > best ? other : best;
    }
    if (lane == 0) keyred[wp] = best;
    __syncthreads();
    for (int c = threadIdx.x; c < kStatsCols; c += blockDim.x) {
        if (c0 + c < ncols) {
            double s = 0.0;
            for (int w = 0; w < 8; ++w) s += static_cast<double>(colred[w][c]);
            colsum[static_cast<int64_t>(pi) * ncols + c0 + c] = s;
        }
    }
    if (threadIdx.x == 0) {
        unsigned long long b = keyred[0];
        for (int w = 1; w < 8; ++w) b = keyred[w] > b ? keyred[w] : b;
        peakpart[static_cast<int64_t>(pi) * nct + blockIdx.x] = b;
    }
}

struct ExtractParams {
    int ndop, spc, spc_eff, nb, bs, R, n_coh, ndb, n_be, n_nc, path, combos, n_pat;
    int streamed_rot, noise_estimator, samples_per_chip, interp, nct;
    // npk peak keys per PRN; rowmode 1: no column sums (the statistics came from the column
    // stage), the global mean is the total of the row sums minus the columns near the peak
    int npk, rowmode;
    double fs, fc, code_length, t_coh, doppler_first, doppler_step, cfar_thr;
};

__device__ __forceinline__ double julia_mod(double x, double y) {
    double r = fmod(x, y);
    if (r != 0.0 && ((r < 0) != (y < 0))) r += y;
    return r;
}

// Parabolic fit src/acquire.jl:9-13 in Float32 with the reference's op order (no FMA).
__device__ __forceinline__ float parabolic(float l, float p, float r, bool* zero) {
    float denom = __fmul_rn(2.f, __fsub_rn(__fsub_rn(__fmul_rn(2.f, p), l), r));
    *zero = denom == 0.f;
    return *zero ? 0.f : __fdiv_rn(__fsub_rn(r, l), denom);
}

// Result extraction, src/acquire.jl:544-671 (materialised) and :681-781 (streamed).
__global__ void k_extract(const float* __restrict__ acc, const uint16_t* __restrict__ win,
                          const double* __restrict__ rowpart, const double* __restrict__ colsum,
                          const unsigned long long* __restrict__ peakpart, const int* __restrict__ prn_ids,
                          ExtractParams P, acq_result* __restrict__ res) {
    __shared__ double dred[256];
    __shared__ unsigned long long kred[256];
    pdl_wait();
    const int pi = blockIdx.x;
    unsigned long long best = 0ULL;
    for (int i = threadIdx.x; i < P.npk; i += blockDim.x) {
        unsigned long long k = peakpart[static_cast<int64_t>(pi) * P.npk + i];
        best = k > best ? k : best;
    }
    kred[threadIdx.x] = best;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s && kred[threadIdx.x + s] > kred[threadIdx.x]) kred[threadIdx.x] = kred[threadIdx.x + s];
        __syncthreads();
    }
    best = kred[0];
    const float peak = __uint_as_float(static_cast<uint32_t>(best >> 32));
    const uint32_t order = 0xFFFFFFFFu - static_cast<uint32_t>(best & 0xFFFFFFFFull);
    int row, col;
    if (P.streamed_rot) {
        const uint32_t cs = order / P.ndop;
        row = static_cast<int>(order - cs * P.ndop);
        const int cp = static_cast<int>(cs / P.R), s = static_cast<int>(cs % P.R);
        col = s * P.spc + cp;
    } else {
        col = static_cast<int>(order / P.ndop);
        row = static_cast<int>(order - static_cast<uint32_t>(col) * P.ndop);
    }
    // a key outside the surface can only come from a stage that gave up (its error word is set and
    // the host reports it): keep every index below in bounds
    if (order / P.ndop >= static_cast<uint32_t>(P.spc_eff) || col < 0 || col >= P.spc_eff) {
        col = 0;
        row = 0;
    }
    // noise power (FP64 sums)
    double part = 0.0;
    int lo = 0, hi = -1;
    if (P.noise_estimator == ACQ_NOISE_GLOBAL_MEAN) {
        lo = max(0, col - P.samples_per_chip);
        hi = min(P.spc_eff - 1, col + P.samples_per_chip);
        if (P.rowmode) {
            const float* apk = acc + static_cast<int64_t>(pi) * P.ndop * P.spc_eff;
            for (int i = threadIdx.x; i < P.nct * P.ndop; i += blockDim.x)
                part += rowpart[static_cast<int64_t>(pi) * P.nct * P.ndop + i];
            const int w = hi - lo + 1;
            for (int i = threadIdx.x; i < w * P.ndop; i += blockDim.x) {
                const int r = i / w, c = lo + (i - r * w);
                part -= static_cast<double>(apk[static_cast<int64_t>(r) * P.spc_eff + c]);
            }
        } else {
            for (int c = threadIdx.x; c < P.spc_eff; c += blockDim.x)
                if (c < lo || c > hi) part += colsum[static_cast<int64_t>(pi) * P.spc_eff + c];
        }
    } else {
        const int opp = (row + P.ndop / 2) % P.ndop;
        for (int i = threadIdx.x; i < P.nct; i += blockDim.x)
            part += rowpart[(static_cast<int64_t>(pi) * P.nct + i) * P.ndop + opp];
    }
    dred[threadIdx.x] = part;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) dred[threadIdx.x] += dred[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    double noise_d;
    if (P.noise_estimator == ACQ_NOISE_GLOBAL_MEAN)
        noise_d = dred[0] / (static_cast<double>(P.spc_eff - (hi - lo + 1)) * P.ndop);
    else
        noise_d = dred[0] / static_cast<double>(P.spc_eff);
    const float noise = __double2float_rn(noise_d);
    const float signal = __fsub_rn(peak, noise);
    const float pnr = __fdiv_rn(__fadd_rn(signal, noise), noise);
    const float sn = __fdiv_rn(signal, noise);
    const double cn0 = 10.0 * log10(static_cast<double>(sn) / P.t_coh);
    const int rotation_block = col / P.spc;
    const int scrambled = col - rotation_block * P.spc;
    const int block_row = scrambled / P.bs;
    const int delay = ((P.nb - block_row) % P.nb) * P.bs + (scrambled - block_row * P.bs);
    double code_phase = julia_mod((-static_cast<double>(delay)) * P.fc / P.fs, P.code_length);
    double doppler = P.doppler_first + row * P.doppler_step;
    const float* ap = acc + static_cast<int64_t>(pi) * P.ndop * P.spc_eff;
    if (P.interp) {
        const int col_l = (scrambled - 1 + P.spc) % P.spc + rotation_block * P.spc;
        const int col_r = (scrambled + 1) % P.spc + rotation_block * P.spc;
        const int row_l = row == 0 ? P.ndop - 1 : row - 1;
        const int row_r = row == P.ndop - 1 ? 0 : row + 1;
        const float pl = ap[static_cast<int64_t>(row) * P.spc_eff + col_l];
        const float pr = ap[static_cast<int64_t>(row) * P.spc_eff + col_r];
        const float dl = ap[static_cast<int64_t>(row_l) * P.spc_eff + col];
        const float dr = ap[static_cast<int64_t>(row_r) * P.spc_eff + col];
        const float sq = __fsqrt_rn(noise);
        if (fmaxf(pl, pr) > sq) {
            bool z;
            const float frac = parabolic(pl, peak, pr, &z);
            const double d_int = z ? static_cast<double>(delay)
                                   : static_cast<double>(__fadd_rn(static_cast<float>(delay), frac));
            code_phase = julia_mod((-d_int) * P.fc / P.fs, P.code_length);
        }
        if (fmaxf(dl, dr) > sq) {
            bool z;
            const float frac = parabolic(dl, peak, dr, &z);
            doppler = doppler + static_cast<double>(frac) * P.doppler_step;
        }
    }
    acq_result r;
    r.prn = prn_ids[pi];
    r.secondary_code_phase = -1;
    r.carrier_doppler_hz = doppler;
    r.code_phase = code_phase;
    r.cn0_dbhz = cn0;
    r.noise_power = noise;
    r.peak_to_noise_ratio = pnr;
    r.peak_power = peak;
    r.num_noncoherent_integrations = P.n_nc;
    r.peak_doppler_bin = row;
    r.peak_code_bin = col;
    r.sign_pattern = -1;
    r.bit_edge = -1;
    if (P.path != 0) {
        const int wv = win[(static_cast<int64_t>(pi) * P.ndop + row) * P.spc_eff + col];
        const int per_edge = P.path == 2 ? P.combos : P.n_pat;
        r.bit_edge = wv / per_edge;
        r.sign_pattern = wv - r.bit_edge * per_edge;
    }
    r.detected = static_cast<double>(pnr) > P.cfar_thr ? 1 : 0;
    r.reserved = 0;
    res[pi] = r;
}

// ------------------------------------------------------------------ (c) secondary-code phase
// Prompt correlation of each of the first L code periods at the acquired (Doppler, code phase),
// src/acquire.jl:503-523. One CTA per (requested PRN, period k); only detected PRNs
// (src/acquire.jl:750-757) do work.
__global__ void k_secondary_prompt(const void* __restrict__ in, int dtype, const int8_t* __restrict__ chips,
                                   int64_t chips_len, const int* __restrict__ slots, int spc, double fs, double fc,
                                   double interm_freq, const acq_result* __restrict__ res, double2* __restrict__ zs,
                                   int L) {
    __shared__ double red[2][256];
    const int pi = blockIdx.x, k = blockIdx.y;
    const acq_result r = res[pi];
    if (!r.detected) return;
    const int8_t* ch = chips + static_cast<int64_t>(slots[pi]) * chips_len;
    const double phase_step = -2.0 * 3.14159265358979323846 * (interm_freq + r.carrier_doppler_hz) / fs;
    const double ratio = fc / fs;
    double sp = fmod(r.code_phase, static_cast<double>(chips_len));
    if (sp < 0) sp += static_cast<double>(chips_len);
    double ar = 0.0, ai = 0.0;
    const int64_t base = static_cast<int64_t>(k) * spc;
    for (int n = threadIdx.x; n < spc; n += blockDim.x) {
        const double ph = __dadd_rn(sp, __dmul_rn(static_cast<double>(n), ratio));
        int64_t idx = static_cast<int64_t>(floor(ph));
        idx %= chips_len;
        const float c = static_cast<float>(ch[idx]);
        const float2 x = load_sample(in, dtype, base + n);
        double s, co;
        sincos(phase_step * static_cast<double>(base) + phase_step * static_cast<double>(n), &s, &co);
        const float cr = static_cast<float>(co), ci = static_cast<float>(s);
        const float pr = (x.x * cr - x.y * ci) * c, pim = (x.x * ci + x.y * cr) * c;
        ar += pr;
        ai += pim;
    }
    red[0][threadIdx.x] = ar;
    red[1][threadIdx.x] = ai;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            red[0][threadIdx.x] += red[0][threadIdx.x + s];
            red[1][threadIdx.x] += red[1][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) zs[static_cast<int64_t>(pi) * L + k] = make_double2(red[0][0], red[1][0]);
}

// Despread against the L rotations and take the strongest (strict >), src/acquire.jl:524-537.
__global__ void k_secondary_argmax(const double2* __restrict__ zs, const int8_t* __restrict__ sec, int L,
                                   acq_result* __restrict__ res, int n) {
    const int pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= n || !res[pi].detected) return;
    int best_r = 0;
    double best = -1.0;
    for (int r = 0; r < L; ++r) {
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < L; ++k) {
            const double2 z = zs[static_cast<int64_t>(pi) * L + k];
            const double s = sec[(k + r) % L];
            sr += s * z.x;
            si += s * z.y;
        }
        const double mag = sr * sr + si * si;
        if (mag > best) {
            best = mag;
            best_r = r;
        }
    }
    res[pi].secondary_code_phase = best_r;
}

}  // namespace acq
