// acq_fft.cuh — block-cooperative mixed-radix Stockham FFT in shared memory (sm_103a).
//
// Replaces the FFTW calls of the reference (src/plan.jl:469-483) for every transform on the
// FM-DBZP path: the double-block forward FFTs, the code-block FFTs, the inverse correlation
// FFTs and the Doppler column FFTs. Any length is supported: radix 4, 2, 3 and 5 butterflies
// are unrolled; 7 and larger primes use a direct radix-p DFT from shared memory.
//
// Layout: element e of batch item b lives at buf[b * bstride + e * estride]. Each stage
// reads `src`, writes `dst` (auto-sort, no bit reversal) and the caller swaps.
#pragma once

#include <cuda_runtime.h>

namespace acq {

constexpr int kMaxFftStages = 24;

struct FftDesc {
    int n;
    int nst;
    int radix[kMaxFftStages];
    int ns[kMaxFftStages];      // product of the radices before this stage
    int stride[kMaxFftStages];  // n / (ns * radix): twiddle index step
    const float2* tw;           // n entries, exp(-2 pi i k / n)
};

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 c_mi(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV>
__device__ __forceinline__ float2 tw_load(const float2* tw, int idx) {
    float2 w = __ldg(tw + idx);
    if (INV) w.y = -w.y;
    return w;
}

template <bool INV>
__device__ __forceinline__ void bf2(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = c_add(a, b);
    v[1] = c_sub(a, b);
}

template <bool INV>
__device__ __forceinline__ void bf4(float2* v) {
    float2 s02 = c_add(v[0], v[2]), d02 = c_sub(v[0], v[2]);
    float2 s13 = c_add(v[1], v[3]), d13 = c_mi<INV>(c_sub(v[1], v[3]));
    v[0] = c_add(s02, s13);
    v[2] = c_sub(s02, s13);
    v[1] = c_add(d02, d13);
    v[3] = c_sub(d02, d13);
}

template <bool INV>
__device__ __forceinline__ void bf3(float2* v) {
    const float S3 = 0.86602540378443864676f;  // sin(2 pi / 3)
    float2 t1 = c_add(v[1], v[2]);
    float2 t2 = c_sub(v[0], c_scale(t1, 0.5f));
    float2 t3 = c_mi<INV>(c_scale(c_sub(v[1], v[2]), S3));
    v[0] = c_add(v[0], t1);
    v[1] = c_add(t2, t3);
    v[2] = c_sub(t2, t3);
}

template <bool INV>
__device__ __forceinline__ void bf5(float2* v) {
    const float C1 = 0.30901699437494742410f;   // cos(2 pi / 5)
    const float C2 = -0.80901699437494742410f;  // cos(4 pi / 5)
    const float S1 = 0.95105651629515357212f;   // sin(2 pi / 5)
    const float S2 = 0.58778525229247312917f;   // sin(4 pi / 5)
    float2 s14 = c_add(v[1], v[4]), d14 = c_sub(v[1], v[4]);
    float2 s23 = c_add(v[2], v[3]), d23 = c_sub(v[2], v[3]);
    float2 a1 = make_float2(v[0].x + C1 * s14.x + C2 * s23.x, v[0].y + C1 * s14.y + C2 * s23.y);
    float2 a2 = make_float2(v[0].x + C2 * s14.x + C1 * s23.x, v[0].y + C2 * s14.y + C1 * s23.y);
    float2 b1 = c_mi<INV>(make_float2(S1 * d14.x + S2 * d23.x, S1 * d14.y + S2 * d23.y));
    float2 b2 = c_mi<INV>(make_float2(S2 * d14.x - S1 * d23.x, S2 * d14.y - S1 * d23.y));
    v[0] = c_add(v[0], c_add(s14, s23));
    v[1] = c_add(a1, b1);
    v[4] = c_sub(a1, b1);
    v[2] = c_add(a2, b2);
    v[3] = c_sub(a2, b2);
}

template <int R, bool INV>
__device__ __forceinline__ void stage_item(const float2* __restrict__ in, float2* __restrict__ out, const float2* tw,
                                           int j, int m, int k, int Ns, int st, int estride) {
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[(j + r * m) * estride];
    if (k > 0) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = c_mul(v[r], tw_load<INV>(tw, r * k * st));
    }
    if (R == 2) bf2<INV>(v);
    if (R == 3) bf3<INV>(v);
    if (R == 4) bf4<INV>(v);
    if (R == 5) bf5<INV>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[(base + r * Ns) * estride] = v[r];
}

template <bool INV>
__device__ __forceinline__ void stage_item_generic(const float2* __restrict__ in, float2* __restrict__ out,
                                                   const float2* tw, int N, int R, int j, int m, int k, int Ns,
                                                   int st, int estride) {
    const int base = (j - k) * R + k;
    for (int t = 0; t < R; ++t) {
        float2 acc = make_float2(0.f, 0.f);
        const int step = k * st + t * m;
        int idx = 0;
        for (int q = 0; q < R; ++q) {
            float2 x = in[(j + q * m) * estride];
            acc = c_add(acc, c_mul(x, tw_load<INV>(tw, idx)));
            idx += step;
            if (idx >= N) idx -= N * (idx / N);
        }
        out[(base + t * Ns) * estride] = acc;
    }
}

// Runs every stage of an n-point FFT on B vectors. On return `src` points at the result.
// All threads of the block must call it; it ends with __syncthreads().
// batch_fastest: consecutive threads take consecutive batch items (column layouts).
template <bool INV>
__device__ void fft_block(float2*& src, float2*& dst, const FftDesc& d, int B, int bstride, int estride,
                          bool batch_fastest) {
    const int N = d.n;
    for (int s = 0; s < d.nst; ++s) {
        const int R = d.radix[s], Ns = d.ns[s], st = d.stride[s];
        const int m = N / R;
        const int items = B * m;
        for (int w = threadIdx.x; w < items; w += blockDim.x) {
            int b, j;
            if (batch_fastest) { j = w / B; b = w - j * B; }
            else { b = w / m; j = w - b * m; }
            const float2* in = src + b * bstride;
            float2* out = dst + b * bstride;
            const int k = j % Ns;
            switch (R) {
                case 4: stage_item<4, INV>(in, out, d.tw, j, m, k, Ns, st, estride); break;
                case 2: stage_item<2, INV>(in, out, d.tw, j, m, k, Ns, st, estride); break;
                case 3: stage_item<3, INV>(in, out, d.tw, j, m, k, Ns, st, estride); break;
                case 5: stage_item<5, INV>(in, out, d.tw, j, m, k, Ns, st, estride); break;
                default: stage_item_generic<INV>(in, out, d.tw, N, R, j, m, k, Ns, st, estride); break;
            }
        }
        __syncthreads();
        float2* t = src;
        src = dst;
        dst = t;
    }
}

}  // namespace acq
