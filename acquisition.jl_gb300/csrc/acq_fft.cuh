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

#include <type_traits>

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

// Complex add, subtract and real scale as packed two-lane FP32 instructions (add/sub/mul.rn.f32x2
// of sm_100-family GPUs): the same IEEE round-to-nearest result per component as two scalar
// operations, in one issue slot.
__device__ __forceinline__ float2 c_add(float2 a, float2 b) {
    float2 r;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) {
    float2 r;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 c_scale(float2 a, float s) {
    float2 r;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %4};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(s));
    return r;
}
// a + s * y with one rounding per component (packed fused multiply-add)
__device__ __forceinline__ float2 c_axpy(float s, float2 y, float2 a) {
    float2 r;
    asm("{.reg .b64 rs, ry, ra, rd;\n\tmov.b64 rs, {%2, %2};\n\tmov.b64 ry, {%3, %4};\n\t"
        "mov.b64 ra, {%5, %6};\n\tfma.rn.f32x2 rd, rs, ry, ra;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(s), "f"(y.x), "f"(y.y), "f"(a.x), "f"(a.y));
    return r;
}
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


// ======================================================================================
// Register FFTs and the two-pass (four-step) shared-memory FFT for hot sizes.
//
// RegFFT<N> runs an N-point DFT on N values held in registers, fully unrolled: split
// N = P * M with P the first of 4, 2, 3, 5, 7 dividing N; P-point DFTs on the strided
// elements, twiddles W_N^{m k} from constant memory at compile-time indices, then M-point
// DFTs recursively on contiguous sub-blocks. The output is in a compile-time permutation
// (reg_perm<N>(f) is the register holding X[f]).
//
// FourStep<N1, N2>: N = N1 * N2 points in shared memory. Pass 1 (one task per n2): DFT_N1 over
// x[n2 + N2 n1], multiply by W_N^{n2 k1}, store in place. Pass 2 (one task per k1): DFT_N2 over
// the contiguous y[N2 k1 + n2] gives X[k1 + N1 k2].
// ======================================================================================

constexpr int kRegTwMax = 64;  // register-FFT sizes 2..64 have constant twiddle tables
__host__ __device__ constexpr int reg_tw_offset(int n) { return (n - 1) * n / 2 - 1; }  // sum_{k=2}^{n-1} k
constexpr int kRegTwEntries = reg_tw_offset(kRegTwMax + 1);
// One copy per translation unit (no relocatable device code): every unit that instantiates
// register FFTs uploads it through its own acq_inst_*_upload_twiddles().
static __constant__ float2 c_regtw[kRegTwEntries];  // W_n^e = exp(-2 pi i e / n)

__host__ __device__ constexpr int first_factor(int n) {
    return n % 4 == 0 ? 4 : n % 2 == 0 ? 2 : n % 3 == 0 ? 3 : n % 5 == 0 ? 5 : n % 7 == 0 ? 7 : n;
}

__host__ __device__ constexpr int reg_perm(int n, int f) {
    // register index holding X[f] after RegFFT<n>
    return (first_factor(n) == n) ? f
                                  : (f % first_factor(n)) * (n / first_factor(n)) +
                                        reg_perm(n / first_factor(n), f / first_factor(n));
}

// Compile-time loop: f(std::integral_constant<int, I>) for I in [B, E).
template <int B, int E, typename Fn>
__device__ __forceinline__ void static_for(Fn&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

template <int P, bool INV>
__device__ __forceinline__ void base_dft(float2* v) {
    if constexpr (P == 2) bf2<INV>(v);
    else if constexpr (P == 3) bf3<INV>(v);
    else if constexpr (P == 4) bf4<INV>(v);
    else if constexpr (P == 5) bf5<INV>(v);
    else {
        float2 o[P];
#pragma unroll
        for (int t = 0; t < P; ++t) {
            float2 acc = v[0];
#pragma unroll
            for (int q = 1; q < P; ++q) {
                float2 w = c_regtw[reg_tw_offset(P) + (q * t) % P];
                if (INV) w.y = -w.y;
                acc = c_add(acc, c_mul(v[q], w));
            }
            o[t] = acc;
        }
#pragma unroll
        for (int t = 0; t < P; ++t) v[t] = o[t];
    }
}

template <int N, bool INV>
struct RegFFT {
    static constexpr int P = first_factor(N);
    static constexpr int M = N / P;
    __device__ __forceinline__ static void run(float2* v) {
        if constexpr (M == 1) {
            base_dft<P, INV>(v);
        } else {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                float2 t[P];
#pragma unroll
                for (int p = 0; p < P; ++p) t[p] = v[m + M * p];
                base_dft<P, INV>(t);
#pragma unroll
                for (int k = 0; k < P; ++k) {
                    float2 x = t[k];
                    if (m * k != 0) {
                        float2 w = c_regtw[reg_tw_offset(N) + m * k];
                        if (INV) w.y = -w.y;
                        x = c_mul(x, w);
                    }
                    v[m + M * k] = x;
                }
            }
#pragma unroll
            for (int k = 0; k < P; ++k) RegFFT<M, INV>::run(v + k * M);
        }
    }
};

__host__ __device__ constexpr int best_split_n1(int n) {
    // largest divisor d <= sqrt(n) with n / d <= 64; 0 when none
    int best = 0;
    for (int d = 2; d * d <= n; ++d)
        if (n % d == 0 && n / d <= 64) best = d;
    return best;
}

// Pass 1 of the four-step FFT for one (vector, n2): in-place on shared memory `x` with element
// stride ES. `tw` is the N-point table exp(-2 pi i e / N) (global, read through L1).
template <int N1, int N2, bool INV>
__device__ __forceinline__ void fourstep_pass1(float2* x, int es, int n2, const float2* __restrict__ tw) {
    constexpr int N = N1 * N2;
    float2 v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = x[(n2 + N2 * n1) * es];
    RegFFT<N1, INV>::run(v);
    static_for<0, N1>([&](auto kc) {
        constexpr int k1 = decltype(kc)::value;
        constexpr int pr = reg_perm(N1, k1);
        float2 y = v[pr];
        if (k1 != 0 && n2 != 0) y = c_mul(y, tw_load<INV>(tw, n2 * k1));
        x[(n2 + N2 * k1) * es] = y;
    });
    (void)N;
}

}  // namespace acq
