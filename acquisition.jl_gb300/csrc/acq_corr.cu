// acq_corr.cu — continuous correlator of the fine search: power, closed-form gradient and
// Hessian, batched Newton refinement, and the adjoint with respect to the input samples.
//
// Model (declared in acqgb300.h). For samples x[n], n = 0..N-1, at rate fs and intermediate
// frequency IF, and a cell (PRN, code phase tau in chips at sample 0, Doppler f in Hz):
//   phi_n   = tau + n rho(f),           rho(f) = (f_code + f f_code / f_carrier) / fs
//   theta_n = 2 pi (IF + f) n / fs
//   z       = sum_n x[n] c(phi_n) exp(-i theta_n),          P = |z|^2
// which is the correlation of the signal model of src/generate_test_signal.jl:45-68 (code
// sampled at the Doppler-shifted code rate, carrier exp(+i theta)). The replica c is the code
// table (M entries per chip: M = 2 half chips for BOC(1,1), else 1; the secondary code folded
// in) smoothed by the quadratic B-spline centred on each entry:
//   c(phi) = S(M phi),  S(psi) = sum_j tab[j] B2(psi - j - 1/2).
// With j = floor(psi), t = psi - j - 1/2 and a, b, d = tab[j-1], tab[j], tab[j+1]:
//   S = alpha + t (beta + gamma t),  S' = beta + 2 gamma t,  S'' = 2 gamma,
//   alpha = (a + 6b + d)/8, beta = (d - a)/2, gamma = (a - 2b + d)/2.
//
// Derivatives (kappa = f_code / (f_carrier fs), beta_c = 2 pi / fs; sums over n of
// y_n = x[n] exp(-i theta_n) times S_k = S, S', S'' at psi_n, weighted by 1, n, n^2:
// S_k, T_k, U_k):
//   z     = S_0                     z_tau   = M S_1                  z_tt = M^2 S_2
//   z_f   = M kappa T_1 - i beta_c T_0
//   z_tf  = M^2 kappa T_2 - i beta_c M T_1
//   z_ff  = M^2 kappa^2 U_2 - 2 i beta_c kappa M U_1 - beta_c^2 U_0
//   dP/dv = 2 Re(conj(z) z_v),   d2P/dv dw = 2 Re(conj(z_v) z_w + conj(z) z_vw).
//
// Arithmetic. The table position psi / L_t and the carrier phase in cycles run as 0.64
// fixed-point integers (exact, wrapping modulo one table period and one cycle), so phases
// stay exact over long recordings. The per-sample sums run in FP32 with n centred on N/2
// (recombined exactly in FP64); the carrier phasor advances by an FP32 recurrence reseeded
// from the exact phase every kReseed steps. Power, gradient and Hessian are formed in FP64
// from the reduced FP32 sums.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "acq_host.h"
#include "acqgb300.h"

struct acq_corr {
    int system = 0;
    double fs = 0.0, f_code = 0.0, f_carrier = 0.0;
    int M = 1;           // table entries per chip
    int Lt = 0;          // table entries per period (primary x secondary x M)
    std::vector<int> prns;
    uint8_t* d_codes = nullptr;   // n_prns x Lt spline codes (bit0 a<0, bit1 b<0, bit2 d<0)
    int* d_slot = nullptr;        // PRN -> table offset, -1 when absent (max_prn + 1 entries)
    int max_prn = 0;
    float* d_partial = nullptr;   // VJP partial sums
    size_t partial_bytes = 0;
    ~acq_corr() {
        if (d_codes) cudaFree(d_codes);
        if (d_slot) cudaFree(d_slot);
        if (d_partial) cudaFree(d_partial);
    }
};

namespace {

using acq::AcqError;

#define CKC(x)                                                                                          \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess)                                                                          \
            throw AcqError(ACQ_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorName(e_) + " " +          \
                                             cudaGetErrorString(e_));                                   \
    } while (0)

constexpr int kThreads = 256;     // samples per block step
constexpr int kCells = 2;         // cells per block (eval / refine)
constexpr int kReseed = 16;       // carrier recurrence steps between exact reseeds
constexpr int kVjpSpt = 16;       // samples per thread (VJP)
constexpr int kVjpCells = 2048;   // cells per VJP block row
constexpr int kVjpTile = 256;     // cells staged in shared memory at a time
constexpr int kMaxSamples = 1 << 24;   // sample indices stay exact in FP32

struct CorrConsts {
    const uint8_t* codes;
    const int* slot;
    int max_prn;
    int Lt;
    int M;
    double fs, f_code, f_carrier, interm_freq;
};

// Per-cell fixed-point stepping parameters.
struct CellStep {
    uint64_t u0, du, du_step;     // table position / Lt: at sample 0, per sample, per block step
    uint64_t dv, dv_step;         // carrier cycles per sample, per block step
    float2 w_step;                // exp(-i 2 pi dv_step) in FP32
    int table;                    // offset of the PRN's table, -1 when the PRN is absent
};

__host__ __device__ inline uint64_t frac_u64(double x) {
    const double f = x - floor(x);
    const double s = f * 18446744073709551616.0;   // 2^64
    if (!(s < 18446744073709551616.0)) return 0ULL;
    return static_cast<uint64_t>(s);
}

__device__ inline CellStep cell_step(const CorrConsts& k, int prn, double tau, double f) {
    CellStep s;
    s.table = (prn >= 1 && prn <= k.max_prn) ? k.slot[prn] : -1;
    const double rho = (k.f_code + f * k.f_code / k.f_carrier) / k.fs;
    s.u0 = frac_u64(static_cast<double>(k.M) * tau / k.Lt);
    s.du = frac_u64(static_cast<double>(k.M) * rho / k.Lt);
    s.du_step = s.du * static_cast<uint64_t>(kThreads);
    s.dv = frac_u64((k.interm_freq + f) / k.fs);
    s.dv_step = s.dv * static_cast<uint64_t>(kThreads);
    const double cyc = static_cast<double>(static_cast<int64_t>(s.dv_step)) * 5.421010862427522e-20;   // 2^-64
    double sn, cs;
    sincospi(2.0 * cyc, &sn, &cs);
    s.w_step = make_float2(static_cast<float>(cs), static_cast<float>(-sn));
    return s;
}

// exp(-i 2 pi v / 2^64) in FP32 (v read as a signed fraction of a cycle, |arg| <= pi)
__device__ __forceinline__ float2 carrier(uint64_t v) {
    const float cyc = static_cast<float>(static_cast<int64_t>(v)) * 5.421010862e-20f;
    float sn, cs;
    sincospif(2.0f * cyc, &sn, &cs);
    return make_float2(cs, -sn);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// table entry index and fraction of psi for position u (0.64 fixed point of psi / Lt)
__device__ __forceinline__ int table_pos(uint64_t u, uint32_t Lt, float* frac) {
    const uint32_t uh = static_cast<uint32_t>(u >> 32), ul = static_cast<uint32_t>(u);
    const uint64_t s = static_cast<uint64_t>(uh) * Lt + ((static_cast<uint64_t>(ul) * Lt) >> 32);
    *frac = __uint2float_rn(static_cast<uint32_t>(s)) * 2.3283064365386963e-10f;   // 2^-32
    return static_cast<int>(s >> 32);
}

template <int DT>
__device__ __forceinline__ float2 load_x(const void* x, int64_t i) {
    if (DT == ACQ_CF32) return __ldg(reinterpret_cast<const float2*>(x) + i);
    if (DT == ACQ_CI16) {
        const short2 v = __ldg(reinterpret_cast<const short2*>(x) + i);
        return make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
    }
    if (DT == ACQ_CI8) {
        const char2 v = __ldg(reinterpret_cast<const char2*>(x) + i);
        return make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
    }
    const double2 v = __ldg(reinterpret_cast<const double2*>(x) + i);
    return make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
}

__device__ __forceinline__ void load_coefs(float4* coef) {
    if (threadIdx.x < 8) {
        const int k = threadIdx.x;
        const float a = (k & 1) ? -1.f : 1.f, b = (k & 2) ? -1.f : 1.f, d = (k & 4) ? -1.f : 1.f;
        const float g = 0.5f * (a - 2.f * b + d);
        coef[k] = make_float4(0.125f * (a + 6.f * b + d), 0.5f * (d - a), g, 2.f * g);
    }
}

constexpr int kAcc = 18;   // S0,S1,S2,T0,T1,T2,U0,U1,U2 (re, im)

struct CellEval {
    double P, gt, gf, htt, htf, hff, zr, zi;
};

// FP64 power / gradient / Hessian from the reduced sums (n centred on nc).
__device__ CellEval finish(const double* a, double nc, const CorrConsts& k, bool hess) {
    struct C {
        double r, i;
    };
    auto mk = [&](int q) { return C{a[2 * q], a[2 * q + 1]}; };
    C S0 = mk(0), S1 = mk(1), S2 = mk(2), T0 = mk(3), T1 = mk(4), T2 = mk(5), U0 = mk(6), U1 = mk(7), U2 = mk(8);
    // uncentre: sum n y = T' + nc S, sum n^2 y = U' + 2 nc T' + nc^2 S
    auto add = [](C p, C q, double s) { return C{p.r + s * q.r, p.i + s * q.i}; };
    C V0 = add(add(U0, T0, 2.0 * nc), S0, nc * nc), V1 = add(add(U1, T1, 2.0 * nc), S1, nc * nc),
      V2 = add(add(U2, T2, 2.0 * nc), S2, nc * nc);
    T0 = add(T0, S0, nc);
    T1 = add(T1, S1, nc);
    T2 = add(T2, S2, nc);
    const double M = k.M, kap = k.f_code / (k.f_carrier * k.fs), bc = 6.283185307179586 / k.fs;
    const C z = S0;
    const C zt{M * S1.r, M * S1.i};
    // -i beta T = (beta T.i, -beta T.r)
    const C zf{M * kap * T1.r + bc * T0.i, M * kap * T1.i - bc * T0.r};
    auto re_conj = [](C p, C q) { return p.r * q.r + p.i * q.i; };   // Re(conj(p) q)
    CellEval e{};
    e.zr = z.r;
    e.zi = z.i;
    e.P = z.r * z.r + z.i * z.i;
    e.gt = 2.0 * re_conj(z, zt);
    e.gf = 2.0 * re_conj(z, zf);
    if (hess) {
        const C ztt{M * M * S2.r, M * M * S2.i};
        const C ztf{M * M * kap * T2.r + bc * M * T1.i, M * M * kap * T2.i - bc * M * T1.r};
        const C zff{M * M * kap * kap * V2.r + 2.0 * bc * kap * M * V1.i - bc * bc * V0.r,
                    M * M * kap * kap * V2.i - 2.0 * bc * kap * M * V1.r - bc * bc * V0.i};
        e.htt = 2.0 * (re_conj(zt, zt) + re_conj(z, ztt));
        e.htf = 2.0 * (re_conj(zt, zf) + re_conj(z, ztf));
        e.hff = 2.0 * (re_conj(zf, zf) + re_conj(z, zff));
    }
    return e;
}

struct RefineArgs {
    int max_iter;        // 0: evaluate once
    double tol_t, tol_f, step_t, step_f;
};

// One block: kCells cells, all samples. Evaluates (refine: iterates Newton steps).
template <int DT, bool HESS>
__global__ void __launch_bounds__(kThreads) k_corr(const void* __restrict__ x, int64_t n, CorrConsts k,
                                                   acq_corr_cell* __restrict__ cells, int n_cells, RefineArgs ra,
                                                   acq_corr_result* __restrict__ out) {
    __shared__ float4 coef[8];
    __shared__ CellStep cs[kCells];
    __shared__ int active[kCells];
    __shared__ float red[kCells][kThreads / 32][kAcc];
    __shared__ double sums[kCells][kAcc];
    __shared__ double cur_t[kCells], cur_f[kCells];
    __shared__ double prv_t[kCells], prv_f[kCells], stp_t[kCells], stp_f[kCells];
    __shared__ CellEval prv_e[kCells];
    __shared__ int iters[kCells];
    __shared__ int any_active;
    load_coefs(coef);
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
    const int c0 = blockIdx.x * kCells;
    if (tid < kCells) {
        const int ci = c0 + tid;
        active[tid] = ci < n_cells;
        iters[tid] = 0;
        if (ci < n_cells) {
            cur_t[tid] = cells[ci].code_phase;
            cur_f[tid] = cells[ci].doppler_hz;
        }
    }
    const float nc = static_cast<float>(n / 2);
    const uint32_t Lt = static_cast<uint32_t>(k.Lt);
    for (int round = 0;; ++round) {
        __syncthreads();
        if (tid < kCells) {
            const int ci = c0 + tid;
            if (active[tid]) {
                cs[tid] = cell_step(k, cells[ci].prn, cur_t[tid], cur_f[tid]);
                if (cs[tid].table < 0) {
                    acq_corr_result o{};
                    o.status = ACQ_CORR_BAD_PRN;
                    out[ci] = o;
                    active[tid] = 0;
                }
            }
        }
        if (tid == 0) {
            int a = 0;
            for (int c = 0; c < kCells; ++c) a |= active[c];
            any_active = a;
        }
        __syncthreads();
        if (!any_active) break;
        float acc[kCells][kAcc];
        uint64_t u[kCells], v[kCells];
        CellStep sc[kCells];
        bool act[kCells];
#pragma unroll
        for (int c = 0; c < kCells; ++c) {
#pragma unroll
            for (int q = 0; q < kAcc; ++q) acc[c][q] = 0.f;
            sc[c] = cs[c];
            act[c] = active[c] != 0;
            u[c] = sc[c].u0 + static_cast<uint64_t>(tid) * sc[c].du;
            v[c] = static_cast<uint64_t>(tid) * sc[c].dv;
        }
        for (int64_t base = 0; base < n; base += static_cast<int64_t>(kThreads) * kReseed) {
            float2 e[kCells];
            // n^2-weighted sums span the widest range: accumulate them per group, then fold in
            float ug[kCells][6];
#pragma unroll
            for (int c = 0; c < kCells; ++c) {
                e[c] = carrier(v[c]);
#pragma unroll
                for (int q = 0; q < 6; ++q) ug[c][q] = 0.f;
            }
            for (int r = 0; r < kReseed; ++r) {
                const int64_t i = base + static_cast<int64_t>(r) * kThreads + tid;
                if (i >= n) break;
                const float2 xs = load_x<DT>(x, i);
                const float nf = static_cast<float>(i) - nc;
#pragma unroll
                for (int c = 0; c < kCells; ++c) {
                    if (act[c]) {
                        float fr;
                        const int j = table_pos(u[c], Lt, &fr);
                        const float4 q = coef[__ldg(k.codes + sc[c].table + j)];
                        const float t = fr - 0.5f;
                        const float S = fmaf(t, fmaf(q.z, t, q.y), q.x);
                        const float S1 = fmaf(q.w, t, q.y);
                        const float2 y = cmulf(xs, e[c]);
                        float* a = acc[c];
                        a[0] = fmaf(y.x, S, a[0]);
                        a[1] = fmaf(y.y, S, a[1]);
                        a[2] = fmaf(y.x, S1, a[2]);
                        a[3] = fmaf(y.y, S1, a[3]);
                        const float2 yn = make_float2(y.x * nf, y.y * nf);
                        a[6] = fmaf(yn.x, S, a[6]);
                        a[7] = fmaf(yn.y, S, a[7]);
                        a[8] = fmaf(yn.x, S1, a[8]);
                        a[9] = fmaf(yn.y, S1, a[9]);
                        if (HESS) {
                            const float S2 = q.w;
                            a[4] = fmaf(y.x, S2, a[4]);
                            a[5] = fmaf(y.y, S2, a[5]);
                            a[10] = fmaf(yn.x, S2, a[10]);
                            a[11] = fmaf(yn.y, S2, a[11]);
                            const float2 ynn = make_float2(yn.x * nf, yn.y * nf);
                            float* g = ug[c];
                            g[0] = fmaf(ynn.x, S, g[0]);
                            g[1] = fmaf(ynn.y, S, g[1]);
                            g[2] = fmaf(ynn.x, S1, g[2]);
                            g[3] = fmaf(ynn.y, S1, g[3]);
                            g[4] = fmaf(ynn.x, S2, g[4]);
                            g[5] = fmaf(ynn.y, S2, g[5]);
                        }
                    }
                    u[c] += sc[c].du_step;
                    v[c] += sc[c].dv_step;
                    e[c] = cmulf(e[c], sc[c].w_step);
                }
            }
            if (HESS) {
#pragma unroll
                for (int c = 0; c < kCells; ++c)
#pragma unroll
                    for (int q = 0; q < 6; ++q) acc[c][12 + q] += ug[c][q];
            }
        }
        // block reduction: warp shuffles, then FP64 over warps
#pragma unroll
        for (int c = 0; c < kCells; ++c) {
#pragma unroll
            for (int q = 0; q < kAcc; ++q) {
                float s = acc[c][q];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) red[c][wp][q] = s;
            }
        }
        __syncthreads();
        if (tid < kCells * kAcc) {
            const int c = tid / kAcc, q = tid - (tid / kAcc) * kAcc;
            double s = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) s += static_cast<double>(red[c][w][q]);
            sums[c][q] = s;
        }
        __syncthreads();
        if (tid < kCells && active[tid]) {
            const int c = tid, ci = c0 + tid;
            const CellEval E = finish(sums[c], static_cast<double>(nc), k, HESS);
            bool done = false;
            CellEval R = E;
            double rt = cur_t[c], rf = cur_f[c];
            int st = ACQ_CORR_OK;
            if (ra.max_iter <= 0) {
                done = true;
            } else if (iters[c] > 0 && E.P < prv_e[c].P) {
                // power dropped: halve the step from the last accepted point
                stp_t[c] *= 0.5;
                stp_f[c] *= 0.5;
                if (fabs(stp_t[c]) < ra.tol_t && fabs(stp_f[c]) < ra.tol_f) {
                    done = true;
                    R = prv_e[c];
                    rt = prv_t[c];
                    rf = prv_f[c];
                } else {
                    cur_t[c] = prv_t[c] + stp_t[c];
                    cur_f[c] = prv_f[c] + stp_f[c];
                }
            } else {
                prv_e[c] = E;
                prv_t[c] = cur_t[c];
                prv_f[c] = cur_f[c];
                double dt, df;
                const double det = E.htt * E.hff - E.htf * E.htf;
                if (E.htt < 0.0 && det > 0.0) {   // Newton step towards the maximum
                    dt = -(E.hff * E.gt - E.htf * E.gf) / det;
                    df = -(-E.htf * E.gt + E.htt * E.gf) / det;
                } else {                           // scaled gradient ascent to the trust-region edge
                    const double a = E.gt * ra.step_t, b = E.gf * ra.step_f;
                    const double nrm = sqrt(a * a + b * b);
                    dt = nrm > 0.0 ? ra.step_t * a / nrm : 0.0;
                    df = nrm > 0.0 ? ra.step_f * b / nrm : 0.0;
                }
                double sc = 1.0;
                if (fabs(dt) > ra.step_t) sc = fmin(sc, ra.step_t / fabs(dt));
                if (fabs(df) > ra.step_f) sc = fmin(sc, ra.step_f / fabs(df));
                dt *= sc;
                df *= sc;
                if (fabs(dt) < ra.tol_t && fabs(df) < ra.tol_f) {
                    done = true;
                } else {
                    stp_t[c] = dt;
                    stp_f[c] = df;
                    cur_t[c] += dt;
                    cur_f[c] += df;
                }
            }
            if (!done && ra.max_iter > 0 && iters[c] + 1 >= ra.max_iter) {
                done = true;
                st = ACQ_CORR_NOT_CONVERGED;
                R = prv_e[c];
                rt = prv_t[c];
                rf = prv_f[c];
            }
            if (ra.max_iter > 0) iters[c] += 1;
            if (done) {
                acq_corr_result o;
                o.power = R.P;
                o.grad[0] = R.gt;
                o.grad[1] = R.gf;
                o.hess[0] = R.htt;
                o.hess[1] = R.htf;
                o.hess[2] = R.hff;
                o.z_re = R.zr;
                o.z_im = R.zi;
                o.iterations = ra.max_iter > 0 ? iters[c] : 0;
                o.status = st;
                out[ci] = o;
                if (ra.max_iter > 0) {
                    cells[ci].code_phase = rt;
                    cells[ci].doppler_hz = rf;
                }
                active[c] = 0;
            }
        }
    }
}

// Adjoint: partial[y][n] = sum over this block row's cells of zbar_c S(psi_{c,n}) exp(+i theta_{c,n}).
__global__ void __launch_bounds__(kThreads) k_corr_vjp(int64_t n, CorrConsts k, const acq_corr_cell* __restrict__ cells,
                                                       const float2* __restrict__ zbar, int n_cells,
                                                       float2* __restrict__ partial) {
    __shared__ float4 coef[8];
    __shared__ CellStep cs[kVjpTile];
    __shared__ float2 wz[kVjpTile];
    load_coefs(coef);
    const int tid = threadIdx.x;
    const int64_t x0 = static_cast<int64_t>(blockIdx.x) * kThreads * kVjpSpt;
    const int64_t n_first = x0 + tid;
    const int cbeg = blockIdx.y * kVjpCells, cend = min(n_cells, cbeg + kVjpCells);
    const uint32_t Lt = static_cast<uint32_t>(k.Lt);
    float2 acc[kVjpSpt];
#pragma unroll
    for (int j = 0; j < kVjpSpt; ++j) acc[j] = make_float2(0.f, 0.f);
    for (int tb = cbeg; tb < cend; tb += kVjpTile) {
        const int nt = min(kVjpTile, cend - tb);
        __syncthreads();
        if (tid < nt) {
            const acq_corr_cell cl = cells[tb + tid];
            cs[tid] = cell_step(k, cl.prn, cl.code_phase, cl.doppler_hz);
            wz[tid] = zbar[tb + tid];
        }
        __syncthreads();
        for (int c = 0; c < nt; ++c) {
            const CellStep s = cs[c];
            if (s.table < 0) continue;
            const float2 w = wz[c];
            uint64_t u = s.u0 + static_cast<uint64_t>(n_first) * s.du;
            const uint64_t v = static_cast<uint64_t>(n_first) * s.dv;
            float2 e = carrier(v);
            e.y = -e.y;                                   // exp(+i theta)
            const float2 ws = make_float2(s.w_step.x, -s.w_step.y);
#pragma unroll
            for (int j = 0; j < kVjpSpt; ++j) {
                float fr;
                const int jj = table_pos(u, Lt, &fr);
                const float4 q = coef[__ldg(k.codes + s.table + jj)];
                const float t = fr - 0.5f;
                const float S = fmaf(t, fmaf(q.z, t, q.y), q.x);
                const float2 we = cmulf(w, e);
                acc[j].x = fmaf(we.x, S, acc[j].x);
                acc[j].y = fmaf(we.y, S, acc[j].y);
                u += s.du_step;
                e = cmulf(e, ws);
            }
        }
    }
    float2* pp = partial + static_cast<int64_t>(blockIdx.y) * n;
#pragma unroll
    for (int j = 0; j < kVjpSpt; ++j) {
        const int64_t i = n_first + static_cast<int64_t>(j) * kThreads;
        if (i < n) pp[i] = acc[j];
    }
}

__global__ void k_corr_vjp_sum(int64_t n, int rows, const float2* __restrict__ partial, float2* __restrict__ xbar) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int r = 0; r < rows; ++r) {
            const float2 p = partial[static_cast<int64_t>(r) * n + i];
            re += p.x;
            im += p.y;
        }
        xbar[i] = make_float2(static_cast<float>(re), static_cast<float>(im));
    }
}

template <typename F>
int guarded_corr(F&& f) {
    try {
        f();
        return ACQ_OK;
    } catch (const AcqError& e) {
        acq::set_last_error(e.what());
        return e.status;
    } catch (const std::bad_alloc&) {
        acq::set_last_error("host allocation failed");
        return ACQ_ERR_ALLOC;
    } catch (const std::exception& e) {
        acq::set_last_error(e.what());
        return ACQ_ERR_CUDA;
    }
}

CorrConsts consts(const acq_corr* C, double interm_freq) {
    CorrConsts k;
    k.codes = C->d_codes;
    k.slot = C->d_slot;
    k.max_prn = C->max_prn;
    k.Lt = C->Lt;
    k.M = C->M;
    k.fs = C->fs;
    k.f_code = C->f_code;
    k.f_carrier = C->f_carrier;
    k.interm_freq = interm_freq;
    return k;
}

void check_samples(const void* d_samples, int32_t dtype, int64_t n) {
    if (!d_samples) throw AcqError(ACQ_ERR_ARGUMENT, "null samples");
    if (dtype < ACQ_CF32 || dtype > ACQ_CF64) throw AcqError(ACQ_ERR_ARGUMENT, "unknown sample dtype");
    if (n < 1 || n > kMaxSamples)
        throw AcqError(ACQ_ERR_ARGUMENT, "n_samples must be in 1:" + std::to_string(kMaxSamples));
}

template <bool HESS>
void launch_corr(acq_corr* C, const void* x, int32_t dtype, int64_t n, double fi, acq_corr_cell* cells, int n_cells,
                 const RefineArgs& ra, acq_corr_result* out, cudaStream_t st) {
    const CorrConsts k = consts(C, fi);
    const dim3 grid((n_cells + kCells - 1) / kCells);
    switch (dtype) {
        case ACQ_CF32: k_corr<ACQ_CF32, HESS><<<grid, kThreads, 0, st>>>(x, n, k, cells, n_cells, ra, out); break;
        case ACQ_CI16: k_corr<ACQ_CI16, HESS><<<grid, kThreads, 0, st>>>(x, n, k, cells, n_cells, ra, out); break;
        case ACQ_CI8: k_corr<ACQ_CI8, HESS><<<grid, kThreads, 0, st>>>(x, n, k, cells, n_cells, ra, out); break;
        default: k_corr<ACQ_CF64, HESS><<<grid, kThreads, 0, st>>>(x, n, k, cells, n_cells, ra, out); break;
    }
    CKC(cudaGetLastError());
}

}  // namespace

extern "C" {

int acq_corr_create(int32_t system, double fs, const int32_t* prns, int32_t n_prns, const int8_t* codes,
                    acq_corr** out) {
    return guarded_corr([&] {
        if (!out || (!prns && n_prns > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        if (n_prns <= 0) throw AcqError(ACQ_ERR_ARGUMENT, "prns must not be empty");
        if (!(fs > 0.0) || !std::isfinite(fs)) throw AcqError(ACQ_ERR_ARGUMENT, "sampling frequency must be positive");
        const acq::SystemInfo& s = acq::system_info(system);
        std::unique_ptr<acq_corr> C(new acq_corr());
        C->system = system;
        C->fs = fs;
        C->f_code = s.code_freq;
        C->f_carrier = s.center_freq;
        C->M = s.boc11 ? 2 : 1;
        C->max_prn = s.max_prn;
        const int L = s.code_length * s.secondary_length;
        C->Lt = L * C->M;
        std::vector<int> slot(s.max_prn + 1, -1);
        std::vector<uint8_t> tab(static_cast<size_t>(n_prns) * C->Lt);
        for (int i = 0; i < n_prns; ++i) {
            const int prn = prns[i];
            if (prn < 1 || prn > s.max_prn)
                throw AcqError(ACQ_ERR_ARGUMENT, std::string(s.name) + " PRN must be in 1:" +
                                                     std::to_string(s.max_prn) + ", got " + std::to_string(prn));
            if (slot[prn] >= 0) throw AcqError(ACQ_ERR_ARGUMENT, "duplicate PRN " + std::to_string(prn));
            std::vector<int8_t> full;
            if (codes) {
                const int8_t* p = codes + static_cast<size_t>(i) * s.code_length;
                full.resize(L);
                for (int k = 0; k < s.secondary_length; ++k)
                    for (int c = 0; c < s.code_length; ++c)
                        full[static_cast<size_t>(k) * s.code_length + c] =
                            static_cast<int8_t>(p[c] * (s.secondary_length > 1 ? s.secondary[k] : 1));
            } else {
                full = acq::full_chips(system, prn);
            }
            std::vector<int8_t> e(C->Lt);
            for (int c = 0; c < L; ++c) {
                if (C->M == 2) {
                    e[2 * c] = full[c];
                    e[2 * c + 1] = static_cast<int8_t>(-full[c]);
                } else {
                    e[c] = full[c];
                }
            }
            uint8_t* t = &tab[static_cast<size_t>(i) * C->Lt];
            for (int j = 0; j < C->Lt; ++j) {
                const int8_t a = e[(j + C->Lt - 1) % C->Lt], b = e[j], d = e[(j + 1) % C->Lt];
                t[j] = static_cast<uint8_t>((a < 0 ? 1 : 0) | (b < 0 ? 2 : 0) | (d < 0 ? 4 : 0));
            }
            slot[prn] = i * C->Lt;
            C->prns.push_back(prn);
        }
        CKC(cudaMalloc(&C->d_codes, tab.size()));
        CKC(cudaMemcpy(C->d_codes, tab.data(), tab.size(), cudaMemcpyHostToDevice));
        CKC(cudaMalloc(&C->d_slot, sizeof(int) * slot.size()));
        CKC(cudaMemcpy(C->d_slot, slot.data(), sizeof(int) * slot.size(), cudaMemcpyHostToDevice));
        *out = C.release();
    });
}

int acq_corr_destroy(acq_corr* C) {
    return guarded_corr([&] { delete C; });
}

int acq_corr_eval(acq_corr* C, const void* d_samples, int32_t dtype, int64_t n, double fi, const acq_corr_cell* d_cells,
                  int32_t n_cells, int32_t want_hessian, acq_corr_result* d_out, void* stream) {
    return guarded_corr([&] {
        if (!C || !d_out || (!d_cells && n_cells > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        check_samples(d_samples, dtype, n);
        if (n_cells <= 0) return;
        RefineArgs ra{0, 0.0, 0.0, 0.0, 0.0};
        auto* cells = const_cast<acq_corr_cell*>(d_cells);   // not written when max_iter == 0
        if (want_hessian)
            launch_corr<true>(C, d_samples, dtype, n, fi, cells, n_cells, ra, d_out, static_cast<cudaStream_t>(stream));
        else
            launch_corr<false>(C, d_samples, dtype, n, fi, cells, n_cells, ra, d_out, static_cast<cudaStream_t>(stream));
    });
}

int acq_corr_refine(acq_corr* C, const void* d_samples, int32_t dtype, int64_t n, double fi, acq_corr_cell* d_cells,
                    int32_t n_cells, int32_t max_iterations, double tol_chips, double tol_hz, double max_step_chips,
                    double max_step_hz, acq_corr_result* d_out, void* stream) {
    return guarded_corr([&] {
        if (!C || !d_out || (!d_cells && n_cells > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        check_samples(d_samples, dtype, n);
        if (max_iterations < 1) throw AcqError(ACQ_ERR_ARGUMENT, "max_iterations must be >= 1");
        if (!(tol_chips > 0) || !(tol_hz > 0) || !(max_step_chips > 0) || !(max_step_hz > 0))
            throw AcqError(ACQ_ERR_ARGUMENT, "tolerances and step bounds must be positive");
        if (n_cells <= 0) return;
        RefineArgs ra{max_iterations, tol_chips, tol_hz, max_step_chips, max_step_hz};
        launch_corr<true>(C, d_samples, dtype, n, fi, d_cells, n_cells, ra, d_out, static_cast<cudaStream_t>(stream));
    });
}

int acq_corr_vjp_samples(acq_corr* C, int64_t n, double fi, const acq_corr_cell* d_cells, const float* d_zbar,
                         int32_t n_cells, float* d_xbar, void* stream) {
    return guarded_corr([&] {
        if (!C || !d_xbar || ((!d_cells || !d_zbar) && n_cells > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (n < 1 || n > kMaxSamples)
            throw AcqError(ACQ_ERR_ARGUMENT, "n_samples must be in 1:" + std::to_string(kMaxSamples));
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (n_cells <= 0) {
            CKC(cudaMemsetAsync(d_xbar, 0, sizeof(float) * 2 * n, st));
            return;
        }
        const int rows = (n_cells + kVjpCells - 1) / kVjpCells;
        const size_t need = sizeof(float2) * static_cast<size_t>(rows) * n;
        if (need > C->partial_bytes) {
            CKC(cudaStreamSynchronize(st));
            if (C->d_partial) cudaFree(C->d_partial);
            C->d_partial = nullptr;
            C->partial_bytes = 0;
            CKC(cudaMalloc(&C->d_partial, need));
            C->partial_bytes = need;
        }
        const CorrConsts k = consts(C, fi);
        const dim3 grid(static_cast<unsigned>((n + kThreads * kVjpSpt - 1) / (kThreads * kVjpSpt)), rows);
        k_corr_vjp<<<grid, kThreads, 0, st>>>(n, k, d_cells, reinterpret_cast<const float2*>(d_zbar), n_cells,
                                             reinterpret_cast<float2*>(C->d_partial));
        CKC(cudaGetLastError());
        k_corr_vjp_sum<<<std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(
            n, rows, reinterpret_cast<const float2*>(C->d_partial), reinterpret_cast<float2*>(d_xbar));
        CKC(cudaGetLastError());
    });
}

}  // extern "C"
