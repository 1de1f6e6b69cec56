// acq_runtime.cu — plan lifetime, device memory, launch sequence and the C ABI of
// libacqgb300. Host logic mirrors plan_acquire / acquire! (src/plan.jl:312-697,
// src/acquire.jl:54-215); all per-sample work runs in the kernels of acq_kernels.cuh.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "acq_host.h"
#include "acq_inst.h"
#include "acq_mma.cuh"
#include "acq_kernels.cuh"
#include "acq_tile_mma.cuh"

using namespace acq;

ACQ_BC_SET_TABLE_IMPL(acq_bounds_set_table_runtime)

namespace {
std::mutex g_name_mu;
std::unordered_map<const void*, const char*>& name_table() {
    static std::unordered_map<const void*, const char*> t;
    return t;
}
}  // namespace

void acq::note_kernel_name(const void* fn, const char* name) {
    std::lock_guard<std::mutex> lk(g_name_mu);
    name_table()[fn] = name;
}

const char* acq::kernel_name(const void* fn) {
    std::lock_guard<std::mutex> lk(g_name_mu);
    auto it = name_table().find(fn);
    return it == name_table().end() ? nullptr : it->second;
}

namespace {

thread_local std::string g_last_error;

struct CudaError : AcqError {
    explicit CudaError(const std::string& m) : AcqError(ACQ_ERR_CUDA, m) {}
};

#define CK(x)                                                                                        \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess)                                                                       \
            throw CudaError(std::string(#x) + ": " + cudaGetErrorName(e_) + " " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int kThreads = 256;
constexpr size_t kSmemBudget = 200 * 1024;   // dynamic shared memory per CTA we plan for

// Sampled codes on the device with GNSSSignals gen_code semantics (the host restatement is
// acq::gen_code): sample i of PRN p takes chip floor(sp + i fc / fs) mod L of that PRN's table,
// negated in the second half of the chip for BOC(1,1). Whole fs and fc with sp = 0 use exact
// integer arithmetic; otherwise the FP64 phase is formed with explicit round-to-nearest
// multiply and add (no contraction), as on the host.
__global__ void k_sample_codes(const int8_t* __restrict__ chips, int64_t L, int n_prns, int64_t n, int64_t fci,
                               int64_t fsi, int whole, double sp, double ratio, int boc, int8_t* __restrict__ out) {
    const int64_t total = static_cast<int64_t>(n_prns) * n;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = k / n, i = k - p * n;
        int64_t idx;
        bool second;
        if (whole) {
            const int64_t num = i * fci;
            idx = num / fsi;
            second = 2 * (num - idx * fsi) >= fsi;
        } else {
            const double ph = __dadd_rn(sp, __dmul_rn(static_cast<double>(i), ratio));
            const double fl = floor(ph);
            idx = static_cast<int64_t>(fl);
            second = __dsub_rn(ph, fl) >= 0.5;
        }
        int8_t v = chips[p * L + ((idx % L) + L) % L];
        if (boc && second) v = static_cast<int8_t>(-v);
        out[k] = v;
    }
}

void sample_codes_device(int system, const int8_t* d_chips, int64_t L, int n_prns, int64_t n, double fs, double fc,
                         double start, int8_t* d_out, cudaStream_t st) {
    const SystemInfo& s = system_info(system);
    if (fc <= 0) fc = s.code_freq;
    double sp = std::fmod(start, static_cast<double>(L));
    if (sp < 0) sp += L;
    const int whole = (sp == 0.0 && is_whole_freq(fs) && is_whole_freq(fc)) ? 1 : 0;
    const int64_t total = static_cast<int64_t>(n_prns) * n;
    if (total <= 0) return;
    k_sample_codes<<<static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 16384)), 256, 0, st>>>(
        d_chips, L, n_prns, n, whole ? static_cast<int64_t>(fc) : 0, whole ? static_cast<int64_t>(fs) : 1, whole, sp,
        fc / fs, s.boc11 ? 1 : 0, d_out);
    CK(cudaGetLastError());
}

// Bounded-wait self test: an mbarrier that nothing arrives on; the wait must give up after
// `polls` polls and record code 9, leaving the context usable.
__global__ void k_wait_selftest(uint32_t polls, int* err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    mbar_wait_bounded(&bar, 0, err, 9, polls);
}

// out[r][i] = in[r][perm[i]] for rows of `width` columns (chip-sorted power surfaces)
__global__ void k_gather_cols(const float* __restrict__ in, int64_t rows, int64_t width, const int32_t* __restrict__ perm,
                              float* __restrict__ out) {
    const int64_t total = rows * width;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = k / width, i = k - r * width;
        out[k] = in[r * width + perm[i]];
    }
}

// Peak keys of the accumulator cells the Doppler-group column stage adds to atomically (the
// columns within H of a column-block boundary: multiples of W, and spc, wrapping to 0), whose
// final values exist only once that stage has finished. One CTA per (boundary, requested PRN);
// key j of the PRN's slots after `slot0`.
__global__ void k_edge_peaks(const float* __restrict__ acc, int ndop, int spc, int spc_eff, int W, int H, int n_bound,
                             int slot0, int npk, unsigned long long* __restrict__ peakpart) {
    __shared__ unsigned long long kred[8];
    pdl_trigger();
    pdl_wait();
    const int j = blockIdx.x, pi = blockIdx.y;
    const int b = j == n_bound - 1 ? spc : j * W;
    const float* ap = acc + static_cast<int64_t>(pi) * ndop * spc_eff;
    unsigned long long best = 0ULL;
    for (int i = threadIdx.x; i < ndop * 2 * H; i += blockDim.x) {
        const int r = i / (2 * H), o = i - r * 2 * H - H;
        int c = b + o;
        if (c < 0) c += spc;
        if (c >= spc) c -= spc;
        float v = 0.f;
        ACQ_BC(&ap[static_cast<int64_t>(r) * spc_eff + c], 20) v = ap[static_cast<int64_t>(r) * spc_eff + c];
        const unsigned long long key = peak_key(v, static_cast<uint32_t>(c) * ndop + r);
        best = key > best ? key : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other > best ? other : best;
    }
    if ((threadIdx.x & 31) == 0) kred[threadIdx.x / 32] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = kred[0];
        for (int w = 1; w < static_cast<int>(blockDim.x / 32); ++w) m = kred[w] > m ? kred[w] : m;
        ACQ_BC(&peakpart[static_cast<int64_t>(pi) * npk + slot0 + j], 21) peakpart[static_cast<int64_t>(pi) * npk + slot0 + j] = m;
    }
}

// Zeroes the accumulator cells that the TMA column stages add to atomically: the columns within
// H of a column-block boundary (multiples of W, and spc, wrapping to 0). Every other cell is
// stored by exactly one work item, so the accumulator needs no full clear.
__global__ void k_zero_edges(float* __restrict__ acc, int64_t rows, int spc, int spc_eff, int W, int H,
                             int n_bound) {
    pdl_trigger();
    const int per_row = n_bound * 2 * H;
    const int64_t total = rows * per_row;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t r = k / per_row;
        const int e = static_cast<int>(k - r * per_row);
        const int j = e / (2 * H), o = e - j * 2 * H - H;   // boundary j, offset in [-H, H)
        const int b = j == n_bound - 1 ? spc : j * W;
        int c = b + o;
        if (c < 0) c += spc;
        if (c >= spc) c -= spc;
        ACQ_BC(&acc[r * spc_eff + c], 22) acc[r * spc_eff + c] = 0.f;
    }
    pdl_wait();   // nothing here reads the tile; the wait keeps the chain's ordering transitive
}

#ifdef ACQ_BOUNDS_CHECK
// Checked build: every device allocation of the library (and the caller's input of the current
// request) is registered in a per-device table that the instrumented kernels check against.
namespace bc {
std::mutex mu;
struct DeviceTable {
    BoundsTable* d = nullptr;
    std::map<unsigned long long, unsigned long long> ranges;   // base -> end
};
std::map<int, DeviceTable>& tables() {
    static std::map<int, DeviceTable> t;
    return t;
}
// (lock held) the current device's table, created and handed to every translation unit on first use
DeviceTable& current() {
    int dev = 0;
    cudaGetDevice(&dev);
    DeviceTable& t = tables()[dev];
    if (!t.d) {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(BoundsTable)) != cudaSuccess) throw AcqError(ACQ_ERR_ALLOC, "bounds table");
        cudaMemset(p, 0, sizeof(BoundsTable));
        t.d = static_cast<BoundsTable*>(p);
        for (auto set : {acq_bounds_set_table_runtime, acq_inst_tile_set_bounds_table, acq_inst_col_set_bounds_table,
                         acq_inst_sign_set_bounds_table, acq_inst_mma_set_bounds_table})
            if (set(p) != cudaSuccess) throw AcqError(ACQ_ERR_CUDA, "bounds table upload");
    }
    return t;
}
void upload(DeviceTable& t) {
    if (t.ranges.size() > static_cast<size_t>(kBcMaxRanges)) throw AcqError(ACQ_ERR_UNSUPPORTED, "bounds table full");
    std::vector<unsigned long long> b(kBcMaxRanges, 0), e(kBcMaxRanges, 0);
    int n = 0;
    for (auto& kv : t.ranges) {
        b[n] = kv.first;
        e[n] = kv.second;
        ++n;
    }
    cudaDeviceSynchronize();
    cudaMemcpy(t.d->base, b.data(), sizeof(unsigned long long) * kBcMaxRanges, cudaMemcpyHostToDevice);
    cudaMemcpy(t.d->end, e.data(), sizeof(unsigned long long) * kBcMaxRanges, cudaMemcpyHostToDevice);
    cudaMemcpy(&t.d->n, &n, sizeof(int), cudaMemcpyHostToDevice);
}
void add(const void* p, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu);
    DeviceTable& t = current();
    const unsigned long long a = reinterpret_cast<unsigned long long>(p);
    t.ranges[a] = a + bytes;
    upload(t);
}
void remove(const void* p) {
    std::lock_guard<std::mutex> lk(mu);
    DeviceTable& t = current();
    t.ranges.erase(reinterpret_cast<unsigned long long>(p));
    upload(t);
}
// after the stream has finished: report (and clear) the first skipped access
void check() {
    std::lock_guard<std::mutex> lk(mu);
    DeviceTable& t = current();
    constexpr size_t kTail = sizeof(BoundsTable) - offsetof(BoundsTable, err_site);   // err_site .. hits
    static BoundsTable h;
    cudaMemcpy(&h.err_site, &t.d->err_site, kTail, cudaMemcpyDeviceToHost);
    if (h.err_site != 0) {
        const int site = h.err_site;
        const unsigned long long addr = h.err_addr, hits = h.hits;
        cudaMemset(&t.d->err_site, 0, kTail);
        char buf[160];
        std::snprintf(buf, sizeof buf, "device bounds check: access at 0x%llx (site %d) outside every buffer; %llu accesses skipped",
                      addr, site, hits);
        throw AcqError(ACQ_ERR_CUDA, buf);
    }
}
}  // namespace bc
#endif

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void reset() {
#ifdef ACQ_BOUNDS_CHECK
        if (p) bc::remove(p);
#endif
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t n) {
        if (n <= bytes) return;
        reset();
        if (n == 0) return;
        cudaError_t e = cudaMalloc(&p, n);
        if (e != cudaSuccess) {
            p = nullptr;
            throw AcqError(ACQ_ERR_ALLOC, "cudaMalloc(" + std::to_string(n) + ") failed: " + cudaGetErrorString(e));
        }
        bytes = n;
#ifdef ACQ_BOUNDS_CHECK
        bc::add(p, n);
#endif
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

// Page-locked host staging (results and the error word), so fetches are asynchronous copies
// followed by one stream synchronisation.
struct PinnedBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void reset() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    void ensure(size_t n) {
        if (n <= bytes) return;
        reset();
        if (n == 0) return;
        cudaError_t e = cudaHostAlloc(&p, n, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            p = nullptr;
            throw AcqError(ACQ_ERR_ALLOC, "cudaHostAlloc(" + std::to_string(n) + ") failed: " + cudaGetErrorString(e));
        }
        bytes = n;
    }
};

FftDesc make_fft_desc(int n, DevBuf& tw) {
    FftDesc d{};
    d.n = n;
    std::vector<int> r = fft_radices(n);
    if (static_cast<int>(r.size()) > kMaxFftStages) throw AcqError(ACQ_ERR_UNSUPPORTED, "FFT has too many stages");
    d.nst = static_cast<int>(r.size());
    int ns = 1;
    for (int s = 0; s < d.nst; ++s) {
        d.radix[s] = r[s];
        d.ns[s] = ns;
        d.stride[s] = n / (ns * r[s]);
        ns *= r[s];
    }
    std::vector<float2> h(n);
    for (int k = 0; k < n; ++k) {
        // exp(-2 pi i k / n) from a reduced angle, computed in double then rounded
        double a = -2.0 * M_PI * static_cast<double>(k) / static_cast<double>(n);
        h[k] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
    }
    tw.ensure(sizeof(float2) * n);
    CK(cudaMemcpy(tw.p, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    d.tw = tw.as<float2>();
    return d;
}

// Register-FFT twiddles W_n^e for n = 2..kRegTwMax (constant memory, per device).
void upload_reg_twiddles() {
    std::vector<float2> h(kRegTwEntries);
    for (int n = 2; n <= kRegTwMax; ++n)
        for (int e = 0; e < n; ++e) {
            double a = -2.0 * M_PI * static_cast<double>(e) / static_cast<double>(n);
            h[reg_tw_offset(n) + e] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
        }
    for (auto up : {acq_inst_tile_upload_twiddles, acq_inst_col_upload_twiddles, acq_inst_sign_upload_twiddles,
                    acq_inst_mma_upload_twiddles}) {
        cudaError_t e = up(h.data(), h.size());
        if (e != cudaSuccess) throw CudaError(std::string("twiddle upload: ") + cudaGetErrorString(e));
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}
int pow2_floor(int x) {
    int p = 1;
    while (p * 2 <= x) p *= 2;
    return p;
}

bool getenv_flag(const char* name) {
    const char* v = std::getenv(name);
    return v && v[0] && v[0] != '0';
}

size_t sample_bytes(int dtype) {
    switch (dtype) {
        case ACQ_CF32: return 8;
        case ACQ_CI16: return 4;
        case ACQ_CI8: return 2;
        case ACQ_CF64: return 16;
        default: throw AcqError(ACQ_ERR_ARGUMENT, "unknown sample dtype " + std::to_string(dtype));
    }
}

}  // namespace

struct acq_plan {
    acq_plan_desc desc{};
    Geometry g{};
    const SystemInfo* sys = nullptr;
    std::vector<int> prns;
    int device = 0;
    cudaStream_t stream = nullptr;
    FftDesc fftF{}, fftD{};
    DevBuf twF, twD;
    DevBuf U;     // signal spectra after the first Doppler pass (PRE column mode), like S
    DevBuf twT;   // pass-1 twiddles of the tile FFT, [k1][n2] = W_F^{n2 k1} (coalesced per k1)
    // plan-time constants
    DevBuf codes, conj, chips, pats, drift, sec, if_off;
    int64_t chips_len = 0;
    int n_pat = 1, combos = 1, edge_step = 1;
    // per-acquisition buffers
    DevBuf input, S, T, accb, winb, rowpart, colsum, peakpart, zs, res, slots, prn_ids;
    int tileB = 1, Wsimple = 1, Wsign = 1, nct = 1;
    size_t smem_front = 0, smem_tile = 0, smem_simple = 0, smem_sign = 0;
    // specialised two-pass FFT kernels for the plan's sizes (nullptr: generic kernels)
    TileFsFn tile_fs = nullptr;
    ColFsFn col_fs = nullptr;
    int tileNF = 1, Wfs = 1, tileThreads = 256, tileFS = 1, tileRows = 1;
    int tileBase = 1;   // pass-1 buffer size before padding: N1 rows of pitch tile_row_pitch(N2)
    std::vector<int> step_has_drift;
    size_t smem_tile_fs = 0, smem_col_fs = 0;
    // data-bit / bit-edge stage split by sub-blocks
    SignSbFn sign_sb = nullptr;
    size_t smem_ssb = 0;
    int Wssb = 8, threads_ssb = 256, n1ssb = 0;
    // rotation stage split by sub-blocks
    RotSbFn rot_sb = nullptr;
    size_t smem_rsb = 0;
    // tensor-core rotation combine (ACQ_OPT_ROTATION_PRECISION != FP32)
    RotMmaFn rot_mma = nullptr;
    size_t smem_mma = 0;
    int rot_prec = ACQ_PREC_FP32;
    // tensor-core Doppler DFT of the simple path (ACQ_OPT_DOPPLER_PRECISION != FP32)
    DftMmaFn dft_mma = nullptr;
    DevBuf dftB;
    int dftNpad = 0, dftKsteps = 0, dft_prec = ACQ_PREC_FP32;
    size_t smem_dft = 0;
    int mma_scale_log2 = 127;   // 127: by input type
    int Wrsb = 8, threads_rsb = 256;
    // specialised sign / rotation stages
    SignFsFn sign_fs = nullptr;
    RotFsFn rot_fs = nullptr;
    int Wsfs = 8;
    size_t smem_sfs = 0;
    // TMA-staged column stage over all steps (simple path)
    ColTmaFn col_tma = nullptr;
    bool col_pre = false;   // col_tma runs only the nb-point pass; the tile reads U
    // PRE-mode column stage by Doppler group (used instead of col_tma when set)
    ColTmaFn col_k1 = nullptr;
    CUtensorMap tmapK1{};
    int k1W = 128, k1Grid = 1, k1CtasPerSm = 0;
    uint32_t k1WaitPolls = kWaitLimit;   // ACQ_OPT_COLUMN_WAIT_POLLS (test-only)
    size_t smem_col_k1 = 0;
    // coherent tile as a correlation GEMM on the tensor cores (TMA simple path, block size <= 256):
    // time-domain operand blocks per (step, row), their inverse scales, one CTA per SM
    bool tmma = false;
    bool tmma_enabled = true;   // ACQ_OPT_TILE_MMA
    DevBuf stubs, invsc;
    int tmmaSms = 1;
    size_t smem_tmma = 0;
    CUtensorMap tmapT{};
    DevBuf Tall, errflag;
    PinnedBuf hstage;   // fetch staging: error word, then the results
    // request metadata (slots, PRN ids, IF offsets) staged in page-locked memory for one
    // asynchronous copy; two buffers, each reused only after its previous copy has run
    PinnedBuf hreq[2];
    cudaEvent_t hreq_ev[2] = {nullptr, nullptr};
    // the launch sequence of a repeated request, replayed as one CUDA graph (captured on the second
    // identical request in a row; `version` changes with every plan option)
    struct RequestKey {
        const void* d_in = nullptr;
        const void* dreq = nullptr;
        int dtype = -1, n = -1, use_if = 0;
        uint32_t flags = 0;
        float if_step = 0.f;
        double interm = 0.0;
        uint64_t version = 0;
        bool operator==(const RequestKey& o) const {
            return d_in == o.d_in && dreq == o.dreq && dtype == o.dtype && n == o.n && use_if == o.use_if &&
                   flags == o.flags && if_step == o.if_step && interm == o.interm && version == o.version;
        }
    };
    RequestKey last_key, graph_key;
    cudaGraphExec_t gexec = nullptr;
    int64_t graph_launches = 0;
    uint64_t version = 1;
    int hreq_next = 0;
    DevBuf dreq;
    DevBuf chipperm, sorted;   // chip-sorted surface export (src/plot.jl:35-57)
    int tmaW = 16, tmaBoxRows = 1, tmaBoxes = 1, tmaGrid = 1, tmaH = 0, tmaCtasPerSm = 0;
    int n_plan_prns = 0;
    size_t smem_col_tma = 0;
    // fused cluster form
    FusedFn fused = nullptr;
    int form = ACQ_FORM_PLAIN;
    int fusedCL = 8, fusedRPC = 1, fusedCPC = 1, fusedNF = 1, fusedH = 0;
    size_t smem_fused = 0;
    // last acquisition
    std::vector<std::string> klog;   // kernels of the last launch sequence, in launch order
    int last_n = 0;
    uint32_t last_flags = 0;
    int64_t launches = 0;
    std::vector<int> req_prns;
    // optional per-launch timing (acq_plan_set_kernel_timing)
    bool timing = false;
    std::vector<cudaEvent_t> ev_start, ev_stop;
    std::vector<int> ev_kind;
    size_t ev_used = 0;
    double kt_ms[ACQ_KERNEL_KINDS] = {0};
    int64_t kt_n[ACQ_KERNEL_KINDS] = {0};
};

namespace {

// Allow every kernel the opt-in maximum once (per device); the launch decides what it uses,
// so plans with different shapes never shrink each other's limit.
constexpr int kSmemOptIn = 227 * 1024;
void set_smem(const void* fn, size_t bytes) {
    if (bytes > static_cast<size_t>(kSmemOptIn))
        throw AcqError(ACQ_ERR_UNSUPPORTED, "kernel needs " + std::to_string(bytes) + " bytes of shared memory");
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemOptIn));
}

void t_begin(acq_plan* P, int kind) {
    if (!P->timing) return;
    if (P->ev_used == P->ev_start.size()) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        P->ev_start.push_back(a);
        P->ev_stop.push_back(b);
        P->ev_kind.push_back(kind);
    }
    P->ev_kind[P->ev_used] = kind;
    CK(cudaEventRecord(P->ev_start[P->ev_used], P->stream));
}

void t_end(acq_plan* P) {
    if (!P->timing) return;
    CK(cudaEventRecord(P->ev_stop[P->ev_used], P->stream));
    ++P->ev_used;
}

// Launch with programmatic stream serialisation when `pdl` is set (the kernel may start while the
// previous kernel of the stream finishes; it calls pdl_wait before using that kernel's results).
template <typename... KArgs, typename... Args>
void launch(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    CK(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
}

// Launch log: the kernel about to be launched (a size-specialised kernel by its registered name).
void klog(acq_plan* P, const void* fn, const char* fallback) {
    const char* nm = fn ? kernel_name(fn) : nullptr;
    P->klog.emplace_back(nm ? nm : fallback);
}

void t_collect(acq_plan* P) {
    for (size_t i = 0; i < P->ev_used; ++i) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, P->ev_start[i], P->ev_stop[i]));
        P->kt_ms[P->ev_kind[i]] += ms;
        P->kt_n[P->ev_kind[i]] += 1;
    }
    P->ev_used = 0;
}

// Choose the fused cluster form when the plan's sizes have a fused kernel, its shared memory
// fits and a cluster of that shape can be resident.
void setup_fused(acq_plan* P) {
    const Geometry& g = P->g;
    P->fused = nullptr;
    if (g.path != 0 || getenv_flag("ACQ_GENERIC_FFT")) return;
    FusedFn fn = pick_fused(g.fft_tile, g.ndop);
    if (!fn) return;
    // signed drift bound over all steps (src/noncoherent_integration.jl:600-619)
    int H = 0;
    std::vector<int32_t> dr(g.ndop);
    for (int m = 0; m < g.n_nc; ++m) {
        code_drift_shifts(g, *P->sys, P->desc.sampling_freq_hz, m, dr.data());
        for (int v : dr) H = std::max(H, std::min(v, g.spc - v));
    }
    const int CL = 8;
    const int rpc = (g.ndop + CL - 1) / CL;
    const int cpc = (g.bs + CL - 1) / CL;
    if (H > cpc) return;
    const int nf = 8;   // one FFT buffer per warp
    const size_t smem = sizeof(float2) * (size_t)g.ndop * cpc + sizeof(float2) * (size_t)nf * g.fft_tile +
                        sizeof(float) * (size_t)g.ndop * (cpc + 2 * H) + sizeof(int) * (size_t)g.ndop;
    if (smem > 220 * 1024) return;
    set_smem((const void*)fn, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.nb * CL, 1, 1);
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, (const void*)fn, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        return;
    }
    P->fused = fn;
    P->fusedCL = CL;
    P->fusedRPC = rpc;
    P->fusedCPC = cpc;
    P->fusedNF = nf;
    P->fusedH = H;
    P->smem_fused = smem;
}

// First pass of the Doppler four-step FFT applied to the signal block spectra (the PRE mode of
// k_col_tma): for every step, code-block class k (< nb) and frequency bin nu,
//   U[k + nb k1][nu] = W_ndop^{k k1} sum_q W_{n_coh}^{q k1} S[k + nb q][nu],   k1 < n_coh,
// a direct n_coh-point DFT with the ndop-point table (W_{n_coh}^e = W_ndop^{e nb}).
// The coherent tile is linear in S and uses the code block (k + r) mod nb for every row of class
// k, so tiling U gives the first pass's output of the Doppler FFT of the tile of S.
__global__ void __launch_bounds__(128) k_doppler_prepass(const float2* __restrict__ S, float2* __restrict__ U,
                                                         int G, int nb, int n_coh, int F,
                                                         const float2* __restrict__ twD) {
    // one output per thread: nu from x, (k1, k) from y, step from z
    const int nu = blockIdx.x * blockDim.x + threadIdx.x;
    if (nu >= F) return;
    const int k1 = blockIdx.y / nb, k = blockIdx.y - k1 * nb;
    const int64_t base = static_cast<int64_t>(blockIdx.z) * G;
    float2 acc = S[(base + k) * F + nu];
    int e = 0;   // (q k1) mod n_coh
#pragma unroll 4
    for (int q = 1; q < n_coh; ++q) {
        e += k1;
        if (e >= n_coh) e -= n_coh;
        const float2 x = S[(base + k + nb * q) * F + nu];
        acc = c_add(acc, e ? c_mul(x, __ldg(twD + e * nb)) : x);
    }
    if (k * k1) acc = c_mul(acc, __ldg(twD + k * k1));
    U[(base + k + nb * k1) * F + nu] = acc;
}

// Transform length of the block FFTs and the coherent tile. Any length >= 2 bs gives the same lags
// 0..bs-1 of the linear correlation (the circular wrap never reaches them), so a power of two, or
// five times one, within 5 % above the reference's fft_size replaces it when a specialised tile
// kernel exists: radix-4/8 stages are cheaper than radix-5/7 ones and the four-step split then
// fills warps evenly. ACQ_REFERENCE_FFT_SIZE=1 keeps fft_size.
int choose_fft_tile(const Geometry& g) {
    if (getenv_flag("ACQ_REFERENCE_FFT_SIZE") || getenv_flag("ACQ_GENERIC_FFT")) return g.fft_size;
    const int lo = 2 * g.bs;
    for (int base : {1, 5}) {
        long long L = base;
        while (L < lo) L *= 2;
        if (L == g.fft_size) return g.fft_size;
        if (L * 100 <= 105LL * g.fft_size && pick_tile_fs(static_cast<int>(L), 1)) return static_cast<int>(L);
    }
    return g.fft_size;
}

// Coherent-tile launch shape: shared memory (R rows of S, R * NF FFT buffers of stride FS) and
// grid width (one CTA per group of R rows sharing g mod nb).
size_t tile_smem(const acq_plan* P) {
    return sizeof(float2) * static_cast<size_t>(P->tileRows) *
           (P->g.fft_tile + static_cast<size_t>(P->tileFS) * P->tileNF);
}

int tile_grid_x(const acq_plan* P) {
    return P->g.nb * ((P->g.n_coh + P->tileRows - 1) / P->tileRows);
}

// PRE-mode column stage by Doppler group k1: tiles of nb rows x W columns of the all-steps tile
// buffer (set up by setup_col_tma), 128 threads, a persistent grid. Leaves col_k1 null when the
// shape does not fit.
void setup_col_k1(acq_plan* P, int n_prns, int W, int ctas_per_sm) {
    const Geometry& g = P->g;
    P->col_k1 = nullptr;
    if (!P->col_tma || !P->col_pre || getenv_flag("ACQ_NO_COL_K1")) return;
    ColTmaFn fn = pick_col_tma_k1(g.nb);
    if (!fn || W < 2 || W > 256 || W % 2 || P->tmaH > W) return;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return;
    const int H = P->tmaH;
    const size_t bs = (static_cast<size_t>(g.nb) * W + 15) & ~static_cast<size_t>(15);
    const size_t smem = 2 * sizeof(float2) * bs + sizeof(float) * (size_t)g.nb * (W + 2 * H) +
                        sizeof(int) * (size_t)(g.n_nc + 1) * g.nb + 16 + 16;
    if (smem > 200 * 1024) return;
    cuuint64_t gdim[2] = {static_cast<cuuint64_t>(g.spc), static_cast<cuuint64_t>(g.n_nc) * n_prns * g.ndop};
    cuuint64_t gstride[1] = {static_cast<cuuint64_t>(g.spc) * sizeof(float2)};
    cuuint32_t bdim[2] = {static_cast<cuuint32_t>(W), static_cast<cuuint32_t>(g.nb)};
    cuuint32_t estr[2] = {1, 1};
    CUtensorMap map{};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, P->Tall.p, gdim, gstride, bdim, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return;
    set_smem((const void*)fn, smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, 128, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return;
    }
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, P->device));
    // per-item statistics of this form: row sums per column block, and a peak key per item plus
    // one per block boundary
    const int n_cblk = (g.spc + W - 1) / W;
    P->rowpart.ensure(sizeof(double) * (size_t)n_prns * n_cblk * g.ndop);
    P->peakpart.ensure(sizeof(unsigned long long) * (size_t)n_prns * (g.n_coh * n_cblk + n_cblk + 1));
    P->tmapK1 = map;
    P->col_k1 = fn;
    P->k1W = W;
    P->k1CtasPerSm = ctas_per_sm > 0 ? std::min(per_sm, ctas_per_sm) : per_sm;
    P->k1Grid = sms * P->k1CtasPerSm;
    P->smem_col_k1 = smem;
}

// Tensor-core coherent tile (k_tile_mma): used when the block size fits its operands
// (bs <= 256) and ACQ_OPT_TILE_MMA is on, for all steps in one launch on the TMA simple path and
// one launch per step on the others. The FP32 FFT tiles stay the fallback (and ACQ_GENERIC_FFT
// keeps the generic kernels).
bool tile_mma_possible(const acq_plan* P) {
    // the drain addresses a step's tile (the plan's PRNs x rows x spc cells) with 32-bit offsets
    const int64_t step_cells = static_cast<int64_t>(P->n_plan_prns) * P->g.n_coh * P->g.nb * P->g.spc;
    return P->tmma_enabled && P->g.bs <= kTmmaMaxBs && step_cells < (int64_t{1} << 31) &&
           !getenv_flag("ACQ_NO_TILE_MMA") && !getenv_flag("ACQ_GENERIC_FFT");
}

void setup_tile_mma(acq_plan* P) {
    const Geometry& g = P->g;
    P->tmma = false;
    if (!tile_mma_possible(P)) return;
    const int G = g.n_coh * g.nb;
    const size_t row_bytes = tmma_row_bytes(g.bs);
    // one CTA per SM: a CTA holds up to 512 tensor-memory columns
    const size_t smem = std::max<size_t>(tmma_smem_bytes(g.bs), 120 * 1024);
    if (smem > 227 * 1024) return;
    P->stubs.ensure(row_bytes * g.n_nc * G);
    P->invsc.ensure(sizeof(float) * g.n_nc * G);
    set_smem((const void*)k_tile_mma, smem);
    CK(cudaDeviceGetAttribute(&P->tmmaSms, cudaDevAttrMultiProcessorCount, P->device));
    if (!P->errflag.p) {
        P->errflag.ensure(sizeof(int));
        CK(cudaMemset(P->errflag.p, 0, sizeof(int)));
    }
    P->smem_tmma = smem;
    P->tmma = true;
}

// TMA-staged column stage: T for all steps in HBM, a tensor map over it, a persistent grid.
void setup_col_tma(acq_plan* P, int n_prns, int W = 16, int ctas_per_sm = 0) {
    const Geometry& g = P->g;
    P->col_tma = nullptr;
    P->col_pre = false;
    P->col_k1 = nullptr;
    // the all-steps column stage needs an all-steps tile: the FFT tile's instantiation for the
    // transform length, or the tensor-core tile (any length)
    if (g.path != 0 || (!P->tile_fs && !tile_mma_possible(P)) || getenv_flag("ACQ_GENERIC_FFT") ||
        getenv_flag("ACQ_NO_TMA"))
        return;
    ColTmaFn fn = pick_col_tma(g.ndop);
    bool pre = false;
    if (g.n_coh <= 64 && !getenv_flag("ACQ_NO_PREPASS"))
        if (ColTmaFn f2 = pick_col_tma_pre(g.nb)) {
            fn = f2;
            pre = true;
        }
    if (!fn || (g.spc % 2) != 0) return;
    const size_t tall = sizeof(float2) * (size_t)g.n_nc * n_prns * g.ndop * g.spc;
    // all-steps tile buffer per plan: up to 16 GB and an eighth of the device's memory (batches hold
    // many plans); larger requests run the per-step column kernels
    size_t cap = 16ull << 30;
    {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) cap = std::min(cap, total_b / 8);
        else cudaGetLastError();
    }
    if (const char* e = std::getenv("ACQ_TALL_CAP_GB")) cap = static_cast<size_t>(std::atof(e) * (1ull << 30));
    if (tall > cap) return;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return;
    int H = 0;
    std::vector<int32_t> dr(g.ndop);
    for (int m = 0; m < g.n_nc; ++m) {
        code_drift_shifts(g, *P->sys, P->desc.sampling_freq_hz, m, dr.data());
        for (int v : dr) H = std::max(H, std::min(v, g.spc - v));
    }
    if (H > W || W < 2 || W > 256 || W % 2) return;   // TMA: x * 8 B a multiple of 16 B, box <= 256
    // rows per TMA box: the largest divisor of ndop up to 256 whose box keeps every box start in
    // the shared tile on a 128-byte boundary (one box per tile always does)
    int box = 0;
    for (int d = 1; d <= 256 && d <= g.ndop; ++d)
        if (g.ndop % d == 0 && (d == g.ndop || (static_cast<size_t>(d) * W * sizeof(float2)) % 128 == 0)) box = d;
    if (box == 0) return;
    const size_t tile_stride = (static_cast<size_t>(g.ndop) * W + 15) & ~static_cast<size_t>(15);
    const size_t smem = 2 * sizeof(float2) * tile_stride + sizeof(float) * (size_t)g.ndop * (W + 2 * H) +
                        sizeof(int) * (size_t)g.n_nc * g.ndop + 16 + 16;
    if (smem > 200 * 1024) return;
    P->Tall.ensure(tall);
    cuuint64_t gdim[2] = {static_cast<cuuint64_t>(g.spc), static_cast<cuuint64_t>(g.n_nc) * n_prns * g.ndop};
    cuuint64_t gstride[1] = {static_cast<cuuint64_t>(g.spc) * sizeof(float2)};
    cuuint32_t bdim[2] = {static_cast<cuuint32_t>(W), static_cast<cuuint32_t>(box)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&P->tmapT, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, P->Tall.p, gdim, gstride, bdim, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        P->Tall.reset();
        return;
    }
    set_smem((const void*)fn, smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)fn, kThreads, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        P->Tall.reset();
        return;
    }
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, P->device));
    P->errflag.ensure(sizeof(int));
    CK(cudaMemset(P->errflag.p, 0, sizeof(int)));
    if (pre && g.n_coh > 1) P->U.ensure(sizeof(float2) * (size_t)g.n_nc * g.ndop * g.fft_tile);
    P->col_tma = fn;
    P->col_pre = pre;
    P->tmaW = W;
    P->tmaBoxRows = box;
    P->tmaBoxes = g.ndop / box;
    P->tmaGrid = sms * (ctas_per_sm > 0 ? std::min(per_sm, ctas_per_sm) : per_sm);
    P->tmaCtasPerSm = ctas_per_sm > 0 ? std::min(per_sm, ctas_per_sm) : per_sm;
    P->tmaH = H;
    P->smem_col_tma = smem;
    if (pre) setup_col_k1(P, n_prns, P->k1W, P->k1CtasPerSm);
    if (!tile_mma_possible(P) && !P->tile_fs) {   // no tile for this stage: the per-step kernels
        P->col_tma = nullptr;
        P->col_pre = false;
        P->col_k1 = nullptr;
    }
}

// Split bit-edge search (path 1, even ndop): the instantiation for the plan's size with the
// wanted columns per CTA and first-pass length (0: the size's default). Returns false, leaving
// the plan's kernel as it was, when none matches.
bool setup_sign_search(acq_plan* P, int want_w, int want_n1) {
    const Geometry& g = P->g;
    if (g.path != 1 || (g.ndop % 2) != 0 || getenv_flag("ACQ_GENERIC_FFT") || (g.n_coh % g.ndb) != 0) return false;
    int w = 8, n1 = 0, th = 256;
    size_t smem = 0;
    SignSbFn fn = pick_sign_sb(g.ndop, g.ndb, want_w, want_n1, &w, &n1, &th, &smem);
    if (!fn || smem > 220 * 1024) return false;
    set_smem((const void*)fn, smem);
    P->sign_sb = fn;
    P->smem_ssb = smem;
    P->Wssb = w;
    P->n1ssb = n1;
    P->threads_ssb = th;
    return true;
}

// Split rotation search (path 2, even ndop), likewise for the columns per CTA.
bool setup_rot_search(acq_plan* P, int want_w) {
    const Geometry& g = P->g;
    if (g.path != 2 || (g.ndop % 2) != 0 || getenv_flag("ACQ_GENERIC_FFT")) return false;
    int w = 8, th = 256;
    RotSbFn fn = pick_rot_sb(g.n_coh, g.nb, want_w, &w, &th);
    if (!fn) return false;
    const size_t need = sizeof(float2) * ((size_t)2 * g.ndop * w + g.ndop) + sizeof(int) * w +
                        sizeof(float) * (size_t)g.R * ((size_t)1 << (g.ndb - 1)) * g.n_coh;
    if (need > 200 * 1024) return false;
    set_smem((const void*)fn, need);
    P->rot_sb = fn;
    P->smem_rsb = need;
    P->Wrsb = w;
    P->threads_rsb = th;
    return true;
}

void plan_setup(acq_plan* P, const int32_t* prns, int n_prns, const int8_t* user_codes) {
    const Geometry& g = P->g;
    CK(cudaSetDevice(P->device));
    CK(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    P->fftF = make_fft_desc(g.fft_tile, P->twF);
    P->fftD = make_fft_desc(g.ndop, P->twD);
    // launch shapes
    P->smem_front = 2 * sizeof(float2) * g.fft_tile;
    if (P->smem_front > kSmemBudget)
        throw AcqError(ACQ_ERR_UNSUPPORTED, "fft_size=" + std::to_string(g.fft_tile) + " exceeds shared memory");
    P->tileB = std::max(1, std::min(8, static_cast<int>((96 * 1024 / (sizeof(float2) * g.fft_tile) - 1) / 2)));
    P->smem_tile = sizeof(float2) * g.fft_tile * (1 + 2 * P->tileB);
    P->Wsimple = std::max(1, std::min(32, pow2_floor(static_cast<int>(kSmemBudget / (16 * (size_t)g.ndop)))));
    if (16ull * g.ndop > kSmemBudget) throw AcqError(ACQ_ERR_UNSUPPORTED, "num_doppler_bins too large");
    P->smem_simple = 16ull * g.ndop * P->Wsimple;
    const size_t per_col_sign = 3 * 8 + 4 + 2;  // tile + 2 work buffers + stage + winner, per row
    P->Wsign = std::max(1, std::min(16, pow2_floor(static_cast<int>(kSmemBudget / (per_col_sign * g.ndop + 8)))));
    if (per_col_sign * g.ndop + 8 > kSmemBudget) throw AcqError(ACQ_ERR_UNSUPPORTED, "num_doppler_bins too large");
    P->smem_sign = per_col_sign * (size_t)g.ndop * P->Wsign + 4 * P->Wsign + 16;
    set_smem((const void*)k_frontend, P->smem_front);
    set_smem((const void*)k_code_spectra, P->smem_front);
    set_smem((const void*)k_tile, P->smem_tile);
    set_smem((const void*)k_col_simple, P->smem_simple);
    set_smem((const void*)k_col_sign, P->smem_sign);
    set_smem((const void*)k_col_rot, P->smem_sign);
    upload_reg_twiddles();
    if (!getenv_flag("ACQ_GENERIC_FFT")) {
        P->tile_fs = pick_tile_fs(g.fft_tile, 1);
        P->col_fs = g.path == 0 ? pick_col_fs(g.ndop) : nullptr;
    }
    if (P->tile_fs) {
        // one round of pass-1 tasks per chunk: NF * N2 <= threads (N2 = fft_size / best_split_n1)
        const int n1 = best_split_n1(g.fft_tile), n2 = g.fft_tile / std::max(1, n1);
        P->tileThreads = 128;
        P->tileNF = std::max(1, std::min(g.nb, P->tileThreads / std::max(1, n2)));
        if (const char* e = std::getenv("ACQ_TILE_THREADS")) P->tileThreads = std::max(32, std::min(256, std::atoi(e)));
        if (const char* e = std::getenv("ACQ_TILE_NF")) P->tileNF = std::max(1, std::min(g.nb, std::atoi(e)));
        // stagger neighbouring FFT buffers by 9 float2 (18 banks) so warps spanning two FFTs don't conflict
        P->tileBase = n1 * tile_row_pitch(n2);
        P->tileFS = P->tileBase + ((9 - (P->tileBase % 16) + 16) % 16);
        if (const char* e = std::getenv("ACQ_TILE_PAD")) P->tileFS = P->tileBase + std::atoi(e);
        // two rows per CTA share the code-spectrum loads where the plan has rows to pair (the
        // larger FFT sizes would need about twice the registers per thread for the second row)
        int rows = (g.n_coh >= 2 && g.fft_tile <= 1250) ? 2 : 1;
        if (const char* e = std::getenv("ACQ_TILE_ROWS")) rows = std::atoi(e);
        if (rows != 1) {
            if (TileFsFn fn = pick_tile_fs(g.fft_tile, rows)) {
                P->tile_fs = fn;
                P->tileRows = rows;
                if (tile_smem(P) > 200 * 1024) {
                    P->tile_fs = pick_tile_fs(g.fft_tile, 1);
                    P->tileRows = 1;
                }
            }
        }
        P->smem_tile_fs = tile_smem(P);
        set_smem((const void*)P->tile_fs, P->smem_tile_fs);
        // the same values as the F-point table at n2 * k1, laid out so that the threads of a warp
        // (consecutive n2) read consecutive entries for each compile-time k1
        std::vector<float2> h(static_cast<size_t>(g.fft_tile));
        for (int k1 = 0; k1 < n1; ++k1)
            for (int q = 0; q < n2; ++q) {
                const double a = -2.0 * M_PI * static_cast<double>(q * k1) / static_cast<double>(g.fft_tile);
                h[static_cast<size_t>(k1) * n2 + q] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
            }
        P->twT.ensure(sizeof(float2) * h.size());
        CK(cudaMemcpy(P->twT.p, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice));
    }
    if (!getenv_flag("ACQ_GENERIC_FFT") && (g.ndop % 2) == 0) {
        if (g.path == 1) P->sign_fs = pick_sign_fs(g.ndop);
        if (g.path == 2) P->rot_fs = pick_rot_fs(g.ndop);
    }
    setup_sign_search(P, 0, 0);
    setup_rot_search(P, 0);
    if (P->sign_fs || P->rot_fs) {
        const size_t per = 2 * 8 + 4 + 2;   // tile + work (float2), stage (float), winner (u16)
        int W = 16;
        while (W > 1 && per * (size_t)g.ndop * W + 4 * W + 16 > 110 * 1024) W /= 2;
        P->Wsfs = W;
        P->smem_sfs = per * (size_t)g.ndop * W + 4 * W + 16;
        if (P->sign_fs) set_smem((const void*)P->sign_fs, P->smem_sfs);
        if (P->rot_fs) set_smem((const void*)P->rot_fs, P->smem_sfs);
    }
    if (P->col_fs) {
        P->Wfs = g.ndop <= 400 ? 32 : g.ndop <= 800 ? 16 : 8;
        if (const char* e = std::getenv("ACQ_COL_W")) P->Wfs = std::max(1, std::min(64, std::atoi(e)));
        P->smem_col_fs = sizeof(float2) * g.ndop * P->Wfs + sizeof(int) * g.ndop;
        set_smem((const void*)P->col_fs, P->smem_col_fs);
    }
    P->nct = (g.spc_eff + kStatsCols - 1) / kStatsCols;
    setup_fused(P);
    P->n_plan_prns = n_prns;
    setup_col_tma(P, n_prns);
    setup_tile_mma(P);
    {
        std::vector<int32_t> perm(g.spc_eff);
        chip_order(g.nb, g.bs, g.spc_eff, P->sys->code_freq, P->desc.sampling_freq_hz, perm.data(), nullptr);
        P->chipperm.ensure(sizeof(int32_t) * perm.size());
        CK(cudaMemcpy(P->chipperm.p, perm.data(), sizeof(int32_t) * perm.size(), cudaMemcpyHostToDevice));
    }

    // codes (GNSSSignals gen_code semantics) and conj code-block spectra, src/plan.jl:230-251:
    // chip tables (LFSR / memory codes, secondary folded in) built on the host, sampled on the
    // device; user codes are uploaded as given
    {
        std::vector<int8_t> c0 = full_chips(P->desc.system, prns[0]);
        P->chips_len = static_cast<int64_t>(c0.size());
        std::vector<int8_t> all((size_t)n_prns * P->chips_len);
        for (int i = 0; i < n_prns; ++i) {
            std::vector<int8_t> c = i == 0 ? c0 : full_chips(P->desc.system, prns[i]);
            std::memcpy(&all[(size_t)i * P->chips_len], c.data(), P->chips_len);
        }
        P->chips.ensure(all.size());
        CK(cudaMemcpy(P->chips.p, all.data(), all.size(), cudaMemcpyHostToDevice));
    }
    P->codes.ensure((size_t)n_prns * g.spc);
    if (user_codes) {
        CK(cudaMemcpy(P->codes.p, user_codes, (size_t)n_prns * g.spc, cudaMemcpyHostToDevice));
    } else {
        sample_codes_device(P->desc.system, P->chips.as<int8_t>(), P->chips_len, n_prns, g.spc,
                            P->desc.sampling_freq_hz, 0.0, 0.0, P->codes.as<int8_t>(), P->stream);
    }
    P->conj.ensure(sizeof(float2) * (size_t)n_prns * g.nb * g.fft_tile);
    k_code_spectra<<<n_prns * g.nb, kThreads, P->smem_front, P->stream>>>(P->codes.as<int8_t>(), g.spc, g.nb, g.bs,
                                                                           P->fftF, P->conj.as<float2>());
    CK(cudaGetLastError());
    // secondary code for the secondary-code despread (rotation path only)
    if (g.path == 2) {
        P->sec.ensure(P->sys->secondary_length);
        CK(cudaMemcpy(P->sec.p, P->sys->secondary, P->sys->secondary_length, cudaMemcpyHostToDevice));
    }
    // sign patterns per PRN, src/sign_patterns.jl:23-47
    if (g.path != 0) {
        P->combos = 1 << (g.ndb - 1);
        std::vector<float> all;
        for (int i = 0; i < n_prns; ++i) {
            std::vector<float> p = sign_patterns(P->desc.system, prns[i], g.ndb, g.R, g.n_coh, g.use_secondary_code != 0);
            P->n_pat = static_cast<int>(p.size() / g.n_coh);
            all.insert(all.end(), p.begin(), p.end());
        }
        P->pats.ensure(sizeof(float) * all.size());
        CK(cudaMemcpy(P->pats.p, all.data(), sizeof(float) * all.size(), cudaMemcpyHostToDevice));
        const int bpc_k = g.n_coh / g.ndb;
        P->edge_step = bpc_k * g.nb / g.n_be;   // src/acquire.jl:298-299
    }
    // drift shifts per step, src/noncoherent_integration.jl:600-619
    std::vector<int32_t> dr((size_t)g.n_nc * g.ndop);
    for (int m = 0; m < g.n_nc; ++m) code_drift_shifts(g, *P->sys, P->desc.sampling_freq_hz, m, &dr[(size_t)m * g.ndop]);
    P->step_has_drift.assign(g.n_nc, 0);
    for (int m = 0; m < g.n_nc; ++m)
        for (int r = 0; r < g.ndop; ++r)
            if (dr[(size_t)m * g.ndop + r] != 0) P->step_has_drift[m] = 1;
    P->drift.ensure(sizeof(int32_t) * dr.size());
    CK(cudaMemcpy(P->drift.p, dr.data(), sizeof(int32_t) * dr.size(), cudaMemcpyHostToDevice));
    // per-acquisition buffers sized for all plan PRNs
    const size_t np = n_prns;
    P->S.ensure(sizeof(float2) * (size_t)g.n_nc * g.ndop * g.fft_tile);
    P->T.ensure(sizeof(float2) * np * g.ndop * g.spc);
    P->accb.ensure(sizeof(float) * np * g.ndop * g.spc_eff);
    if (g.path != 0) P->winb.ensure(sizeof(uint16_t) * np * g.ndop * g.spc_eff);
    P->rowpart.ensure(sizeof(double) * np * P->nct * g.ndop);
    P->colsum.ensure(sizeof(double) * np * g.spc_eff);
    P->peakpart.ensure(sizeof(unsigned long long) * np * P->nct);
    P->zs.ensure(sizeof(double2) * np * std::max(1, g.R));
    P->res.ensure(sizeof(acq_result) * np);
    P->slots.ensure(sizeof(int) * np);
    P->prn_ids.ensure(sizeof(int) * np);
    P->if_off.ensure(sizeof(float) * g.n_nc);
    CK(cudaStreamSynchronize(P->stream));
}

// Device-resident arguments of one acquisition's launch sequence.
struct LaunchArgs {
    int n = 0;
    const int* d_slots = nullptr;
    const int* d_prn_ids = nullptr;
    const float* d_if_off = nullptr;
    int use_if = 0;
    float if_step = 0.f;
    double interm_freq = 0.0;
    uint32_t flags = 0;
    acq_result* d_res = nullptr;
};

// Validation and host-side constants of acquire! (src/acquire.jl:62-72, :96-97).
void prepare_request(const acq_plan* P, int64_t n_samples, const int32_t* prns, int n, double interm_freq,
                     std::vector<int>& slots, std::vector<float>& offs, int& use_if, float& if_step) {
    const Geometry& g = P->g;
    const int64_t seg_len = static_cast<int64_t>(g.n_coh) * g.spc;
    if (n <= 0) throw AcqError(ACQ_ERR_ARGUMENT, "no PRNs requested");
    // the per-acquisition device buffers hold one surface per plan PRN; a request can repeat PRNs
    // (each repeat is searched again, as in the reference) up to that count
    if (n > static_cast<int>(P->prns.size()))
        throw AcqError(ACQ_ERR_ARGUMENT, "a request may list at most " + std::to_string(P->prns.size()) +
                                             " PRNs (the plan's PRN count), got " + std::to_string(n));
    slots.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        auto it = std::find(P->prns.begin(), P->prns.end(), prns[i]);
        if (it == P->prns.end()) {
            std::string got = "[", av = "[";
            for (int j = 0; j < n; ++j) got += (j ? ", " : "") + std::to_string(prns[j]);
            for (size_t j = 0; j < P->prns.size(); ++j) av += (j ? ", " : "") + std::to_string(P->prns[j]);
            throw AcqError(ACQ_ERR_PRN_NOT_IN_PLAN,
                           "All requested PRNs must be in plan.avail_prns. Got: " + got + "], available: " + av + "]");
        }
        slots[i] = static_cast<int>(it - P->prns.begin());
    }
    const int64_t nseg = n_samples / seg_len;
    if (nseg < g.n_nc)
        throw AcqError(ACQ_ERR_SHORT_SIGNAL, "Signal has " + std::to_string(n_samples) + " samples → " +
                                                 std::to_string(nseg) + " full segments of " + std::to_string(seg_len) +
                                                 ", but plan.num_noncoherent_accumulations=" + std::to_string(g.n_nc) +
                                                 ". Provide a longer signal.");
    use_if = interm_freq != 0.0;
    if_step = 0.f;
    offs.assign(g.n_nc, 0.f);
    if (use_if) {
        if_step = static_cast<float>(-2.0 * M_PI * interm_freq / P->desc.sampling_freq_hz);
        for (int m = 0; m < g.n_nc; ++m) {
            const float seg0 = static_cast<float>(static_cast<int64_t>(m) * seg_len);
            volatile float prod = seg0 * if_step;
            offs[m] = prod;
        }
    }
}

// The whole launch sequence of one acquisition on `st` (capturable into a CUDA graph: no host
// memory is touched). Returns the number of this library's kernel launches.
int64_t launch_sequence(acq_plan* P, cudaStream_t st, const void* d_in, int dtype, const LaunchArgs& a) {
    const Geometry& g = P->g;
    const int64_t seg_len = static_cast<int64_t>(g.n_coh) * g.spc;
    const int n = a.n;
    const uint32_t flags = a.flags;
    const int use_if = a.use_if;
    const float if_step = a.if_step;
    int64_t L = 0;
    P->klog.clear();
    int stats_nct = 0, stats_npk = 0;   // set when the column stage produced the statistics
    const int G = g.n_coh * g.nb;
    const bool use_fused = P->fused && P->form == ACQ_FORM_FUSED;
    const bool use_tma = !use_fused && P->col_tma != nullptr && P->dft_mma == nullptr;
    // the tensor-core tile reads the samples itself: no block spectra (all steps in one launch on
    // the TMA path, one launch per step otherwise)
    const bool use_tmma = use_tma && P->tmma;
    const bool use_tmma_step = !use_fused && !use_tma && P->tmma;
    // the all-steps tensor-core chain (operand blocks -> tile -> edge zeroing -> Doppler-group column
    // stage -> edge keys -> extraction) overlaps each kernel's launch with its predecessor's tail;
    // not while the kernels are timed one by one. Only for steps whose tile is small (at most
    // 256 MB): there the launch gaps are a visible share of the step (1 ms, 32 PRNs at 4 MHz:
    // +3 % acquisitions/s); on multi-GB tiles the early-resident blocks cost more than the gaps
    // (10 ms x 8 at 5 MHz: -1.3 %)
    const size_t step_tile_bytes = sizeof(float2) * (size_t)g.n_nc * P->prns.size() * g.ndop * g.spc;
    const bool pdl = use_tmma && P->col_k1 && !P->timing &&
                     (step_tile_bytes <= (256ull << 20) || getenv_flag("ACQ_PDL")) && !getenv_flag("ACQ_NO_PDL");
    if (!use_tmma && !use_tmma_step) {
        t_begin(P, ACQ_KERNEL_FRONTEND);
        klog(P, nullptr, "k_frontend");
        k_frontend<<<g.n_nc * G, kThreads, P->smem_front, st>>>(d_in, dtype, seg_len, G, g.bs, P->fftF,
                                                                P->S.as<float2>(), use_if, if_step, a.d_if_off);
        t_end(P);
        ++L;
    }
    if (use_fused) {
        if (P->fusedH > 0)
            CK(cudaMemsetAsync(P->accb.p, 0, sizeof(float) * (size_t)n * g.ndop * g.spc_eff, st));
        FusedParams fp{};
        fp.G = G; fp.nb = g.nb; fp.bs = g.bs; fp.spc = g.spc; fp.spc_eff = g.spc_eff; fp.n_nc = g.n_nc;
        fp.rpc = P->fusedRPC; fp.cpc = P->fusedCPC; fp.nf = P->fusedNF; fp.halo = P->fusedH;
        fp.S = P->S.as<float2>(); fp.C = P->conj.as<float2>(); fp.slots = a.d_slots;
        fp.twF = P->fftF.tw; fp.twD = P->fftD.tw; fp.drift = P->drift.as<int>(); fp.acc = P->accb.as<float>();
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(g.nb * P->fusedCL, n, 1);
        cfg.blockDim = dim3(kThreads, 1, 1);
        cfg.dynamicSmemBytes = P->smem_fused;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = P->fusedCL;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        t_begin(P, ACQ_KERNEL_FUSED);
        klog(P, (const void*)P->fused, "k_fused_simple");
        CK(cudaLaunchKernelEx(&cfg, P->fused, fp));
        t_end(P);
        ++L;
    }
    if (use_tmma) {
        // operand blocks of every (step, row), then the correlation GEMM for all steps
        const int nprn = static_cast<int>(P->prns.size());
        t_begin(P, ACQ_KERNEL_FRONTEND);
        klog(P, nullptr, "k_tile_stubs");
        // the column stage's accumulator edges are zeroed by the same launch
        EdgeZero ez{};
        if (P->tmaH > 0) {
            ez.acc = P->accb.as<float>();
            ez.rows = static_cast<int64_t>(n) * g.ndop;
            ez.spc = g.spc;
            ez.spc_eff = g.spc_eff;
            ez.W = P->col_k1 ? P->k1W : P->tmaW;
            ez.H = P->tmaH;
            ez.n_bound = (g.spc + ez.W - 1) / ez.W + 1;
        }
        k_tile_stubs<<<dim3(G, g.n_nc), kTmmaStubThreads, 0, st>>>(
            d_in, dtype, seg_len, G, g.nb, g.n_coh, g.bs, P->col_pre ? 1 : 0, use_if, if_step, a.d_if_off,
            P->fftD.tw, P->stubs.as<uint8_t>(), P->invsc.as<float>(), ez);
        t_end(P);
        ++L;
        TileMmaParams tp{};
        tp.stubs = P->stubs.as<uint8_t>(); tp.inv_scale = P->invsc.as<float>(); tp.codes = P->codes.as<int8_t>();
        tp.slots = a.d_slots; tp.T = P->Tall.as<float2>(); tp.t_step_stride = static_cast<int64_t>(nprn) * G * g.spc;
        tp.n = n; tp.G = G; tp.nb = g.nb; tp.bs = g.bs; tp.spc = g.spc;
        tp.n_chunks = (n * g.nb + kTmmaRows - 1) / kTmmaRows;
        tp.units = g.n_nc * G;
        tp.cpc = std::max(1, std::min(tp.units, P->tmmaSms / tp.n_chunks));
        tp.err = P->errflag.as<int>();
        t_begin(P, ACQ_KERNEL_TILE);
        klog(P, nullptr, "k_tile_mma");
        launch(pdl, k_tile_mma, dim3(tp.n_chunks * tp.cpc), dim3(kTmmaThreads), P->smem_tmma, st, tp);
        t_end(P);
        ++L;
    }
    if (use_tma) {
        // coherent tiles of every step in one launch, then the TMA-staged column stage
        const int nprn = static_cast<int>(P->prns.size());
        const float2* spectra = P->S.as<float2>();
        if (!use_tmma && P->col_pre && g.n_coh > 1) {   // one coherent period: the first pass is the identity
            t_begin(P, ACQ_KERNEL_FRONTEND);
            klog(P, nullptr, "k_doppler_prepass");
            k_doppler_prepass<<<dim3((g.fft_tile + 127) / 128, g.nb * g.n_coh, g.n_nc), 128, 0, st>>>(
                P->S.as<float2>(), P->U.as<float2>(), G, g.nb, g.n_coh, g.fft_tile, P->fftD.tw);
            t_end(P);
            ++L;
            spectra = P->U.as<float2>();
        }
        if (!use_tmma) {
            t_begin(P, ACQ_KERNEL_TILE);
            klog(P, (const void*)P->tile_fs, "k_tile_fs");
            P->tile_fs<<<dim3(tile_grid_x(P), n, g.n_nc), P->tileThreads, P->smem_tile_fs, st>>>(
                spectra, P->conj.as<float2>(), a.d_slots, G, g.nb, g.bs, g.spc, P->twT.as<float2>(), P->tileNF,
                P->Tall.as<float2>(), static_cast<int64_t>(nprn) * G * g.spc, P->tileFS);
            t_end(P);
            ++L;
        }
        if (P->tmaH > 0 && !use_tmma) {   // (the tensor-core path zeroes them in k_tile_stubs)
            const int wc = P->col_k1 ? P->k1W : P->tmaW;
            const int n_bound = (g.spc + wc - 1) / wc + 1;
            const int64_t rows = static_cast<int64_t>(n) * g.ndop;
            const int64_t total = rows * n_bound * 2 * P->tmaH;
            klog(P, nullptr, "k_zero_edges");
            launch(pdl, k_zero_edges, dim3(static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 4096))),
                   dim3(256), 0, st, P->accb.as<float>(), rows, g.spc, g.spc_eff, wc, P->tmaH, n_bound);
            ++L;
        }
        ColTmaParams cp{};
        cp.spc = g.spc; cp.spc_eff = g.spc_eff; cp.n_nc = g.n_nc; cp.W = P->tmaW; cp.halo = P->tmaH;
        cp.box_rows = P->tmaBoxRows; cp.n_boxes = P->tmaBoxes; cp.n_cblk = (g.spc + P->tmaW - 1) / P->tmaW;
        cp.n_items = n * cp.n_cblk; cp.rows_per_step = nprn * g.ndop; cp.n1 = g.n_coh;
        cp.twD = P->fftD.tw; cp.drift = P->drift.as<int>(); cp.acc = P->accb.as<float>(); cp.err = P->errflag.as<int>();
        cp.wait_polls = P->k1WaitPolls;
        t_begin(P, ACQ_KERNEL_COLUMN);
        if (P->col_k1) {
            cp.W = P->k1W;
            cp.n_cblk = (g.spc + P->k1W - 1) / P->k1W;
            cp.n_items = n * g.n_coh * cp.n_cblk;
            // the extraction's statistics come from this stage (no separate pass over the surface)
            const int n_bound = cp.n_cblk + 1;
            cp.rowpart = P->rowpart.as<double>();
            cp.peakpart = P->peakpart.as<unsigned long long>();
            cp.npk = g.n_coh * cp.n_cblk + (P->tmaH > 0 ? n_bound : 0);
            const int grid = std::max(1, std::min(P->k1Grid, cp.n_items));
            klog(P, (const void*)P->col_k1, "k_col_tma_k1");
            launch(pdl, P->col_k1, dim3(grid), dim3(128), P->smem_col_k1, st, P->tmapK1, cp);
            t_end(P);
            ++L;
            if (P->tmaH > 0) {
                t_begin(P, ACQ_KERNEL_STATS);
                klog(P, nullptr, "k_edge_peaks");
                launch(pdl, k_edge_peaks, dim3(n_bound, n), dim3(128), 0, st, P->accb.as<float>(), g.ndop, g.spc,
                       g.spc_eff, P->k1W, P->tmaH, n_bound, g.n_coh * cp.n_cblk, cp.npk,
                       P->peakpart.as<unsigned long long>());
                t_end(P);
                ++L;
            }
            stats_nct = cp.n_cblk;
            stats_npk = cp.npk;
        } else {
            const int grid = std::max(1, std::min(P->tmaGrid, cp.n_items));
            klog(P, (const void*)P->col_tma, "k_col_tma");
            P->col_tma<<<grid, kThreads, P->smem_col_tma, st>>>(P->tmapT, cp);
            t_end(P);
            ++L;
        }
    }
    if (use_tmma_step) {
        t_begin(P, ACQ_KERNEL_FRONTEND);
        klog(P, nullptr, "k_tile_stubs");
        k_tile_stubs<<<dim3(G, g.n_nc), kTmmaStubThreads, 0, st>>>(
            d_in, dtype, seg_len, G, g.nb, g.n_coh, g.bs, 0, use_if, if_step, a.d_if_off, P->fftD.tw,
            P->stubs.as<uint8_t>(), P->invsc.as<float>(), EdgeZero{});
        t_end(P);
        ++L;
    }
    for (int m = 0; m < ((use_fused || use_tma) ? 0 : g.n_nc); ++m) {
        const float2* Sm = P->S.as<float2>() + (size_t)m * G * g.fft_tile;
        t_begin(P, ACQ_KERNEL_TILE);
        if (use_tmma_step) {
            TileMmaParams tp{};
            const size_t row_bytes = tmma_row_bytes(g.bs);
            tp.stubs = P->stubs.as<uint8_t>() + (size_t)m * G * row_bytes;
            tp.inv_scale = P->invsc.as<float>() + (size_t)m * G;
            tp.codes = P->codes.as<int8_t>(); tp.slots = a.d_slots; tp.T = P->T.as<float2>(); tp.t_step_stride = 0;
            tp.n = n; tp.G = G; tp.nb = g.nb; tp.bs = g.bs; tp.spc = g.spc;
            tp.n_chunks = (n * g.nb + kTmmaRows - 1) / kTmmaRows;
            tp.units = G;
            tp.cpc = std::max(1, std::min(tp.units, P->tmmaSms / tp.n_chunks));
            tp.err = P->errflag.as<int>();
            klog(P, nullptr, "k_tile_mma");
            k_tile_mma<<<tp.n_chunks * tp.cpc, kTmmaThreads, P->smem_tmma, st>>>(tp);
        } else if (P->tile_fs) {
            klog(P, (const void*)P->tile_fs, "k_tile_fs");
            P->tile_fs<<<dim3(tile_grid_x(P), n), P->tileThreads, P->smem_tile_fs, st>>>(
                Sm, P->conj.as<float2>(), a.d_slots, G, g.nb, g.bs, g.spc, P->twT.as<float2>(), P->tileNF,
                P->T.as<float2>(), 0, P->tileFS);
        } else {
            klog(P, nullptr, "k_tile");
            k_tile<<<dim3(G, n), kThreads, P->smem_tile, st>>>(Sm, P->conj.as<float2>(), a.d_slots, G, g.nb,
                                                               g.bs, g.spc, P->fftF, P->tileB, P->T.as<float2>());
        }
        t_end(P);
        ++L;
        const int* dr = P->drift.as<int>() + (size_t)m * g.ndop;
        const int first = m == 0;
        const bool last = m == g.n_nc - 1;
        t_begin(P, ACQ_KERNEL_COLUMN);
        if (g.path == 0 && P->dft_mma) {
            DftMmaParams dp{};
            dp.T = P->T.as<float2>(); dp.spc = g.spc; dp.nd = g.ndop; dp.spc_eff = g.spc_eff; dp.n_pad = P->dftNpad;
            dp.ksteps = P->dftKsteps; dp.first = first; dp.has_drift = P->step_has_drift[m]; dp.drift = dr;
            dp.acc = P->accb.as<float>(); dp.B = P->dftB.as<uint8_t>();
            int sl = P->mma_scale_log2;
            if (sl == 127) sl = dtype == ACQ_CI16 ? -10 : dtype == ACQ_CI8 ? -2 : 0;
            dp.scale = std::ldexp(1.0f, sl);
            dp.err = P->errflag.as<int>();
            klog(P, (const void*)P->dft_mma, "k_col_dft_mma");
            P->dft_mma<<<dim3((g.spc + kDftCols - 1) / kDftCols, n), kDftThreads, P->smem_dft, st>>>(dp);
        } else if (g.path == 0 && P->col_fs) {
            const int W = P->Wfs;
            klog(P, (const void*)P->col_fs, "k_col_simple_fs");
            P->col_fs<<<dim3((g.spc + W - 1) / W, n), kThreads, P->smem_col_fs, st>>>(
                P->T.as<float2>(), g.spc, W, P->fftD.tw, dr, first, P->step_has_drift[m], P->accb.as<float>(),
                g.spc_eff);
        } else if (g.path == 0) {
            const int W = P->Wsimple;
            klog(P, nullptr, "k_col_simple");
            k_col_simple<<<dim3((g.spc + W - 1) / W, n), kThreads, P->smem_simple, st>>>(
                P->T.as<float2>(), g.ndop, g.spc, W, P->fftD, dr, first, P->accb.as<float>(), g.spc_eff);
        } else if (g.path == 2 && P->rot_mma) {
            RotMmaParams rp{};
            rp.T = P->T.as<float2>(); rp.spc = g.spc; rp.spc_eff = g.spc_eff; rp.bs = g.bs; rp.R = g.R;
            rp.combos = P->combos; rp.use_max = (P->combos > 1 || g.n_be > 1) ? 1 : 0;
            rp.first = first | (last ? 2 : 0); rp.twD = P->fftD.tw; rp.pats = P->pats.as<float>();
            rp.slots = a.d_slots; rp.drift = dr; rp.acc = P->accb.as<float>(); rp.win = P->winb.as<uint16_t>();
            int sl = P->mma_scale_log2;
            if (sl == 127) sl = dtype == ACQ_CI16 ? -10 : dtype == ACQ_CI8 ? -2 : 0;
            rp.scale = std::ldexp(1.0f, sl);
            rp.err = P->errflag.as<int>();
            klog(P, (const void*)P->rot_mma, "k_rot_mma");
            P->rot_mma<<<dim3((g.spc + kRotMmaW - 1) / kRotMmaW, n), 256, P->smem_mma, st>>>(rp);
        } else if (g.path == 2 && P->rot_sb) {
            const int W = P->Wrsb;
            const int use_max = (P->combos > 1 || g.n_be > 1) ? 1 : 0;
            klog(P, (const void*)P->rot_sb, "k_col_rot_sb");
            P->rot_sb<<<dim3((g.spc + W - 1) / W, n), P->threads_rsb, P->smem_rsb, st>>>(
                P->T.as<float2>(), g.spc, P->fftD.tw, P->pats.as<float>(), g.bs, g.R, P->combos, g.n_be,
                P->edge_step, use_max, a.d_slots, dr, first | (last ? 2 : 0), P->accb.as<float>(),
                P->winb.as<uint16_t>(), g.spc_eff);
        } else if (g.path == 1 && P->sign_sb) {
            const int W = P->Wssb;
            klog(P, (const void*)P->sign_sb, "k_col_sign_sb");
            P->sign_sb<<<dim3((g.spc + W - 1) / W, n), P->threads_ssb, P->smem_ssb, st>>>(
                P->T.as<float2>(), g.spc, P->fftD.tw, P->pats.as<float>(), g.n_coh, g.n_be, P->edge_step, a.d_slots,
                dr, first | (last ? 2 : 0), P->accb.as<float>(), P->winb.as<uint16_t>(), g.spc_eff);
        } else if (g.path == 1 && P->sign_fs) {
            const int W = P->Wsfs;
            klog(P, (const void*)P->sign_fs, "k_col_sign_fs");
            P->sign_fs<<<dim3((g.spc + W - 1) / W, n), kThreads, P->smem_sfs, st>>>(
                P->T.as<float2>(), g.spc, W, P->fftD.tw, P->pats.as<float>(), P->n_pat, g.n_coh, g.ndb, g.n_be,
                P->edge_step, a.d_slots, dr, first | (last ? 2 : 0), P->accb.as<float>(), P->winb.as<uint16_t>(),
                g.spc_eff);
        } else if (g.path == 2 && P->rot_fs) {
            const int W = P->Wsfs;
            const int use_max = (P->combos > 1 || g.n_be > 1) ? 1 : 0;
            klog(P, (const void*)P->rot_fs, "k_col_rot_fs");
            P->rot_fs<<<dim3((g.spc + W - 1) / W, n), kThreads, P->smem_sfs, st>>>(
                P->T.as<float2>(), g.spc, W, P->fftD.tw, P->pats.as<float>(), g.n_coh, g.nb, g.bs, g.R, P->combos,
                g.n_be, P->edge_step, use_max, a.d_slots, dr, first, P->accb.as<float>(),
                P->winb.as<uint16_t>(), g.spc_eff);
        } else if (g.path == 1) {
            const int W = P->Wsign;
            klog(P, nullptr, "k_col_sign");
            k_col_sign<<<dim3((g.spc + W - 1) / W, n), kThreads, P->smem_sign, st>>>(
                P->T.as<float2>(), g.ndop, g.spc, W, P->fftD, P->pats.as<float>(), P->n_pat, g.n_coh, g.ndb, g.n_be,
                P->edge_step, a.d_slots, dr, first, P->accb.as<float>(), P->winb.as<uint16_t>(), g.spc_eff);
        } else {
            const int W = P->Wsign;
            const int use_max = (P->combos > 1 || g.n_be > 1) ? 1 : 0;
            klog(P, nullptr, "k_col_rot");
            k_col_rot<<<dim3((g.spc + W - 1) / W, n), kThreads, P->smem_sign, st>>>(
                P->T.as<float2>(), g.ndop, g.spc, W, P->fftD, P->pats.as<float>(), g.n_coh, g.nb, g.bs, g.R, P->combos,
                g.n_be, P->edge_step, use_max, a.d_slots, dr, first, P->accb.as<float>(),
                P->winb.as<uint16_t>(), g.spc_eff);
        }
        t_end(P);
        ++L;
    }
    const int streamed_rot = (g.n_nc == 1 && g.R > 1) ? 1 : 0;
    if (stats_npk == 0) {
        t_begin(P, ACQ_KERNEL_STATS);
        klog(P, nullptr, "k_stats");
        k_stats<<<dim3(P->nct, n), kThreads, 0, st>>>(P->accb.as<float>(), g.ndop, g.spc_eff, g.spc, g.R, streamed_rot,
                                                      P->rowpart.as<double>(), P->colsum.as<double>(),
                                                      P->peakpart.as<unsigned long long>());
        t_end(P);
        ++L;
    }
    ExtractParams EP{};
    EP.ndop = g.ndop; EP.spc = g.spc; EP.spc_eff = g.spc_eff; EP.nb = g.nb; EP.bs = g.bs; EP.R = g.R;
    EP.n_coh = g.n_coh; EP.ndb = g.ndb; EP.n_be = g.n_be; EP.n_nc = g.n_nc; EP.path = g.path;
    EP.combos = P->combos; EP.n_pat = P->n_pat; EP.streamed_rot = streamed_rot;
    EP.noise_estimator = g.noise_estimator;
    EP.samples_per_chip = static_cast<int>(std::floor(P->desc.sampling_freq_hz / P->sys->code_freq));
    EP.interp = (flags & ACQ_FLAG_SUBSAMPLE_INTERP) ? 1 : 0;
    EP.nct = stats_npk ? stats_nct : P->nct;
    EP.npk = stats_npk ? stats_npk : P->nct;
    EP.rowmode = stats_npk ? 1 : 0;
    EP.fs = P->desc.sampling_freq_hz; EP.fc = P->sys->code_freq; EP.code_length = P->sys->code_length;
    EP.t_coh = g.n_coh * (static_cast<double>(P->sys->code_length) / P->sys->code_freq);
    EP.doppler_first = g.doppler_first; EP.doppler_step = g.doppler_step; EP.cfar_thr = g.cfar_thr;
    t_begin(P, ACQ_KERNEL_EXTRACT);
    klog(P, nullptr, "k_extract");
    launch(pdl && stats_npk > 0, k_extract, dim3(n), dim3(kThreads), 0, st, P->accb.as<float>(),
           P->winb.as<uint16_t>(), P->rowpart.as<double>(), P->colsum.as<double>(),
           P->peakpart.as<unsigned long long>(), a.d_prn_ids, EP, a.d_res);
    t_end(P);
    ++L;
    if (g.R > 1) {
        t_begin(P, ACQ_KERNEL_SECONDARY);
        klog(P, nullptr, "k_secondary_prompt");
        k_secondary_prompt<<<dim3(n, g.R), kThreads, 0, st>>>(d_in, dtype, P->chips.as<int8_t>(), P->chips_len,
                                                              a.d_slots, g.spc, P->desc.sampling_freq_hz,
                                                              P->sys->code_freq, a.interm_freq, a.d_res,
                                                              P->zs.as<double2>(), g.R);
        klog(P, nullptr, "k_secondary_argmax");
        k_secondary_argmax<<<(n + 127) / 128, 128, 0, st>>>(P->zs.as<double2>(), P->sec.as<int8_t>(), g.R,
                                                            a.d_res, n);
        t_end(P);
        L += 2;
    }
    CK(cudaGetLastError());
    return L;
}

void enqueue_acquire(acq_plan* P, const void* d_in, int dtype, int64_t n_samples, const int32_t* prns, int n,
                     double interm_freq, uint32_t flags) {
    std::vector<int> slots;
    std::vector<float> offs;
    LaunchArgs a;
    prepare_request(P, n_samples, prns, n, interm_freq, slots, offs, a.use_if, a.if_step);
    CK(cudaSetDevice(P->device));
#ifdef ACQ_BOUNDS_CHECK
    if (d_in != P->input.p) bc::add(d_in, static_cast<size_t>(n_samples) * sample_bytes(dtype));   // caller's buffer
#endif
    cudaStream_t st = P->stream;
    // [slots (n) | PRN ids (n) | IF offsets (n_nc)] in one copy from page-locked memory
    const size_t bytes = sizeof(int) * 2 * static_cast<size_t>(n) + sizeof(float) * offs.size();
    const int hb = P->hreq_next;
    P->hreq_next ^= 1;
    if (P->hreq_ev[hb]) CK(cudaEventSynchronize(P->hreq_ev[hb]));
    else CK(cudaEventCreateWithFlags(&P->hreq_ev[hb], cudaEventDisableTiming));
    P->hreq[hb].ensure(bytes);
    P->dreq.ensure(bytes);
    char* h = static_cast<char*>(P->hreq[hb].p);
    std::memcpy(h, slots.data(), sizeof(int) * n);
    std::memcpy(h + sizeof(int) * n, prns, sizeof(int) * n);
    if (!offs.empty()) std::memcpy(h + sizeof(int) * 2 * n, offs.data(), sizeof(float) * offs.size());
    CK(cudaMemcpyAsync(P->dreq.p, h, bytes, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(P->hreq_ev[hb], st));
    a.n = n;
    char* d = P->dreq.as<char>();
    a.d_slots = reinterpret_cast<const int*>(d);
    a.d_prn_ids = reinterpret_cast<const int*>(d + sizeof(int) * n);
    a.d_if_off = reinterpret_cast<const float*>(d + sizeof(int) * 2 * n);
    a.interm_freq = interm_freq;
    a.flags = flags;
    a.d_res = P->res.as<acq_result>();
    acq_plan::RequestKey key;
    key.d_in = d_in; key.dreq = P->dreq.p; key.dtype = dtype; key.n = n; key.use_if = a.use_if; key.flags = flags;
    key.if_step = a.if_step; key.interm = interm_freq; key.version = P->version;
    if (P->timing || getenv_flag("ACQ_NO_GRAPH")) {
        P->launches = launch_sequence(P, st, d_in, dtype, a);
    } else if (P->gexec && key == P->graph_key) {
        CK(cudaGraphLaunch(P->gexec, st));
        P->launches = P->graph_launches;
    } else if (key == P->last_key) {   // second identical request in a row: capture, then replay
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int64_t L = 0;
        try {
            L = launch_sequence(P, st, d_in, dtype, a);
        } catch (...) {
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            throw;
        }
        CK(cudaStreamEndCapture(st, &graph));
        if (P->gexec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(P->gexec, graph, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(P->gexec);
                P->gexec = nullptr;
            }
        }
        cudaError_t e = P->gexec ? cudaSuccess : cudaGraphInstantiate(&P->gexec, graph, 0);
        cudaGraphDestroy(graph);
        CK(e);
        P->graph_key = key;
        P->graph_launches = L;
        CK(cudaGraphLaunch(P->gexec, st));
        P->launches = L;
    } else {
        P->launches = launch_sequence(P, st, d_in, dtype, a);
    }
    P->last_key = key;
    P->last_n = n;
    P->last_flags = flags;
    P->req_prns.assign(prns, prns + n);
}

}  // namespace

struct acq_batch {
    int device = 0;
    cudaStream_t s0 = nullptr;
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> events;
    struct Item {
        acq_plan* plan;
        int dtype;
        int64_t n_samples;
        size_t in_off, in_bytes;
        int n, res_off, branch;
        LaunchArgs args;
        size_t meta_slots, meta_ids, meta_if;
    };
    std::vector<Item> items;
    DevBuf arena, meta, res;
    int total_res = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
};

namespace {

void batch_build(acq_batch* B, const acq_batch_item* items, int n_items) {
    if (n_items <= 0) throw AcqError(ACQ_ERR_ARGUMENT, "empty batch");
    B->device = items[0].plan ? items[0].plan->device : 0;
    std::vector<acq_plan*> plans;
    std::vector<unsigned char> hmeta;
    auto push = [&](const void* p, size_t bytes) {
        size_t off = (hmeta.size() + 15) & ~size_t(15);
        hmeta.resize(off + bytes);
        if (bytes) std::memcpy(hmeta.data() + off, p, bytes);
        return off;
    };
    size_t arena = 0;
    for (int i = 0; i < n_items; ++i) {
        const acq_batch_item& it = items[i];
        if (!it.plan || !it.prns) throw AcqError(ACQ_ERR_ARGUMENT, "batch item " + std::to_string(i) + ": null plan or prns");
        if (it.plan->device != B->device) throw AcqError(ACQ_ERR_ARGUMENT, "batch plans must share one device");
        if (it.flags & ACQ_FLAG_STORE_POWER_BINS)
            throw AcqError(ACQ_ERR_ARGUMENT, "store_power_bins is not available in a batch");
        acq_batch::Item m{};
        m.plan = it.plan;
        m.dtype = it.dtype;
        m.n_samples = it.n_samples;
        const Geometry& g = it.plan->g;
        const int64_t need = static_cast<int64_t>(g.n_nc) * g.n_coh * g.spc;
        m.in_bytes = sample_bytes(it.dtype) * static_cast<size_t>(std::min<int64_t>(it.n_samples, need));
        m.in_off = arena;
        arena += (m.in_bytes + 255) & ~size_t(255);
        std::vector<int> slots;
        std::vector<float> offs;
        prepare_request(it.plan, it.n_samples, it.prns, it.n_prns, it.interm_freq_hz, slots, offs, m.args.use_if,
                        m.args.if_step);
        m.n = it.n_prns;
        m.meta_slots = push(slots.data(), sizeof(int) * slots.size());
        m.meta_ids = push(it.prns, sizeof(int) * it.n_prns);
        m.meta_if = push(offs.data(), sizeof(float) * offs.size());
        m.args.n = it.n_prns;
        m.args.interm_freq = it.interm_freq_hz;
        m.args.flags = it.flags;
        m.res_off = B->total_res;
        B->total_res += it.n_prns;
        auto pit = std::find(plans.begin(), plans.end(), it.plan);
        m.branch = static_cast<int>(pit - plans.begin());
        if (pit == plans.end()) plans.push_back(it.plan);
        B->items.push_back(m);
    }
    CK(cudaSetDevice(B->device));
    CK(cudaStreamCreateWithFlags(&B->s0, cudaStreamNonBlocking));
    B->branch.resize(plans.size());
    for (auto& s : B->branch) CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    B->events.resize(2 * plans.size());
    for (auto& e : B->events) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    B->arena.ensure(std::max<size_t>(arena, 256));
    B->meta.ensure(std::max<size_t>(hmeta.size(), 16));
    CK(cudaMemcpy(B->meta.p, hmeta.data(), hmeta.size(), cudaMemcpyHostToDevice));
    B->res.ensure(sizeof(acq_result) * B->total_res);
    unsigned char* mb = B->meta.as<unsigned char>();
    for (auto& m : B->items) {
        m.args.d_slots = reinterpret_cast<const int*>(mb + m.meta_slots);
        m.args.d_prn_ids = reinterpret_cast<const int*>(mb + m.meta_ids);
        m.args.d_if_off = reinterpret_cast<const float*>(mb + m.meta_if);
        m.args.d_res = B->res.as<acq_result>() + m.res_off;
    }
    // every plan's stream work is finished before the capture reuses its buffers
    for (acq_plan* P : plans) CK(cudaStreamSynchronize(P->stream));
    std::vector<bool> timing(plans.size());
    for (size_t b = 0; b < plans.size(); ++b) {
        timing[b] = plans[b]->timing;
        plans[b]->timing = false;
    }
    CK(cudaStreamBeginCapture(B->s0, cudaStreamCaptureModeThreadLocal));
    int64_t L = 0;
    try {
        for (size_t b = 0; b < plans.size(); ++b) {
            CK(cudaEventRecord(B->events[2 * b], B->s0));
            CK(cudaStreamWaitEvent(B->branch[b], B->events[2 * b], 0));
        }
        for (const auto& m : B->items)
            L += launch_sequence(m.plan, B->branch[m.branch], B->arena.as<unsigned char>() + m.in_off, m.dtype, m.args);
        for (size_t b = 0; b < plans.size(); ++b) {
            CK(cudaEventRecord(B->events[2 * b + 1], B->branch[b]));
            CK(cudaStreamWaitEvent(B->s0, B->events[2 * b + 1], 0));
        }
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(B->s0, &g);
        if (g) cudaGraphDestroy(g);
        for (size_t b = 0; b < plans.size(); ++b) plans[b]->timing = timing[b];
        throw;
    }
    CK(cudaStreamEndCapture(B->s0, &B->graph));
    for (size_t b = 0; b < plans.size(); ++b) plans[b]->timing = timing[b];
    CK(cudaGraphInstantiate(&B->exec, B->graph, 0));
    B->launches = L;
}

void batch_free(acq_batch* B) {
    if (!B) return;
    cudaSetDevice(B->device);
    if (B->s0) cudaStreamSynchronize(B->s0);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    for (auto e : B->events) cudaEventDestroy(e);
    for (auto s : B->branch) cudaStreamDestroy(s);
    if (B->s0) cudaStreamDestroy(B->s0);
    B->arena.reset();
    B->meta.reset();
    B->res.reset();
    delete B;
}

void fetch(acq_plan* P, acq_result* results, float* power_bins) {
    const Geometry& g = P->g;
    CK(cudaSetDevice(P->device));
    // staging: [0, 8) the error word, [8, ...) the result records
    const size_t res_bytes = (results && P->last_n > 0) ? sizeof(acq_result) * P->last_n : 0;
    P->hstage.ensure(8 + res_bytes);
    int* herr = static_cast<int*>(P->hstage.p);
    acq_result* hres = reinterpret_cast<acq_result*>(static_cast<char*>(P->hstage.p) + 8);
    *herr = 0;
    if (P->errflag.p) CK(cudaMemcpyAsync(herr, P->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, P->stream));
    if (res_bytes) CK(cudaMemcpyAsync(hres, P->res.p, res_bytes, cudaMemcpyDeviceToHost, P->stream));
    if (power_bins && P->last_n > 0 && (P->last_flags & ACQ_FLAG_STORE_POWER_BINS)) {
        const size_t cells = (size_t)P->last_n * g.ndop * g.spc_eff;
        const void* src = P->accb.p;
        if (P->last_flags & ACQ_FLAG_POWER_BINS_CHIP_SORTED) {
            P->sorted.ensure(sizeof(float) * cells);
            const int64_t rows = (int64_t)P->last_n * g.ndop;
            k_gather_cols<<<std::min<int64_t>((rows * g.spc_eff + 255) / 256, 8192), 256, 0, P->stream>>>(
                P->accb.as<float>(), rows, g.spc_eff, P->chipperm.as<int32_t>(), P->sorted.as<float>());
            CK(cudaGetLastError());
            src = P->sorted.p;
        }
        CK(cudaMemcpyAsync(power_bins, src, sizeof(float) * cells, cudaMemcpyDeviceToHost, P->stream));
    }
    CK(cudaStreamSynchronize(P->stream));
    t_collect(P);
#ifdef ACQ_BOUNDS_CHECK
    bc::check();
#endif
    if (res_bytes) std::memcpy(results, hres, res_bytes);
    if (P->errflag.p) {
        const int e = *herr;
        if (e != 0) {
            CK(cudaMemset(P->errflag.p, 0, sizeof(int)));
            throw AcqError(ACQ_ERR_TIMEOUT, "a bounded wait for a TMA tile gave up (device error " +
                                                std::to_string(e) + ")");
        }
    }
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return ACQ_OK;
    } catch (const AcqError& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return ACQ_ERR_ALLOC;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return ACQ_ERR_ARGUMENT;
    }
}

void fill_geometry(const Geometry& g, const SystemInfo& s, int n_prns, acq_geometry* o) {
    o->samples_per_code = g.spc;
    o->samples_per_code_eff = g.spc_eff;
    o->num_blocks = g.nb;
    o->block_size = g.bs;
    o->fft_size = g.fft_size;
    o->num_coherently_integrated_code_periods = g.n_coh;
    o->num_data_bits = g.ndb;
    o->bit_edge_search_steps = g.n_be;
    o->num_noncoherent_accumulations = g.n_nc;
    o->num_doppler_bins = g.ndop;
    o->num_secondary_rotations = g.R;
    o->bit_period_codes = g.bit_period_codes;
    o->num_prns = n_prns;
    o->path = g.path;
    o->doppler_first_hz = g.doppler_first;
    o->doppler_step_hz = g.doppler_step;
    o->code_length = s.code_length;
    o->code_freq_hz = s.code_freq;
    o->center_freq_hz = s.center_freq;
    o->cfar_threshold_pfa001 = g.cfar_thr;
}

}  // namespace

void acq::set_last_error(const std::string& msg) { g_last_error = msg; }

extern "C" {

void acq_plan_desc_init(acq_plan_desc* d) {
    if (!d) return;
    d->system = ACQ_GPS_L1CA;
    d->sampling_freq_hz = 0.0;
    d->min_doppler_coverage_hz = 7000.0;
    d->num_coherently_integrated_code_periods = 1;
    d->bit_edge_search_steps = 1;
    d->num_noncoherent_accumulations = 1;
    d->noise_estimator = ACQ_NOISE_OPPOSITE_ROW;
    d->use_secondary_code = 1;
    d->max_secondary_code_rotations = 32;
    d->device = 0;
}

int acq_plan_query(const acq_plan_desc* desc, acq_geometry* out) {
    return guarded([&] {
        if (!desc || !out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        Geometry g = compute_geometry(*desc);
        fill_geometry(g, system_info(desc->system), 0, out);
    });
}

int acq_plan_create(const acq_plan_desc* desc, const int32_t* prns, int32_t n_prns, const int8_t* codes, acq_plan** out) {
    return guarded([&] {
        if (!desc || !out || (!prns && n_prns > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        if (n_prns <= 0) throw AcqError(ACQ_ERR_ARGUMENT, "prns must not be empty");
        std::unique_ptr<acq_plan> P(new acq_plan());
        P->desc = *desc;
        P->g = compute_geometry(*desc);
        P->g.fft_tile = choose_fft_tile(P->g);
        P->sys = &system_info(desc->system);
        for (int i = 0; i < n_prns; ++i) {
            if (prns[i] < 1 || prns[i] > P->sys->max_prn)
                throw AcqError(ACQ_ERR_ARGUMENT, std::string(P->sys->name) + " PRN must be in 1:" +
                                                     std::to_string(P->sys->max_prn) + ", got " + std::to_string(prns[i]));
            P->prns.push_back(prns[i]);
        }
        P->device = desc->device;
        try {
            plan_setup(P.get(), prns, n_prns, codes);
        } catch (...) {
            acq_plan_destroy(P.release());
            throw;
        }
        *out = P.release();
    });
}

int acq_plan_destroy(acq_plan* P) {
    if (!P) return ACQ_OK;
    cudaSetDevice(P->device);
    if (P->stream) cudaStreamSynchronize(P->stream);
    for (DevBuf* b : {&P->twF, &P->twD, &P->twT, &P->U, &P->codes, &P->conj, &P->chips, &P->pats, &P->drift, &P->sec, &P->if_off,
                      &P->input, &P->S, &P->T, &P->accb, &P->winb, &P->rowpart, &P->colsum, &P->peakpart, &P->zs,
                      &P->res, &P->slots, &P->prn_ids, &P->Tall, &P->errflag, &P->chipperm, &P->sorted,
                      &P->dftB, &P->dreq})
        b->reset();
    P->hstage.reset();
    if (P->gexec) cudaGraphExecDestroy(P->gexec);
    for (int i = 0; i < 2; ++i) {
        P->hreq[i].reset();
        if (P->hreq_ev[i]) cudaEventDestroy(P->hreq_ev[i]);
    }
    for (cudaEvent_t e : P->ev_start) cudaEventDestroy(e);
    for (cudaEvent_t e : P->ev_stop) cudaEventDestroy(e);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
    return ACQ_OK;
}

int acq_plan_get_geometry(const acq_plan* P, acq_geometry* out) {
    return guarded([&] {
        if (!P || !out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        fill_geometry(P->g, *P->sys, static_cast<int>(P->prns.size()), out);
    });
}

int acq_plan_doppler_freqs(const acq_plan* P, double* out) {
    return guarded([&] {
        if (!P || !out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        std::memcpy(out, P->g.doppler_freqs.data(), sizeof(double) * P->g.ndop);
    });
}

// acquire! with an empty PRN list (src/acquire.jl:54-89): the signal length is still checked,
// then there is nothing to compute and the result list is empty.
bool empty_request(acq_plan* P, int64_t n_samples, int32_t n_prns, uint32_t flags) {
    if (n_prns < 0) throw AcqError(ACQ_ERR_ARGUMENT, "n_prns must be >= 0");
    if (n_prns > 0) return false;
    const Geometry& g = P->g;
    const int64_t seg_len = static_cast<int64_t>(g.n_coh) * g.spc;
    const int64_t nseg = n_samples / seg_len;
    if (nseg < g.n_nc)
        throw AcqError(ACQ_ERR_SHORT_SIGNAL, "Signal has " + std::to_string(n_samples) + " samples → " +
                                                 std::to_string(nseg) + " full segments of " + std::to_string(seg_len) +
                                                 ", but plan.num_noncoherent_accumulations=" + std::to_string(g.n_nc) +
                                                 ". Provide a longer signal.");
    P->last_n = 0;
    P->last_flags = flags;
    return true;
}

namespace {
// Device address of a page-locked, device-mapped host buffer; null for pageable or device memory
// and with ACQ_NO_ZERO_COPY=1 (every upload then goes through the copy engines).
const void* mapped_host(const void* h) {
    if (getenv_flag("ACQ_NO_ZERO_COPY")) return nullptr;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

struct Upload {
    const void* host;     // caller's buffer
    const void* mapped;   // its device address (mapped_host), or null
    void* dst;            // device destination
    size_t bytes;
};

// Host -> device copies of recordings. Mapped buffers whose addresses are 16-byte aligned go
// through k_copy_in (one launch per kCopySegs of them: at 1.6 MB and up, the SMs' loads across the
// host link outrun a copy-engine transfer), the others through cudaMemcpyAsync. Enqueued on st.
void upload_inputs(const std::vector<Upload>& ups, int device, cudaStream_t st) {
    CopyList L{};
    int sms = 0;
    auto flush = [&] {
        if (!L.n) return;
        if (!sms) CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        const int64_t chunk = static_cast<int64_t>(kCopyThreads) * kCopyUnroll;
        const int64_t blocks = (L.vec[L.n] + chunk - 1) / chunk;
        const int grid = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(blocks, 8ll * sms)));
        k_copy_in<<<grid, kCopyThreads, 0, st>>>(L);
        CK(cudaGetLastError());
        L = CopyList{};
    };
    for (const Upload& u : ups) {
        if (!u.bytes) continue;
        const bool aligned = ((reinterpret_cast<uintptr_t>(u.mapped) | reinterpret_cast<uintptr_t>(u.dst)) & 15) == 0;
        if (u.mapped && aligned) {
            L.src[L.n] = static_cast<const unsigned char*>(u.mapped);
            L.dst[L.n] = static_cast<unsigned char*>(u.dst);
            L.tail[L.n] = static_cast<int>(u.bytes & 15);
            L.vec[L.n + 1] = L.vec[L.n] + static_cast<int64_t>(u.bytes >> 4);
            if (++L.n == kCopySegs) flush();
        } else {
            CK(cudaMemcpyAsync(u.dst, u.host, u.bytes, cudaMemcpyHostToDevice, st));
        }
    }
    flush();
}
}  // namespace

int acq_acquire(acq_plan* P, const void* samples, int32_t dtype, int64_t n_samples, const int32_t* prns,
                int32_t n_prns, double interm_freq_hz, uint32_t flags, acq_result* results, float* power_bins) {
    return guarded([&] {
        if (!P || !samples) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        sample_bytes(dtype);
        if (empty_request(P, n_samples, n_prns, flags)) return;
        if (!prns || !results) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if ((flags & ACQ_FLAG_STORE_POWER_BINS) && !power_bins)
            throw AcqError(ACQ_ERR_ARGUMENT, "store_power_bins requested without an output buffer");
        const size_t eb = sample_bytes(dtype);
        const Geometry& g = P->g;
        // only the first N_nc segments are read (src/acquire.jl:65-72)
        const int64_t need = static_cast<int64_t>(g.n_nc) * g.n_coh * g.spc;
        const int64_t ncopy = std::min<int64_t>(n_samples, need);
        CK(cudaSetDevice(P->device));
        // The tensor-core all-steps path reads a small (<= 256 KB) page-locked, device-mapped
        // caller buffer in place: its operand-block kernel reads the samples across the host link
        // itself, which saves the copy's fixed cost (1 ms at 4 MHz: e2e +2-4 %). Larger inputs are
        // uploaded first (10 ms x 8 at 5 MHz, 1.6 MB: the in-place reads made the call 16 % slower:
        // each sample is read several times), as are inputs of other paths: mapped buffers by the
        // k_copy_in gather, pageable ones by the copy engines. (ACQ_NO_ZERO_COPY=1: always the
        // copy engines.)
        const void* mapped = mapped_host(samples);
        const bool tensor_path = P->tmma && P->col_tma && !P->dft_mma && !(P->fused && P->form == ACQ_FORM_FUSED);
        const void* d_in = tensor_path && eb * ncopy <= (256u << 10) ? mapped : nullptr;
        if (!d_in) {
            P->input.ensure(eb * std::max<int64_t>(ncopy, 1));
            upload_inputs({{samples, mapped, P->input.p, eb * static_cast<size_t>(ncopy)}}, P->device, P->stream);
            d_in = P->input.p;
        }
        enqueue_acquire(P, d_in, dtype, n_samples, prns, n_prns, interm_freq_hz, flags);
        fetch(P, results, power_bins);
    });
}

int acq_acquire_device_async(acq_plan* P, const void* d_samples, int32_t dtype, int64_t n_samples,
                             const int32_t* prns, int32_t n_prns, double interm_freq_hz, uint32_t flags) {
    return guarded([&] {
        if (!P || !d_samples) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        sample_bytes(dtype);
        if (empty_request(P, n_samples, n_prns, flags)) return;
        if (!prns) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        enqueue_acquire(P, d_samples, dtype, n_samples, prns, n_prns, interm_freq_hz, flags);
    });
}

int acq_fetch_results(acq_plan* P, acq_result* results, float* power_bins) {
    return guarded([&] {
        if (!P) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        fetch(P, results, power_bins);
    });
}

int acq_plan_stream(const acq_plan* P, void** stream) {
    return guarded([&] {
        if (!P || !stream) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *stream = static_cast<void*>(P->stream);
    });
}

int acq_plan_last_launch_count(const acq_plan* P, int64_t* count) {
    return guarded([&] {
        if (!P || !count) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *count = P->launches;
    });
}

int acq_plan_last_kernels(const acq_plan* P, char* buf, size_t len) {
    return guarded([&] {
        if (!P) throw AcqError(ACQ_ERR_ARGUMENT, "null plan");
        std::string out;
        for (size_t i = 0; i < P->klog.size(); ++i) out += (i ? ";" : "") + P->klog[i];
        if (buf && len) {
            const size_t m = std::min(len - 1, out.size());
            std::memcpy(buf, out.data(), m);
            buf[m] = 0;
        }
    });
}

int acq_batch_create(const acq_batch_item* items, int32_t n_items, acq_batch** out) {
    return guarded([&] {
        if (!items || !out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        acq_batch* B = new acq_batch();
        try {
            batch_build(B, items, n_items);
        } catch (...) {
            batch_free(B);
            throw;
        }
        *out = B;
    });
}

int acq_batch_destroy(acq_batch* B) {
    batch_free(B);
    return ACQ_OK;
}

int acq_batch_input_ptr(acq_batch* B, int32_t item, void** d_ptr) {
    return guarded([&] {
        if (!B || !d_ptr || item < 0 || item >= static_cast<int>(B->items.size()))
            throw AcqError(ACQ_ERR_ARGUMENT, "bad batch item");
        *d_ptr = B->arena.as<unsigned char>() + B->items[item].in_off;
    });
}

int acq_batch_upload(acq_batch* B, const void* const* host) {
    return guarded([&] {
        if (!B || !host) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        CK(cudaSetDevice(B->device));
        std::vector<Upload> ups(B->items.size());
        for (size_t i = 0; i < B->items.size(); ++i) {
            if (!host[i]) throw AcqError(ACQ_ERR_ARGUMENT, "null recording for batch item " + std::to_string(i));
            ups[i] = {host[i], mapped_host(host[i]), B->arena.as<unsigned char>() + B->items[i].in_off,
                      B->items[i].in_bytes};
        }
        upload_inputs(ups, B->device, B->s0);
    });
}

int acq_batch_launch(acq_batch* B) {
    return guarded([&] {
        if (!B) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        CK(cudaSetDevice(B->device));
        CK(cudaGraphLaunch(B->exec, B->s0));
    });
}

int acq_batch_fetch(acq_batch* B, acq_result* results) {
    return guarded([&] {
        if (!B || !results) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        CK(cudaSetDevice(B->device));
        CK(cudaMemcpyAsync(results, B->res.p, sizeof(acq_result) * B->total_res, cudaMemcpyDeviceToHost, B->s0));
        CK(cudaStreamSynchronize(B->s0));
        for (const auto& m : B->items)
            if (m.plan->errflag.p) {
                int e = 0;
                CK(cudaMemcpy(&e, m.plan->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
                if (e) {
                    CK(cudaMemset(m.plan->errflag.p, 0, sizeof(int)));
                    throw AcqError(ACQ_ERR_TIMEOUT, "a bounded wait for a TMA tile gave up");
                }
            }
    });
}

int acq_batch_run(acq_batch* B, const void* const* host, acq_result* results) {
    int st = acq_batch_upload(B, host);
    if (st != ACQ_OK) return st;
    st = acq_batch_launch(B);
    if (st != ACQ_OK) return st;
    return acq_batch_fetch(B, results);
}

int acq_batch_stream(const acq_batch* B, void** stream) {
    return guarded([&] {
        if (!B || !stream) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *stream = static_cast<void*>(B->s0);
    });
}

int acq_batch_launch_count(const acq_batch* B, int64_t* count) {
    return guarded([&] {
        if (!B || !count) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *count = B->launches;
    });
}

int acq_plan_set_kernel_timing(acq_plan* P, int32_t enable) {
    return guarded([&] {
        if (!P) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        P->timing = enable != 0;
    });
}

int acq_plan_kernel_times(acq_plan* P, double* total_ms, int64_t* launches, int32_t n_kinds) {
    return guarded([&] {
        if (!P || !total_ms || !launches) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        for (int i = 0; i < n_kinds && i < ACQ_KERNEL_KINDS; ++i) {
            total_ms[i] = P->kt_ms[i];
            launches[i] = P->kt_n[i];
        }
    });
}

int acq_plan_reset_kernel_times(acq_plan* P) {
    return guarded([&] {
        if (!P) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        for (int i = 0; i < ACQ_KERNEL_KINDS; ++i) {
            P->kt_ms[i] = 0;
            P->kt_n[i] = 0;
        }
    });
}

int acq_plan_get_option(const acq_plan* P, int32_t option, int64_t* value) {
    return guarded([&] {
        if (!P || !value) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        switch (option) {
            case ACQ_OPT_FORM: *value = (P->fused && P->form == ACQ_FORM_FUSED) ? ACQ_FORM_FUSED : ACQ_FORM_PLAIN; break;
            case ACQ_OPT_ROTATION_PRECISION: *value = P->rot_prec; break;
            case ACQ_OPT_DOPPLER_PRECISION: *value = P->dft_prec; break;
            case ACQ_OPT_MMA_SCALE_LOG2: *value = P->mma_scale_log2; break;
            case ACQ_OPT_TILE_THREADS: *value = P->tile_fs ? P->tileThreads : 0; break;
            case ACQ_OPT_TILE_BLOCKS: *value = P->tile_fs ? P->tileNF : 0; break;
            case ACQ_OPT_TILE_PAD: *value = P->tile_fs ? P->tileFS - P->tileBase : 0; break;
            case ACQ_OPT_TILE_ROWS: *value = P->tile_fs ? P->tileRows : 0; break;
            case ACQ_OPT_TRANSFORM_LENGTH: *value = P->g.fft_tile; break;
            case ACQ_OPT_TILE_MMA: *value = P->tmma ? 1 : 0; break;
            case ACQ_OPT_COLUMN_WAIT_POLLS: *value = P->col_k1 ? P->k1WaitPolls : 0; break;
            case ACQ_OPT_SEARCH_WIDTH: *value = P->sign_sb ? P->Wssb : P->rot_sb ? P->Wrsb : 0; break;
            case ACQ_OPT_SEARCH_SPLIT: *value = P->sign_sb ? P->n1ssb : 0; break;
            case ACQ_OPT_COLUMN_WIDTH: *value = P->col_k1 ? P->k1W : P->col_tma ? P->tmaW : 0; break;
            case ACQ_OPT_COLUMN_CTAS_PER_SM: *value = P->col_k1 ? P->k1CtasPerSm : P->col_tma ? P->tmaCtasPerSm : 0; break;
            default: throw AcqError(ACQ_ERR_ARGUMENT, "unknown option " + std::to_string(option));
        }
    });
}

int acq_plan_set_option(acq_plan* P, int32_t option, int64_t value, int64_t* effective) {
    return guarded([&] {
        if (!P) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (option == ACQ_OPT_TRANSFORM_LENGTH) throw AcqError(ACQ_ERR_ARGUMENT, "the transform length is read-only");
        ++P->version;   // a replayed launch sequence must be captured again
        if (option == ACQ_OPT_ROTATION_PRECISION) {
            if (value < ACQ_PREC_FP32 || value > ACQ_PREC_BF16_SPLIT)
                throw AcqError(ACQ_ERR_ARGUMENT, "unknown precision " + std::to_string(value));
            const Geometry& g = P->g;
            RotMmaFn fn = nullptr;
            size_t smem = 0;
            const int n_cand = g.R * (1 << (g.ndb - 1));
            if (value != ACQ_PREC_FP32 && g.path == 2 && g.n_be == 1 && n_cand <= 32 && !getenv_flag("ACQ_GENERIC_FFT"))
                fn = pick_rot_mma(g.n_coh, g.nb, n_cand, 1 << (g.ndb - 1), static_cast<int>(value), &smem);
            if (fn) {
                set_smem((const void*)fn, smem);
                P->errflag.ensure(sizeof(int));
                CK(cudaMemset(P->errflag.p, 0, sizeof(int)));
            }
            P->rot_mma = fn;
            P->smem_mma = smem;
            P->rot_prec = fn ? static_cast<int>(value) : ACQ_PREC_FP32;
            if (effective) *effective = P->rot_prec;
            return;
        }
        if (option == ACQ_OPT_TILE_THREADS || option == ACQ_OPT_TILE_BLOCKS || option == ACQ_OPT_TILE_PAD ||
            option == ACQ_OPT_TILE_ROWS) {
            const Geometry& g = P->g;
            if (!P->tile_fs) {
                if (effective) *effective = 0;
                return;
            }
            CK(cudaStreamSynchronize(P->stream));
            const int old_threads = P->tileThreads, old_nf = P->tileNF, old_fs = P->tileFS, old_rows = P->tileRows;
            TileFsFn old_fn = P->tile_fs;
            if (option == ACQ_OPT_TILE_THREADS) {
                if (value < 32 || value > 256 || value % 32) throw AcqError(ACQ_ERR_ARGUMENT, "tile threads must be 32..256, a multiple of 32");
                P->tileThreads = static_cast<int>(value);
            } else if (option == ACQ_OPT_TILE_BLOCKS) {
                if (value < 1 || value > g.nb) throw AcqError(ACQ_ERR_ARGUMENT, "tile blocks per CTA must be in 1:num_blocks");
                P->tileNF = static_cast<int>(value);
            } else if (option == ACQ_OPT_TILE_ROWS) {
                if (value != 1 && value != 2) throw AcqError(ACQ_ERR_ARGUMENT, "tile rows per CTA must be 1 or 2");
                TileFsFn fn = pick_tile_fs(g.fft_tile, static_cast<int>(value));
                if (!fn) throw AcqError(ACQ_ERR_ARGUMENT, "no tile kernel for this FFT size");
                P->tile_fs = fn;
                P->tileRows = static_cast<int>(value);
            } else {
                if (value < 0 || value > 32) throw AcqError(ACQ_ERR_ARGUMENT, "tile padding must be in 0:32");
                P->tileFS = P->tileBase + static_cast<int>(value);
            }
            const size_t smem = tile_smem(P);
            if (smem > 200 * 1024) {   // keep the previous shape
                P->tileThreads = old_threads;
                P->tileNF = old_nf;
                P->tileFS = old_fs;
                P->tileRows = old_rows;
                P->tile_fs = old_fn;
                throw AcqError(ACQ_ERR_ARGUMENT, "tile configuration exceeds shared memory");
            }
            P->smem_tile_fs = smem;
            set_smem((const void*)P->tile_fs, P->smem_tile_fs);
            if (effective)
                *effective = option == ACQ_OPT_TILE_THREADS ? P->tileThreads
                           : option == ACQ_OPT_TILE_BLOCKS  ? P->tileNF
                           : option == ACQ_OPT_TILE_ROWS    ? P->tileRows
                                                            : P->tileFS - P->tileBase;
            return;
        }
        if (option == ACQ_OPT_COLUMN_WIDTH || option == ACQ_OPT_COLUMN_CTAS_PER_SM) {
            if (!P->col_tma) {
                if (effective) *effective = 0;
                return;
            }
            CK(cudaStreamSynchronize(P->stream));
            if (P->col_k1) {   // the Doppler-group form: tiles of nb rows x W columns
                int W = P->k1W, cps = P->k1CtasPerSm;
                if (option == ACQ_OPT_COLUMN_WIDTH) {
                    if (value < 8 || value > 256 || value % 2)
                        throw AcqError(ACQ_ERR_ARGUMENT, "column width must be even, in 8:256");
                    W = static_cast<int>(value);
                } else {
                    if (value < 1 || value > 32) throw AcqError(ACQ_ERR_ARGUMENT, "CTAs per SM must be in 1:32");
                    cps = static_cast<int>(value);
                }
                const int oldW = P->k1W, oldc = P->k1CtasPerSm;
                setup_col_k1(P, P->n_plan_prns, W, cps);
                if (!P->col_k1) setup_col_k1(P, P->n_plan_prns, oldW, oldc);   // keep the previous shape
                if (effective) *effective = option == ACQ_OPT_COLUMN_WIDTH ? P->k1W : P->k1CtasPerSm;
                return;
            }
            int W = P->tmaW, cps = P->tmaCtasPerSm;
            if (option == ACQ_OPT_COLUMN_WIDTH) {
                if (value < 8 || value > 32 || value % 2)
                    throw AcqError(ACQ_ERR_ARGUMENT, "column width must be even, in 8:32");
                W = static_cast<int>(value);
            } else {
                if (value < 1 || value > 32) throw AcqError(ACQ_ERR_ARGUMENT, "CTAs per SM must be in 1:32");
                cps = static_cast<int>(value);
            }
            const int oldW = P->tmaW, oldc = P->tmaCtasPerSm;
            setup_col_tma(P, P->n_plan_prns, W, cps);
            if (!P->col_tma) setup_col_tma(P, P->n_plan_prns, oldW, oldc);   // keep the previous shape
            if (effective) *effective = option == ACQ_OPT_COLUMN_WIDTH ? P->tmaW : P->tmaCtasPerSm;
            return;
        }
        if (option == ACQ_OPT_DOPPLER_PRECISION) {
            if (value < ACQ_PREC_FP32 || value > ACQ_PREC_BF16_SPLIT)
                throw AcqError(ACQ_ERR_ARGUMENT, "unknown precision " + std::to_string(value));
            const Geometry& g = P->g;
            CK(cudaStreamSynchronize(P->stream));
            P->dft_mma = nullptr;
            P->dft_prec = ACQ_PREC_FP32;
            if (value != ACQ_PREC_FP32 && g.path == 0 && g.ndop <= 250 && !getenv_flag("ACQ_GENERIC_FFT")) {
                const int fmt = (value == ACQ_PREC_BF16 || value == ACQ_PREC_BF16_SPLIT) ? 1 : 0;
                const int nsplit = (value == ACQ_PREC_FP16_SPLIT || value == ACQ_PREC_BF16_SPLIT) ? 2 : 1;
                const int npad = (2 * g.ndop + 15) / 16 * 16;
                const int ksteps = npad / 16;
                P->dftB.ensure((size_t)nsplit * ksteps * npad * 32);
                const int64_t total = (int64_t)ksteps * npad * 16;
                const unsigned grid = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 4096));
                if (fmt == 0)
                    k_dft_operand<0><<<grid, 256, 0, P->stream>>>(g.ndop, npad, ksteps, nsplit, P->dftB.as<uint8_t>());
                else
                    k_dft_operand<1><<<grid, 256, 0, P->stream>>>(g.ndop, npad, ksteps, nsplit, P->dftB.as<uint8_t>());
                CK(cudaGetLastError());
                CK(cudaStreamSynchronize(P->stream));
                DftMmaFn fn = fmt == 0 ? (nsplit == 2 ? named(&k_col_dft_mma<0, 2>, "k_col_dft_mma<fp16,2>")
                                                      : named(&k_col_dft_mma<0, 1>, "k_col_dft_mma<fp16,1>"))
                                       : (nsplit == 2 ? named(&k_col_dft_mma<1, 2>, "k_col_dft_mma<bf16,2>")
                                                      : named(&k_col_dft_mma<1, 1>, "k_col_dft_mma<bf16,1>"));
                // one block per SM (the block holds 512 TMEM columns)
                const size_t need = 1024 + 2 * (size_t)nsplit * 4096 + 2 * (size_t)nsplit * npad * 32 + 64;
                const size_t smem = std::max<size_t>(need, 120 * 1024);
                set_smem((const void*)fn, smem);
                P->errflag.ensure(sizeof(int));
                CK(cudaMemset(P->errflag.p, 0, sizeof(int)));
                P->dft_mma = fn;
                P->smem_dft = smem;
                P->dftNpad = npad;
                P->dftKsteps = ksteps;
                P->dft_prec = static_cast<int>(value);
            }
            if (effective) *effective = P->dft_prec;
            return;
        }
        if (option == ACQ_OPT_TILE_MMA) {
            if (value != 0 && value != 1) throw AcqError(ACQ_ERR_ARGUMENT, "tile MMA must be 0 or 1");
            CK(cudaStreamSynchronize(P->stream));
            P->tmma_enabled = value != 0;
            setup_col_tma(P, P->n_plan_prns, P->tmaW, P->tmaCtasPerSm);
            setup_tile_mma(P);
            if (effective) *effective = P->tmma ? 1 : 0;
            return;
        }
        if (option == ACQ_OPT_SEARCH_WIDTH || option == ACQ_OPT_SEARCH_SPLIT) {
            if (value < 1 || value > 1024) throw AcqError(ACQ_ERR_ARGUMENT, "search shape must be in 1:1024");
            CK(cudaStreamSynchronize(P->stream));
            const int v = static_cast<int>(value);
            if (P->sign_sb) {
                // keep the other dimension where an instantiation has both, else take the value's default
                if (option == ACQ_OPT_SEARCH_WIDTH) {
                    if (!setup_sign_search(P, v, P->n1ssb)) setup_sign_search(P, v, 0);
                } else if (!setup_sign_search(P, P->Wssb, v)) {
                    setup_sign_search(P, 0, v);
                }
                if (effective) *effective = option == ACQ_OPT_SEARCH_WIDTH ? P->Wssb : P->n1ssb;
            } else if (P->rot_sb && option == ACQ_OPT_SEARCH_WIDTH) {
                setup_rot_search(P, v);
                if (effective) *effective = P->Wrsb;
            } else if (effective) {
                *effective = 0;
            }
            return;
        }
        if (option == ACQ_OPT_COLUMN_WAIT_POLLS) {
            if (value < 0 || value > static_cast<int64_t>(kWaitLimit))
                throw AcqError(ACQ_ERR_ARGUMENT, "poll limit must be in 0:" + std::to_string(kWaitLimit));
            CK(cudaStreamSynchronize(P->stream));
            P->k1WaitPolls = static_cast<uint32_t>(value);
            if (effective) *effective = P->col_k1 ? P->k1WaitPolls : 0;
            return;
        }
        if (option == ACQ_OPT_MMA_SCALE_LOG2) {
            if (value != 127 && (value < -64 || value > 64))
                throw AcqError(ACQ_ERR_ARGUMENT, "scale exponent must be in -64:64 (or 127 for the default)");
            P->mma_scale_log2 = static_cast<int>(value);
            if (effective) *effective = value;
            return;
        }
        if (option != ACQ_OPT_FORM) throw AcqError(ACQ_ERR_ARGUMENT, "unknown option " + std::to_string(option));
        if (value != ACQ_FORM_FUSED && value != ACQ_FORM_PLAIN)
            throw AcqError(ACQ_ERR_ARGUMENT, "unknown form " + std::to_string(value));
        P->form = static_cast<int>(value);
        if (effective) *effective = (P->fused && P->form == ACQ_FORM_FUSED) ? ACQ_FORM_FUSED : ACQ_FORM_PLAIN;
    });
}

int acq_cfar_threshold(double pfa, int64_t num_cells, int32_t M, double* out) {
    return guarded([&] {
        if (!out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        *out = cfar_threshold(pfa, num_cells, M);
    });
}

int acq_gen_code_device(int32_t system, const int32_t* prns, int32_t n_prns, int64_t n, double fs, double fc,
                        double start_phase, int8_t* d_out, void* stream) {
    return guarded([&] {
        if (!prns || !d_out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (n_prns < 1 || n < 0) throw AcqError(ACQ_ERR_ARGUMENT, "n_prns must be >= 1 and n >= 0");
        if (!(fs > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "sampling frequency must be positive");
        std::vector<int8_t> c0 = full_chips(system, prns[0]);
        const int64_t L = static_cast<int64_t>(c0.size());
        std::vector<int8_t> all((size_t)n_prns * L);
        for (int i = 0; i < n_prns; ++i) {
            std::vector<int8_t> c = full_chips(system, prns[i]);
            std::memcpy(&all[(size_t)i * L], c.data(), L);
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        int8_t* d_chips = nullptr;
        CK(cudaMallocAsync(reinterpret_cast<void**>(&d_chips), all.size(), st));
        CK(cudaMemcpyAsync(d_chips, all.data(), all.size(), cudaMemcpyHostToDevice, st));
        sample_codes_device(system, d_chips, L, n_prns, n, fs, fc, start_phase, d_out, st);
        CK(cudaFreeAsync(d_chips, st));
        CK(cudaStreamSynchronize(st));   // the host chip tables go out of scope
    });
}

int acq_selftest_bounded_wait(int32_t device, uint32_t polls, int32_t* status) {
    return guarded([&] {
        if (!status) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (polls < 1 || polls > (1u << 26)) throw AcqError(ACQ_ERR_ARGUMENT, "polls must be in 1:2^26");
        CK(cudaSetDevice(device));
        int* d_err = nullptr;
        CK(cudaMalloc(&d_err, sizeof(int)));
        CK(cudaMemset(d_err, 0, sizeof(int)));
        k_wait_selftest<<<1, 32>>>(polls, d_err);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        int h = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost);
        cudaFree(d_err);
        if (e != cudaSuccess) throw CudaError(std::string("self test: ") + cudaGetErrorString(e));
        *status = h == 9 ? ACQ_ERR_TIMEOUT : ACQ_OK;
    });
}

int acq_chip_order(int32_t num_blocks, int32_t block_size, int64_t width, double code_freq_hz, double sampling_freq_hz,
                   int32_t* perm, double* chip_axis) {
    return guarded([&] {
        if (!perm) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        chip_order(num_blocks, block_size, width, code_freq_hz, sampling_freq_hz, perm, chip_axis);
    });
}

int acq_sort_power_bins_by_chip(const acq_plan* P, const float* d_power_bins, int32_t n_surfaces, float* d_out,
                                void* stream) {
    return guarded([&] {
        if (!P || !d_power_bins || !d_out) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (n_surfaces < 1) throw AcqError(ACQ_ERR_ARGUMENT, "n_surfaces must be >= 1");
        if (d_power_bins == d_out) throw AcqError(ACQ_ERR_ARGUMENT, "the sort cannot run in place");
        const Geometry& g = P->g;
        CK(cudaSetDevice(P->device));
        const int64_t rows = (int64_t)n_surfaces * g.ndop;
        k_gather_cols<<<std::min<int64_t>((rows * g.spc_eff + 255) / 256, 8192), 256, 0,
                        static_cast<cudaStream_t>(stream)>>>(d_power_bins, rows, g.spc_eff,
                                                             P->chipperm.as<int32_t>(), d_out);
        CK(cudaGetLastError());
    });
}

int acq_gen_code(int32_t system, int32_t prn, int64_t n, double fs, double fc, double start_phase, int8_t* out) {
    return guarded([&] {
        if (!out && n > 0) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (n < 0) throw AcqError(ACQ_ERR_ARGUMENT, "n must be >= 0");
        if (!(fs > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "sampling frequency must be positive");
        gen_code(system, prn, n, fs, fc, start_phase, out);
    });
}

int acq_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return ACQ_ERR_ARGUMENT;
    std::snprintf(buf, len, "%s", g_last_error.c_str());
    return ACQ_OK;
}

#ifdef ACQ_BOUNDS_CHECK
const char* acq_version(void) { return "acqgb300 0.1.0 sm_103a bounds-checked"; }
#else
const char* acq_version(void) { return "acqgb300 0.1.0 sm_103a"; }
#endif

}  // extern "C"
