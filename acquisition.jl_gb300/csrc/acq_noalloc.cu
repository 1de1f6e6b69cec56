// acq_noalloc.cu — peak / noise-power statistics of a power surface without any allocation.
//
// For callers that must not allocate device memory once they are running: a receiver's
// real-time processing thread (cudaMalloc/cudaFree can synchronise the whole device and take
// unbounded time) or a plugin whose host framework owns every byte of device memory. They
// pass the surface and the output in memory they already own; the reduction's scratch lives
// in the fixed static device array below, which every GPU that loads the library holds
// until the process exits.
//
// Contract
//  - Scratch limit: num_doppler_bins <= kNoAllocMaxDopplerBins (4096); larger sizes are
//    rejected with ACQ_ERR_ARGUMENT before any device work.
//  - All calls on a device share the one scratch array. Each call clears the part it uses
//    before the reduction, so nothing carries over between calls, but calls that overlap on
//    the GPU (different streams, or host threads without ordering) race on it: order them.
//  - Every call looks up the array's device address for the current device with
//    cudaGetSymbolAddress (nothing is cached, so a device reset between calls leaves no stale
//    address behind). The first call on a device may load this library's device code there;
//    make that first call before any stream capture.
//  - Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
#include <cuda_runtime.h>

#include <string>

#include "acq_host.h"
#include "acqgb300.h"

namespace {

constexpr int kNoAllocMaxDopplerBins = 4096;
constexpr int kNoAllocHeaderWords = 4;   // [0] peak key, [1] total (double), [2] exclusion sum (double)
constexpr int kNoAllocWords = kNoAllocHeaderWords + kNoAllocMaxDopplerBins;
constexpr int kCols = 256;

// 32 KiB + 32 B of scratch: the peak key, two FP64 sums and one FP64 sum per Doppler row.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocWords];

__device__ __forceinline__ unsigned long long nk(float v, uint32_t order) {
    return (static_cast<unsigned long long>(__float_as_uint(v)) << 32) |
           static_cast<unsigned long long>(0xFFFFFFFFu - order);
}

// Pass 1: per-row FP64 sums, the total and the peak (lowest column, then lowest row under
// strict >, src/est_signal_noise_power.jl:109-135), accumulated into the scratch array.
__global__ void k_noalloc_pass1(const float* __restrict__ P, int ndop, int64_t ncols,
                                unsigned long long* __restrict__ scratch) {
    __shared__ double wtot[8];
    __shared__ unsigned long long wkey[8];
    double* rowsum = reinterpret_cast<double*>(scratch + kNoAllocHeaderWords);
    double* total = reinterpret_cast<double*>(scratch + 1);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int64_t c0 = static_cast<int64_t>(blockIdx.x) * kCols;
    unsigned long long best = 0ULL;
    double tot = 0.0;
    for (int e = wp; e < ndop; e += 8) {
        float rs = 0.f;
        const float* rowp = P + static_cast<int64_t>(e) * ncols;
#pragma unroll
        for (int i = 0; i < kCols / 32; ++i) {
            const int64_t c = c0 + lane + 32 * i;
            if (c < ncols) {
                const float v = rowp[c];
                rs += v;
                const unsigned long long key = nk(v, static_cast<uint32_t>(c * ndop + e));
                best = key > best ? key : best;
            }
        }
        double rsd = static_cast<double>(rs);
        for (int o = 16; o > 0; o >>= 1) rsd += __shfl_xor_sync(0xffffffffu, rsd, o);
        if (lane == 0) {
            atomicAdd(rowsum + e, rsd);
            tot += rsd;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other > best ? other : best;
    }
    if (lane == 0) {
        wtot[wp] = tot;
        wkey[wp] = best;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long b = 0ULL;
        for (int w = 0; w < 8; ++w) {
            t += wtot[w];
            b = wkey[w] > b ? wkey[w] : b;
        }
        atomicAdd(total, t);
        atomicMax(scratch, b);
    }
}

// Pass 2: noise power (OppositeRow, src/est_signal_noise_power.jl:211-227, or GlobalMean with
// the +-samples_per_chip column exclusion, :150-170,229-243) and the output record.
__global__ void k_noalloc_finish(const float* __restrict__ P, int ndop, int64_t ncols, int estimator,
                                 int samples_per_chip, unsigned long long* __restrict__ scratch,
                                 acq_noise_stats* __restrict__ out) {
    __shared__ double red[256];
    const unsigned long long key = scratch[0];
    const float peak = __uint_as_float(static_cast<uint32_t>(key >> 32));
    const uint32_t order = 0xFFFFFFFFu - static_cast<uint32_t>(key & 0xFFFFFFFFull);
    const int64_t col = order / ndop;
    const int row = static_cast<int>(order - static_cast<uint32_t>(col) * ndop);
    const int64_t lo = col - samples_per_chip < 0 ? 0 : col - samples_per_chip;
    const int64_t hi = col + samples_per_chip > ncols - 1 ? ncols - 1 : col + samples_per_chip;
    double part = 0.0;
    if (estimator == ACQ_NOISE_GLOBAL_MEAN) {
        const int64_t w = hi - lo + 1;
        for (int64_t i = threadIdx.x; i < w * ndop; i += blockDim.x) {
            const int e = static_cast<int>(i / w);
            part += static_cast<double>(P[static_cast<int64_t>(e) * ncols + lo + (i - e * w)]);
        }
    }
    red[threadIdx.x] = part;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double* rowsum = reinterpret_cast<const double*>(scratch + kNoAllocHeaderWords);
    const double total = *reinterpret_cast<const double*>(scratch + 1);
    double noise_d;
    if (estimator == ACQ_NOISE_GLOBAL_MEAN)
        noise_d = (total - red[0]) / (static_cast<double>(ncols - (hi - lo + 1)) * ndop);
    else
        noise_d = rowsum[(row + ndop / 2) % ndop] / static_cast<double>(ncols);
    acq_noise_stats r;
    r.noise_power = __double2float_rn(noise_d);
    r.signal_power = __fsub_rn(peak, r.noise_power);
    r.peak_power = peak;
    r.peak_doppler_bin = row;
    r.peak_code_bin = static_cast<int32_t>(col);
    r.reserved = 0;
    *out = r;
}

int fail(int status, const std::string& m) {
    acq::set_last_error(m);
    return status;
}

}  // namespace

extern "C" int acq_est_signal_noise_power_noalloc(const float* d_power_bins, int32_t num_doppler_bins,
                                                  int64_t num_code_bins, double sampling_freq_hz,
                                                  double code_freq_hz, int32_t noise_estimator,
                                                  acq_noise_stats* d_out, void* stream) {
    if (!d_power_bins || !d_out) return fail(ACQ_ERR_ARGUMENT, "null argument");
    if (num_doppler_bins < 1 || num_doppler_bins > kNoAllocMaxDopplerBins)
        return fail(ACQ_ERR_ARGUMENT, "num_doppler_bins=" + std::to_string(num_doppler_bins) +
                                          " is outside 1:" + std::to_string(kNoAllocMaxDopplerBins) +
                                          " (the fixed scratch of the no-allocation entry point)");
    if (num_code_bins < 2 || num_code_bins > 0x7FFFFFFF ||
        static_cast<unsigned long long>(num_code_bins) * num_doppler_bins > 0xFFFFFFFFull)
        return fail(ACQ_ERR_ARGUMENT, "num_code_bins=" + std::to_string(num_code_bins) +
                                          " must be in 2:2^31-1 with num_doppler_bins*num_code_bins < 2^32");
    if (noise_estimator != ACQ_NOISE_OPPOSITE_ROW && noise_estimator != ACQ_NOISE_GLOBAL_MEAN)
        return fail(ACQ_ERR_ARGUMENT, "unknown noise estimator " + std::to_string(noise_estimator));
    if (!(sampling_freq_hz > 0) || !(code_freq_hz > 0))
        return fail(ACQ_ERR_ARGUMENT, "sampling and code frequencies must be positive");
    // the scratch array's address on the current device, looked up on every call
    void* sp = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&sp, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(ACQ_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    unsigned long long* scratch = static_cast<unsigned long long*>(sp);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t clear = sizeof(unsigned long long) * (kNoAllocHeaderWords + num_doppler_bins);
    e = cudaMemsetAsync(scratch, 0, clear, st);
    if (e != cudaSuccess) return fail(ACQ_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const unsigned grid = static_cast<unsigned>((num_code_bins + kCols - 1) / kCols);
    k_noalloc_pass1<<<grid, 256, 0, st>>>(d_power_bins, num_doppler_bins, num_code_bins, scratch);
    const int spchip = static_cast<int>(sampling_freq_hz / code_freq_hz);
    k_noalloc_finish<<<1, 256, 0, st>>>(d_power_bins, num_doppler_bins, num_code_bins, noise_estimator, spchip,
                                        scratch, d_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ACQ_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return ACQ_OK;
}
