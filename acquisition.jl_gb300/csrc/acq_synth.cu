// acq_synth.cu — synthetic GNSS recordings generated on the device (signal model of
// src/generate_test_signal.jl:32-82), written straight into device buffers such as a batch's
// input arena, so test vectors and benchmark inputs need no host round trip.
//
// Per satellite: the code at the Doppler-shifted rate f_code + f_d f_code / f_carrier with
// GNSSSignals gen_code semantics (chip floor(code_phase + i fc / fs) of the full sequence,
// BOC(1,1) half-chip sign; the FP64 phase with explicit round-to-nearest multiply and add as in
// the host generator), times exp(i (2 pi (IF + f_d) i / fs + phi)), times +-1 data bits at the
// system's data rate, at amplitude sqrt(10^(CN0/10) / fs) for unit noise power. Noise: complex
// white Gaussian of unit total power from a counter-based generator (splitmix64 of
// seed, sample and component; Box-Muller). Output: complex64, or quantised like the host
// helpers (CI16: round(x * 2^10) saturated; CI8: 3-bit, odd levels +-1..+-7 at 0.5 sigma).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "acq_host.h"
#include "acqgb300.h"

namespace {

using acq::AcqError;

#define CKS(x)                                                                                          \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess)                                                                          \
            throw AcqError(ACQ_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorName(e_) + " " +          \
                                             cudaGetErrorString(e_));                                   \
    } while (0)

struct SatDev {
    int64_t table;          // offset of the chip table
    double amp, sp, ratio;  // amplitude, start phase (chips, reduced), code chips per sample
    double cyc;             // carrier cycles per sample (IF + f_d) / fs
    double phi;             // carrier phase offset (rad)
    double bit_rate;        // data bits per sample (0: no bits)
    double bit_off;         // bit offset in bits at sample 0
    uint64_t bit_seed;
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double unit_open(uint64_t h) {   // (0, 1]
    return (static_cast<double>(h >> 11) + 1.0) * 1.1102230246251565e-16;
}

__global__ void k_synth(const int8_t* __restrict__ chips, int64_t L, int boc, const SatDev* __restrict__ sats,
                        int n_sats, int64_t n, uint64_t seed, int noise, int dtype, void* __restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double re = 0.0, im = 0.0;
        const double t = static_cast<double>(i);
        for (int s = 0; s < n_sats; ++s) {
            const SatDev sd = sats[s];
            const double ph = __dadd_rn(sd.sp, __dmul_rn(t, sd.ratio));
            const double fl = floor(ph);
            const int64_t idx = static_cast<int64_t>(fl);
            double c = chips[sd.table + ((idx % L) + L) % L];
            if (boc && __dsub_rn(ph, fl) >= 0.5) c = -c;
            const double cy = sd.cyc * t;
            const double a = 6.283185307179586 * (cy - floor(cy)) + sd.phi;
            double sn, cs;
            sincos(a, &sn, &cs);
            double v = sd.amp * c;
            if (sd.bit_rate > 0.0) {
                const int64_t b = static_cast<int64_t>(floor(t * sd.bit_rate + sd.bit_off));
                v = (mix64(sd.bit_seed ^ static_cast<uint64_t>(b)) & 1ull) ? -v : v;
            }
            re += v * cs;
            im += v * sn;
        }
        if (noise) {
            const uint64_t h1 = mix64(seed ^ (static_cast<uint64_t>(i) * 2ull));
            const uint64_t h2 = mix64(seed ^ (static_cast<uint64_t>(i) * 2ull + 1ull) ^ 0x5851F42D4C957F2Dull);
            const double r = sqrt(-2.0 * log(unit_open(h1))) * 0.7071067811865476;
            double sn, cs;
            sincospi(2.0 * unit_open(h2), &sn, &cs);
            re += r * cs;
            im += r * sn;
        }
        if (dtype == ACQ_CF32) {
            reinterpret_cast<float2*>(out)[i] = make_float2(static_cast<float>(re), static_cast<float>(im));
        } else if (dtype == ACQ_CF64) {
            reinterpret_cast<double2*>(out)[i] = make_double2(re, im);
        } else if (dtype == ACQ_CI16) {
            const double qr = fmin(fmax(rint(re * 1024.0), -32768.0), 32767.0);
            const double qi = fmin(fmax(rint(im * 1024.0), -32768.0), 32767.0);
            reinterpret_cast<short2*>(out)[i] = make_short2(static_cast<short>(qr), static_cast<short>(qi));
        } else {
            const double step = 0.5 * 0.7071067811865476;
            const double qr = fmin(fmax(2.0 * floor(re / step) + 1.0, -7.0), 7.0);
            const double qi = fmin(fmax(2.0 * floor(im / step) + 1.0, -7.0), 7.0);
            reinterpret_cast<char2*>(out)[i] = make_char2(static_cast<signed char>(qr), static_cast<signed char>(qi));
        }
    }
}

template <typename F>
int guarded_synth(F&& f) {
    try {
        f();
        return ACQ_OK;
    } catch (const AcqError& e) {
        acq::set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        acq::set_last_error(e.what());
        return ACQ_ERR_CUDA;
    }
}

}  // namespace

extern "C" int acq_synth_signal(int32_t system, double fs, int64_t n, const acq_synth_sat* sats, int32_t n_sats,
                                double interm_freq_hz, uint64_t seed, int32_t noise, int32_t dtype, void* d_out,
                                void* stream) {
    return guarded_synth([&] {
        if (!d_out || (!sats && n_sats > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "null argument");
        if (n < 0 || n_sats < 0) throw AcqError(ACQ_ERR_ARGUMENT, "n and n_sats must be >= 0");
        if (!(fs > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "sampling frequency must be positive");
        if (dtype < ACQ_CF32 || dtype > ACQ_CF64) throw AcqError(ACQ_ERR_ARGUMENT, "unknown sample dtype");
        const acq::SystemInfo& s = acq::system_info(system);
        std::vector<SatDev> sd(static_cast<size_t>(n_sats));
        std::vector<int8_t> chips;
        int64_t L = 0;
        for (int k = 0; k < n_sats; ++k) {
            const acq_synth_sat& q = sats[k];
            std::vector<int8_t> c = acq::full_chips(system, q.prn);
            L = static_cast<int64_t>(c.size());
            sd[k].table = static_cast<int64_t>(chips.size());
            chips.insert(chips.end(), c.begin(), c.end());
            const double fc = s.code_freq + q.doppler_hz * s.code_freq / s.center_freq;
            double sp = std::fmod(q.code_phase, static_cast<double>(L));
            if (sp < 0) sp += L;
            sd[k].sp = sp;
            sd[k].ratio = fc / fs;
            sd[k].amp = std::sqrt(std::pow(10.0, q.cn0_dbhz / 10.0) / fs);
            sd[k].cyc = (interm_freq_hz + q.doppler_hz) / fs;
            sd[k].phi = q.carrier_phase;
            const bool bits = q.data_bits && std::isfinite(s.data_freq) && s.data_freq > 0;
            sd[k].bit_rate = bits ? s.data_freq / fs : 0.0;
            sd[k].bit_off = bits ? q.bit_offset_s * s.data_freq : 0.0;
            sd[k].bit_seed = seed * 0x9E3779B97F4A7C15ull + static_cast<uint64_t>(k + 1) * 0xD1B54A32D192ED03ull;
        }
        if (n == 0) return;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        int8_t* d_chips = nullptr;
        SatDev* d_sats = nullptr;
        const size_t cb = std::max<size_t>(chips.size(), 1);
        CKS(cudaMallocAsync(reinterpret_cast<void**>(&d_chips), cb, st));
        CKS(cudaMallocAsync(reinterpret_cast<void**>(&d_sats), sizeof(SatDev) * std::max<size_t>(sd.size(), 1), st));
        if (!chips.empty()) CKS(cudaMemcpyAsync(d_chips, chips.data(), chips.size(), cudaMemcpyHostToDevice, st));
        if (!sd.empty()) CKS(cudaMemcpyAsync(d_sats, sd.data(), sizeof(SatDev) * sd.size(), cudaMemcpyHostToDevice, st));
        const unsigned grid = static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 8192));
        k_synth<<<grid, 256, 0, st>>>(d_chips, std::max<int64_t>(L, 1), s.boc11 ? 1 : 0, d_sats, n_sats, n, seed,
                                      noise, dtype, d_out);
        CKS(cudaGetLastError());
        CKS(cudaFreeAsync(d_chips, st));
        CKS(cudaFreeAsync(d_sats, st));
        CKS(cudaStreamSynchronize(st));   // the host tables above go out of scope
    });
}
