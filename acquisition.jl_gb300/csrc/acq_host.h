// acq_host.h — host-side (CPU) part of libacqgb300: plan geometry, validation, code
// generation, sign patterns and the CFAR threshold. Shared by the C ABI and the CUDA
// runtime. Nothing here touches the GPU.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "acqgb300.h"

namespace acq {

// Thrown for argument errors; carries the reference's ArgumentError text and a status.
struct AcqError : std::runtime_error {
    int status;
    AcqError(int st, const std::string& msg) : std::runtime_error(msg), status(st) {}
};

struct SystemInfo {
    int id;
    const char* name;
    int code_length;          // primary chips
    double code_freq;         // Hz
    double center_freq;       // Hz
    double data_freq;         // Hz
    int secondary_length;     // 1 when there is none
    const int8_t* secondary;  // +-1, secondary_length entries (nullptr when none)
    bool boc11;
    int max_prn;
};

const SystemInfo& system_info(int id);

// Plan geometry, src/plan.jl:325-525.
struct Geometry {
    int spc, spc_eff, nb, bs, fft_size, n_coh, ndb, n_be, n_nc, ndop, R, bit_period_codes;
    // length of the block and coherent-tile transforms actually run: any length >= 2 bs gives the
    // same lags 0..bs-1 of the linear correlation as fft_size (the reference's field, reported
    // unchanged); the runtime may pick a faster one (see choose_fft_tile)
    int fft_tile;
    int path;                 // 0 simple, 1 sign search, 2 rotation search
    double doppler_first, doppler_step, coverage;
    std::vector<double> doppler_freqs;
    int noise_estimator;
    int use_secondary_code;
    double cfar_thr;          // cfar_threshold(0.01, ndop*spc*R; n_nc)
};

Geometry compute_geometry(const acq_plan_desc& d);   // throws AcqError(ACQ_ERR_ARGUMENT)

// +-1 chips of the full (primary x secondary) code of a PRN.
std::vector<int8_t> full_chips(int system, int prn);

// true when x is an integer representable exactly (gen_code's exact integer phase path)
bool is_whole_freq(double x);

// GNSSSignals gen_code semantics (sample i -> chip floor(start + i*fc/fs) mod full length).
void gen_code(int system, int prn, int64_t n, double fs, double fc, double start_phase, int8_t* out);

// Sign patterns (src/sign_patterns.jl:23-47): (n_coh x num_patterns) column-major floats.
std::vector<float> sign_patterns(int system, int prn, int ndb, int R, int n_coh, bool use_secondary);

// Code drift shifts per sorted row (src/noncoherent_integration.jl:600-619), in [0, spc).
// Returns true when any shift rounds to non-zero.
bool code_drift_shifts(const Geometry& g, const SystemInfo& s, double fs, int step, int32_t* out);

double cfar_threshold(double pfa, int64_t num_cells, int M);   // src/cfar.jl:64-85

// Column order of a power surface sorted by code phase (src/plot.jl:16-20,35-57): perm[i] is the
// FM-DBZP column shown at position i, axis[i] its code phase in chips (monotone).
void chip_order(int num_blocks, int block_size, int64_t width, double code_freq, double fs, int32_t* perm,
                double* axis);

int nextprod_2357(int n);

// Record the calling thread's last error message (read back by acq_last_error).
void set_last_error(const std::string& msg);

// FFT factorisation used by the device Stockham FFT (radices 4,2,3,5,7, then odd primes).
std::vector<int> fft_radices(int n);

}  // namespace acq
