/*
 * acqgb300.h — C ABI of the GB300-native FM-DBZP acquisition library (libacqgb300.so).
 *
 * Drop-in boundary for the FM-DBZP acquisition path of JuliaGNSS/Acquisition.jl v2.6.4:
 * a Julia `ccall` shim (or Python ctypes) maps the reference's public API onto these
 * entry points. Plain pointers and sizes only; no CUDA or torch types cross this boundary
 * (streams are passed as opaque `void*`).
 *
 * Conventions
 *  - Every entry point returns an `int` status: ACQ_OK (0) or one of ACQ_ERR_*.
 *    `acq_last_error` returns the message of the calling thread's last failure; for
 *    ACQ_ERR_ARGUMENT it carries the reference's ArgumentError text.
 *  - A plan owns all of its device memory and one CUDA stream. One acquisition per plan
 *    at a time (the reference's contract, src/plan.jl:186-190); distinct plans may run
 *    concurrently from different host threads.
 *  - Indices in results are 0-based. Frequencies are in Hz, code phases in chips.
 */
#ifndef ACQGB300_H
#define ACQGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define ACQ_OK 0
#define ACQ_ERR_ARGUMENT 1          /* ArgumentError in the reference */
#define ACQ_ERR_SHORT_SIGNAL 2      /* src/acquire.jl:68-72 */
#define ACQ_ERR_PRN_NOT_IN_PLAN 3   /* src/acquire.jl:62-63 */
#define ACQ_ERR_CUDA 4              /* CUDA runtime failure (message has the CUDA error) */
#define ACQ_ERR_TIMEOUT 5           /* a bounded device wait gave up */
#define ACQ_ERR_ALLOC 6             /* device or pinned allocation failed */
#define ACQ_ERR_UNSUPPORTED 7

/* ---- enums ---- */
#define ACQ_GPS_L1CA 0
#define ACQ_GPS_L5I 1
#define ACQ_GALILEO_E1B 2            /* synthetic memory codes, BOC(1,1) */

#define ACQ_CF32 0                   /* interleaved float32 re/im */
#define ACQ_CI16 1                   /* interleaved int16 re/im */
#define ACQ_CI8 2                    /* interleaved int8 re/im */
#define ACQ_CF64 3                   /* interleaved float64 re/im (converted to float32 like ComplexF32(x)) */

#define ACQ_NOISE_OPPOSITE_ROW 0     /* OppositeRowNoiseEstimator, src/est_signal_noise_power.jl:70 */
#define ACQ_NOISE_GLOBAL_MEAN 1      /* GlobalMeanNoiseEstimator, src/est_signal_noise_power.jl:100 */

#define ACQ_FLAG_SUBSAMPLE_INTERP 1u /* acquire!(...; subsample_interpolation = true) */
#define ACQ_FLAG_STORE_POWER_BINS 2u /* acquire!(...; store_power_bins = true) */
#define ACQ_FLAG_POWER_BINS_CHIP_SORTED 4u /* with STORE_POWER_BINS: columns in code-phase order
                                              (src/plot.jl:35-57) instead of FM-DBZP order */

typedef struct acq_plan acq_plan;

/* Keyword arguments of plan_acquire (src/plan.jl:312-324). */
typedef struct {
    int32_t system;                                  /* ACQ_GPS_L1CA, ... */
    double sampling_freq_hz;
    double min_doppler_coverage_hz;                  /* default 7000 */
    int32_t num_coherently_integrated_code_periods;  /* default 1 */
    int32_t bit_edge_search_steps;                   /* default 1 */
    int32_t num_noncoherent_accumulations;           /* default 1 */
    int32_t noise_estimator;                         /* default ACQ_NOISE_OPPOSITE_ROW */
    int32_t use_secondary_code;                      /* default 1 */
    int32_t max_secondary_code_rotations;            /* default 32 */
    int32_t device;                                  /* CUDA device ordinal, default 0 */
} acq_plan_desc;

/* Derived plan geometry (the fields of AcquisitionPlan, src/plan.jl:81-174). */
typedef struct {
    int32_t samples_per_code;
    int32_t samples_per_code_eff;
    int32_t num_blocks;
    int32_t block_size;
    int32_t fft_size;
    int32_t num_coherently_integrated_code_periods;
    int32_t num_data_bits;
    int32_t bit_edge_search_steps;
    int32_t num_noncoherent_accumulations;
    int32_t num_doppler_bins;
    int32_t num_secondary_rotations;
    int32_t bit_period_codes;
    int32_t num_prns;
    int32_t path;                 /* 0 simple, 1 data-bit / bit-edge search, 2 secondary-code rotation */
    double doppler_first_hz;      /* doppler_freqs[0] */
    double doppler_step_hz;       /* step(doppler_freqs) */
    double code_length;           /* chips of the primary code */
    double code_freq_hz;
    double center_freq_hz;
    double cfar_threshold_pfa001; /* cfar_threshold(0.01, cells incl. rotations; N_nc) */
} acq_geometry;

/* One AcquisitionResults (src/Acquisition.jl:81-109) plus the decision indices. */
typedef struct {
    int32_t prn;
    int32_t secondary_code_phase;         /* -1 == `nothing` */
    double carrier_doppler_hz;
    double code_phase;                    /* chips */
    double cn0_dbhz;
    float noise_power;
    float peak_to_noise_ratio;
    float peak_power;
    int32_t num_noncoherent_integrations;
    int32_t peak_doppler_bin;             /* 0-based sorted Doppler row */
    int32_t peak_code_bin;                /* 0-based effective code-phase column */
    int32_t sign_pattern;                 /* data-bit combination at the peak, -1 on the simple path */
    int32_t bit_edge;                     /* bit-edge alignment at the peak, -1 on the simple path */
    int32_t detected;                     /* peak_to_noise_ratio > cfar_threshold(0.01, ...) */
    int32_t reserved;
} acq_result;

/* Fill `desc` with the reference's keyword defaults (src/plan.jl:312-324). */
void acq_plan_desc_init(acq_plan_desc* desc);

/* Validate `desc` and derive the geometry without touching the GPU.
 * Replaces the validation + geometry part of plan_acquire, src/plan.jl:325-525. */
int acq_plan_query(const acq_plan_desc* desc, acq_geometry* out);

/* plan_acquire(system, sampling_freq, prns; kwargs...) — src/plan.jl:312-697.
 * `codes` may be NULL (the library samples its own codes, GNSSSignals gen_code semantics)
 * or point to n_prns * samples_per_code int8 +-1 samples (e.g. from GNSSSignals.gen_code). */
int acq_plan_create(const acq_plan_desc* desc, const int32_t* prns, int32_t n_prns,
                    const int8_t* codes, acq_plan** out);

int acq_plan_destroy(acq_plan* plan);

int acq_plan_get_geometry(const acq_plan* plan, acq_geometry* out);

/* doppler_freqs of the plan (num_doppler_bins doubles, sorted ascending). */
int acq_plan_doppler_freqs(const acq_plan* plan, double* out);

/* acquire!(plan, signal, prns; interm_freq, subsample_interpolation, store_power_bins)
 * — src/acquire.jl:54-89. `samples` is a HOST buffer of n_samples complex samples of `dtype`.
 * `results` receives n_prns entries in the order of `prns`. When flags has
 * ACQ_FLAG_STORE_POWER_BINS, `power_bins` (host, may otherwise be NULL) receives
 * n_prns * num_doppler_bins * samples_per_code_eff float32, per PRN row-major
 * [doppler_row][code_col] (the transpose of Julia's column-major Matrix). Synchronous.
 * n_prns = 0 (prns and results may be NULL) only checks the signal length, like acquire! with
 * an empty PRN vector. */
int acq_acquire(acq_plan* plan, const void* samples, int32_t dtype, int64_t n_samples,
                const int32_t* prns, int32_t n_prns, double interm_freq_hz, uint32_t flags,
                acq_result* results, float* power_bins);

/* Same as acq_acquire, with `samples` already in device memory. Enqueues on the plan's
 * stream and returns without waiting; read the results with acq_fetch_results. */
int acq_acquire_device_async(acq_plan* plan, const void* d_samples, int32_t dtype, int64_t n_samples,
                             const int32_t* prns, int32_t n_prns, double interm_freq_hz, uint32_t flags);

/* Wait for the plan's stream and copy the last acquisition's results (and, when stored,
 * power bins) to host memory. */
int acq_fetch_results(acq_plan* plan, acq_result* results, float* power_bins);

/* The plan's cudaStream_t, as an opaque pointer (for event timing by the caller). */
int acq_plan_stream(const acq_plan* plan, void** stream);

/* Number of this library's kernel launches enqueued by the last acquisition. */
int acq_plan_last_launch_count(const acq_plan* plan, int64_t* count);

/* Names of this library's kernels launched by the last acquisition on the plan, in launch
 * order, separated by ';'; size-specialised kernels carry their template sizes, e.g.
 * "k_tile_stubs;k_tile_mma;k_col_sign_sb<32,25,8,2>;k_extract". Written NUL-terminated to buf (truncated
 * to len). A replayed CUDA graph reports the sequence it was captured from. Diagnostic, for
 * tests that pin which instantiation a geometry runs; no reference counterpart. */
int acq_plan_last_kernels(const acq_plan* plan, char* buf, size_t len);

/* Plan options (acq_plan_set_option). */
#define ACQ_OPT_FORM 0               /* ACQ_FORM_PLAIN (default) or ACQ_FORM_FUSED */
#define ACQ_FORM_FUSED 0             /* cluster kernel: tile + Doppler stage + accumulation in shared memory */
#define ACQ_FORM_PLAIN 1             /* one kernel per stage, coherent tile and accumulator in HBM */
#define ACQ_OPT_ROTATION_PRECISION 1 /* arithmetic of the secondary-code rotation combine: */
#define ACQ_PREC_FP32 0              /*   FP32 FFTs on the CUDA cores (default) */
#define ACQ_PREC_FP16 1              /*   tensor cores, FP16 sub-block spectra, FP32 accumulation */
#define ACQ_PREC_BF16 2              /*   tensor cores, BF16 sub-block spectra */
#define ACQ_PREC_FP16_SPLIT 3        /*   tensor cores, spectra split hi + lo in FP16 (two MMAs) */
#define ACQ_PREC_BF16_SPLIT 4        /*   tensor cores, spectra split hi + lo in BF16 (two MMAs) */
#define ACQ_OPT_MMA_SCALE_LOG2 2     /* power-of-two scale of the spectra before FP16 rounding (default: by
                                        input type, CF32/CF64 0, CI16 -10, CI8 -2) */
/* Launch shapes (the autotuner's knobs; `effective` = the value in effect, 0 where the plan's
 * sizes have no such kernel): */
#define ACQ_OPT_TILE_THREADS 3       /* coherent-tile kernel: threads per CTA (32..256, multiple of 32) */
#define ACQ_OPT_TILE_BLOCKS 4        /*   code blocks (inverse FFTs) per CTA round (1..num_blocks) */
#define ACQ_OPT_TILE_PAD 5           /*   shared-memory padding between FFT buffers, complex elements (0..32) */
#define ACQ_OPT_COLUMN_WIDTH 6       /* TMA column kernel: code-phase columns per tile (even; 8..32, or 8..256
                                        for the Doppler-group form of the simple path) */
#define ACQ_OPT_COLUMN_CTAS_PER_SM 7 /*   persistent CTAs per SM (1..occupancy limit) */
#define ACQ_OPT_DOPPLER_PRECISION 8  /* simple path: the per-column Doppler DFT as a dense DFT-matrix GEMM on the
                                        tensor cores (ACQ_PREC_*; ndop <= 250), or FP32 FFTs (default) */
#define ACQ_OPT_TILE_ROWS 9          /* coherent-tile kernel: rows sharing g mod num_blocks per CTA (1 or 2) */
#define ACQ_OPT_TRANSFORM_LENGTH 10  /* read-only: length of the block and tile transforms (>= 2 block_size;
                                        fft_size, or a power of two or five times one up to 5 % longer) */
#define ACQ_OPT_TILE_MMA 11          /* block_size <= 256: the coherent tile as a time-domain correlation GEMM
                                        on the tensor cores (FP16 codes x FP16 hi + lo samples, FP32
                                        accumulation) = 1 (default where available), FP32 FFTs = 0 */
#define ACQ_OPT_COLUMN_WAIT_POLLS 12 /* test-only: polls of each tile wait in the Doppler-group column stage before
                                        the block gives up (default 2^24; 0 gives up at once and runs the
                                        give-up path: one block-wide decision, a full-limit wait for the copies
                                        in flight, ACQ_ERR_TIMEOUT from acq_fetch_results); 0 where the plan
                                        has no such stage */
#define ACQ_OPT_SEARCH_WIDTH 13      /* bit-edge / rotation search kernel: code-phase columns per CTA (the sizes
                                        instantiated for the plan's geometry; 0 where it has no such kernel) */
#define ACQ_OPT_SEARCH_SPLIT 14      /*   bit-edge search: first-pass length N1 of the num_doppler_bins = N1 x N2
                                        FFT split (instantiated splits; 0 where none) */

/* Set a plan option; ACQ_OPT_FORM selects the kernel form of later acquisitions. The fused
 * form is used only where the plan's sizes have a fused kernel (otherwise plain).
 * ACQ_OPT_ROTATION_PRECISION selects the rotation combine's arithmetic on plans with a
 * secondary-code rotation search; a tensor-core variant is used where the plan's geometry has
 * one (one bit-edge step, at most 32 candidates), otherwise FP32. ACQ_OPT_MMA_SCALE_LOG2 sets
 * the spectra scale (values -64..64; 127 restores the per-input-type default). The launch-shape
 * options wait for the plan's stream and apply to later acquisitions (batches keep the shapes
 * they were captured with). Returns the value now in effect through `effective` (may be NULL).
 * No reference counterpart. */
int acq_plan_set_option(acq_plan* plan, int32_t option, int64_t value, int64_t* effective);
/* Read the value of a plan option now in effect (0 for a launch shape the plan's sizes lack). */
int acq_plan_get_option(const acq_plan* plan, int32_t option, int64_t* value);

/* Kernel classes for per-launch device timing. */
#define ACQ_KERNEL_FRONTEND 0        /* downconversion + double-block FFT */
#define ACQ_KERNEL_TILE 1            /* code-spectrum multiply + inverse FFT (coherent tile) */
#define ACQ_KERNEL_COLUMN 2          /* Doppler column stage (simple / sign / rotation search) */
#define ACQ_KERNEL_STATS 3           /* peak + FP64 noise partial sums */
#define ACQ_KERNEL_EXTRACT 4         /* result extraction, CFAR gate, interpolation */
#define ACQ_KERNEL_SECONDARY 5       /* secondary-code despread */
#define ACQ_KERNEL_FUSED 6           /* fused tile + Doppler + accumulation (cluster kernel) */
#define ACQ_KERNEL_KINDS 8

/* Enable (1) or disable (0) CUDA-event timing of every launch of this plan (on the plan's
 * stream). Diagnostic only; no reference counterpart. */
int acq_plan_set_kernel_timing(acq_plan* plan, int32_t enable);

/* Accumulated device milliseconds and launch counts per kernel class since the last reset
 * (arrays of n_kinds <= ACQ_KERNEL_KINDS entries). Call after acq_fetch_results. */
int acq_plan_kernel_times(acq_plan* plan, double* total_ms, int64_t* launches, int32_t n_kinds);

int acq_plan_reset_kernel_times(acq_plan* plan);

/* ---- ragged batches: many recordings, several plans, one CUDA-graph launch ----
 * Generalises acquire! (src/acquire.jl:54-89) to a list of recordings of uneven length and mixed
 * systems (one plan per geometry; items may share a plan). The batch packs all inputs into one
 * device arena, captures every acquisition into a single CUDA graph (one branch per plan; items
 * that share a plan run in order within their branch) and replays it per batch. The plans must
 * outlive the batch and be on one device; store_power_bins is not available in a batch. */
typedef struct acq_batch acq_batch;

typedef struct {
    acq_plan* plan;
    int32_t dtype;               /* ACQ_CF32 / ACQ_CI16 / ACQ_CI8 / ACQ_CF64 */
    int64_t n_samples;           /* length of this recording */
    const int32_t* prns;         /* requested PRNs (subset of the plan's) */
    int32_t n_prns;
    double interm_freq_hz;
    uint32_t flags;              /* ACQ_FLAG_SUBSAMPLE_INTERP only */
} acq_batch_item;

int acq_batch_create(const acq_batch_item* items, int32_t n_items, acq_batch** out);
int acq_batch_destroy(acq_batch* batch);

/* Device address of item i's input slot in the batch arena (for callers that fill it themselves). */
int acq_batch_input_ptr(acq_batch* batch, int32_t item, void** d_ptr);

/* Copy the items' host recordings into the arena (`host_samples[i]` for item i), asynchronously. */
int acq_batch_upload(acq_batch* batch, const void* const* host_samples);

/* One graph launch over every item (inputs already in the arena); returns without waiting. */
int acq_batch_launch(acq_batch* batch);

/* Wait and copy all results (sum of n_prns entries, items in order). */
int acq_batch_fetch(acq_batch* batch, acq_result* results);

/* upload + launch + fetch. */
int acq_batch_run(acq_batch* batch, const void* const* host_samples, acq_result* results);

/* The batch's cudaStream_t (opaque) and its kernel launches per graph launch. */
int acq_batch_stream(const acq_batch* batch, void** stream);
int acq_batch_launch_count(const acq_batch* batch, int64_t* count);

/* cfar_threshold(pfa, num_cells; num_noncoherent_integrations) — src/cfar.jl:64-85. Host only. */
int acq_cfar_threshold(double pfa, int64_t num_cells, int32_t num_noncoherent_integrations, double* out);

/* gen_code(n, system, prn, sampling_freq, code_freq, start_phase) into `out` (+-1 int8).
 * code_freq_hz <= 0 selects the system's nominal code rate. Host only. */
/* gen_code on the device for n_prns PRNs: d_out (device, n_prns x n int8) receives, per PRN,
 * exactly what acq_gen_code returns for (system, prn, n, fs, fc, start_phase). Waits for
 * `stream` before returning. */
int acq_gen_code_device(int32_t system, const int32_t* prns, int32_t n_prns, int64_t n, double sampling_freq_hz,
                        double code_freq_hz, double start_phase, int8_t* d_out, void* stream);

/* ---- synthetic recordings on the device (src/generate_test_signal.jl:32-82) ---- */
typedef struct {
    int32_t prn;
    int32_t data_bits;        /* 1: +-1 data bits at the system's data rate (counter-based random values) */
    double cn0_dbhz;          /* amplitude sqrt(10^(CN0/10) / fs) for unit noise power */
    double doppler_hz;        /* carrier Doppler; the code runs at f_code + f_d f_code / f_carrier */
    double code_phase;        /* chips at sample 0 */
    double carrier_phase;     /* rad */
    double bit_offset_s;      /* time into the first data bit at sample 0 */
} acq_synth_sat;              /* 48 bytes */

/* Write n samples of `dtype` (ACQ_CF32 / CI16 / CI8 / CF64) to device memory d_out: the sum of the
 * satellites' signals (code with gen_code semantics, carrier, data bits) plus, when noise != 0,
 * complex white Gaussian noise of unit power from a counter-based generator seeded by `seed`.
 * CI16 = round(x 2^10) saturated; CI8 = 3-bit quantiser (odd levels, step 0.5 sigma). Waits for
 * `stream` before returning. */
int acq_synth_signal(int32_t system, double sampling_freq_hz, int64_t n, const acq_synth_sat* sats, int32_t n_sats,
                     double interm_freq_hz, uint64_t seed, int32_t noise, int32_t dtype, void* d_out, void* stream);

/* Failure-detection self test: one block waits (bounded, `polls` polls) on an mbarrier that
 * nothing arrives on, the way every device wait of the library is bounded. *status =
 * ACQ_ERR_TIMEOUT when the wait gave up and reported it (the expected outcome), ACQ_OK otherwise;
 * the context stays usable. */
int acq_selftest_bounded_wait(int32_t device, uint32_t polls, int32_t* status);

/* Column order of a power surface sorted by code phase, src/plot.jl:16-20,35-57 (host, no GPU):
 * perm[i] = the FM-DBZP column at chip-sorted position i (width entries), chip_axis[i] (may be
 * NULL) its code phase in chips, monotone. width = the surface's columns (samples_per_code_eff). */
int acq_chip_order(int32_t num_blocks, int32_t block_size, int64_t width, double code_freq_hz, double sampling_freq_hz,
                   int32_t* perm, double* chip_axis);

/* Chip-sorted copy of n_surfaces device surfaces (num_doppler_bins x samples_per_code_eff each,
 * the layout acquisitions store) into d_out (device; not in place), enqueued on `stream`. */
int acq_sort_power_bins_by_chip(const acq_plan* plan, const float* d_power_bins, int32_t n_surfaces, float* d_out,
                                void* stream);

int acq_gen_code(int32_t system, int32_t prn, int64_t n, double sampling_freq_hz, double code_freq_hz,
                 double start_phase, int8_t* out);

/* Output of acq_est_signal_noise_power_noalloc (device memory owned by the caller). */
typedef struct {
    float signal_power;        /* peak_power - noise_power */
    float noise_power;
    float peak_power;
    int32_t peak_doppler_bin;  /* 0-based row */
    int32_t peak_code_bin;     /* 0-based column */
    int32_t reserved;
} acq_noise_stats;

/* Peak and noise power of a power surface, for callers that cannot allocate device memory
 * once running (a receiver's real-time processing thread, where cudaMalloc/cudaFree may
 * synchronise the device and take unbounded time, or a plugin whose host framework owns all
 * device memory). This entry point has no counterpart in the reference; it computes what
 * acq_acquire reports for a surface (peak with the lowest-column, lowest-row tie-break,
 * OppositeRow or GlobalMean noise in FP64) and allocates nothing: `d_power_bins`
 * (num_doppler_bins rows x num_code_bins columns, row-major float32) and `d_out` are caller
 * device memory; the scratch is a fixed static device array (32 KiB, held by every GPU that
 * loads the library until exit), so num_doppler_bins is limited to 4096 and larger sizes
 * return ACQ_ERR_ARGUMENT. Asynchronous on `stream` (a cudaStream_t, NULL for the default
 * stream). Calls share the scratch and clear it themselves; calls that overlap on the GPU race
 * and must be ordered by the caller. Every call looks up the scratch address on the current
 * device (cudaGetSymbolAddress, nothing cached, so a device reset between calls is safe); the
 * first call on a device may load the library's device code there: make it before any stream
 * capture. */
int acq_est_signal_noise_power_noalloc(const float* d_power_bins, int32_t num_doppler_bins, int64_t num_code_bins,
                                       double sampling_freq_hz, double code_freq_hz, int32_t noise_estimator,
                                       acq_noise_stats* d_out, void* stream);

/* ---- continuous correlator: fine search, gradients, Newton refinement ----
 *
 * Extends the grid search with a continuous correlator over (code phase, Doppler):
 *   phi_n   = code_phase + n * (f_code + doppler * f_code / f_carrier) / fs      [chips]
 *   theta_n = 2 pi (interm_freq + doppler) n / fs
 *   z       = sum_n x[n] c(phi_n) exp(-i theta_n),       power P = |z|^2
 * over the model of src/generate_test_signal.jl:45-68 (the correlation the acquisition grid
 * samples at integer code bins and Doppler bins). c is the PRN's chip sequence (BOC(1,1) half
 * chips for Galileo E1B, the secondary code folded in for GPS L5I) smoothed by the quadratic
 * B-spline centred on each chip, so that P is differentiable twice in code phase and Doppler.
 * Sums run in FP32 on the device; the derived power, gradient and Hessian are formed in FP64.
 * Every pointer named d_* is device memory; `stream` is a cudaStream_t (NULL = default
 * stream). Calls enqueue work and return without waiting. */
typedef struct acq_corr acq_corr;

typedef struct {
    int32_t prn;
    int32_t reserved;       /* 0 */
    double code_phase;      /* chips at sample 0 */
    double doppler_hz;      /* carrier Doppler */
} acq_corr_cell;            /* 24 bytes */

#define ACQ_CORR_OK 0               /* evaluated / converged */
#define ACQ_CORR_NOT_CONVERGED 1    /* acq_corr_refine ran out of iterations */
#define ACQ_CORR_BAD_PRN 3          /* the cell's PRN is not in the context: outputs are zero */

typedef struct {
    double power;           /* P = |z|^2 */
    double grad[2];         /* dP/d code_phase (per chip), dP/d doppler (per Hz) */
    double hess[3];         /* d2P/dtau2, d2P/dtau ddoppler, d2P/ddoppler2 (zero unless requested) */
    double z_re, z_im;      /* correlator output z */
    int32_t iterations;     /* Newton iterations (acq_corr_refine), 0 for acq_corr_eval */
    int32_t status;         /* ACQ_CORR_* */
} acq_corr_result;          /* 72 bytes */

/* A context for `system` at `sampling_freq_hz` over `prns`: uploads the chip tables. `codes`
 * is NULL (built-in generators) or n_prns x primary-code-length chips of +-1 (as in
 * acq_plan_create). */
int acq_corr_create(int32_t system, double sampling_freq_hz, const int32_t* prns, int32_t n_prns,
                    const int8_t* codes, acq_corr** out);
int acq_corr_destroy(acq_corr* ctx);

/* Power, gradient (and the Hessian when want_hessian != 0) at every cell.
 * d_samples: n_samples samples of `dtype` (ACQ_CF32 / ACQ_CI16 / ACQ_CI8 / ACQ_CF64). */
int acq_corr_eval(acq_corr* ctx, const void* d_samples, int32_t dtype, int64_t n_samples, double interm_freq_hz,
                  const acq_corr_cell* d_cells, int32_t n_cells, int32_t want_hessian, acq_corr_result* d_out,
                  void* stream);

/* Adjoint with respect to the samples: d_xbar[n] = sum_cells d_zbar[c] * conj(dz_c / dx[n])
 * = sum_c zbar_c c(phi_{c,n}) exp(+i theta_{c,n}), written as interleaved float32 re/im
 * (2 * n_samples floats, overwritten). zbar_c = dL/dRe z_c + i dL/dIm z_c is the cotangent of
 * z_c (2 * P_bar_c * z_c for a loss on the power). The code replica is recomputed, not read. */
int acq_corr_vjp_samples(acq_corr* ctx, int64_t n_samples, double interm_freq_hz, const acq_corr_cell* d_cells,
                         const float* d_zbar, int32_t n_cells, float* d_xbar, void* stream);

/* Batched Newton refinement of the power maximum from every cell (updated in place): Newton
 * steps on the closed-form gradient and Hessian inside a box trust region of
 * (max_step_chips, max_step_hz), gradient ascent where the Hessian is not negative definite,
 * step halving when the power drops; stops when both step components fall below the
 * tolerances. d_out receives the evaluation at the final point. */
int acq_corr_refine(acq_corr* ctx, const void* d_samples, int32_t dtype, int64_t n_samples, double interm_freq_hz,
                    acq_corr_cell* d_cells, int32_t n_cells, int32_t max_iterations, double tol_chips,
                    double tol_hz, double max_step_chips, double max_step_hz, acq_corr_result* d_out, void* stream);


/* Copy the calling thread's last error message (NUL-terminated, truncated to len). */
int acq_last_error(char* buf, size_t len);

/* Library version string, e.g. "acqgb300 0.1.0 sm_103a". */
const char* acq_version(void);

#ifdef __cplusplus
}
#endif

#endif /* ACQGB300_H */
