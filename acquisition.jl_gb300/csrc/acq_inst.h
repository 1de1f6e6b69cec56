// acq_inst.h — the specialised-kernel dispatch tables. Each acq_inst_*.cu translation unit
// instantiates one family of size-specialised kernels (compiled in parallel) and exports a
// picker returning the kernel for a size (nullptr when that size has no specialisation) plus
// the upload of its own copy of the register-FFT twiddle table.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "acq_kernels_fs.cuh"

namespace acq {

// Names of the size-specialised kernels, for the launch log of acq_plan_last_kernels: each
// picker records the name of the instantiation it returns.
void note_kernel_name(const void* fn, const char* name);
const char* kernel_name(const void* fn);
template <class F>
inline F named(F fn, const char* name) {
    note_kernel_name(reinterpret_cast<const void*>(fn), name);
    return fn;
}

using TileFsFn = void (*)(const float2*, const float2*, const int*, int, int, int, int, const float2*, int, float2*,
                          int64_t, int);
using FusedFn = void (*)(FusedParams);
using ColFsFn = void (*)(const float2*, int, int, const float2*, const int*, int, int, float*, int);
using ColTmaFn = void (*)(const CUtensorMap, ColTmaParams);
using SignFsFn = void (*)(const float2*, int, int, const float2*, const float*, int, int, int, int, int, const int*,
                          const int*, int, float*, uint16_t*, int);
using RotFsFn = void (*)(const float2*, int, int, const float2*, const float*, int, int, int, int, int, int, int, int,
                         const int*, const int*, int, float*, uint16_t*, int);

using RotSbFn = void (*)(const float2*, int, const float2*, const float*, int, int, int, int, int, int, const int*,
                         const int*, int, float*, uint16_t*, int);
// rotation stage split by (coherent periods, blocks per period); nullptr when not instantiated.
// *w = columns per block, *threads = block size.
// want_w: columns per CTA wanted (0: the default for the size); *w, *threads: the kernel's shape
RotSbFn pick_rot_sb(int n_coh, int nb, int want_w, int* w, int* threads);

using SignSbFn = void (*)(const float2*, int, const float2*, const float*, int, int, int, const int*, const int*, int,
                          float*, uint16_t*, int);
// data-bit / bit-edge search split by sub-blocks for (ndop, data bits); nullptr when not
// instantiated. *w = columns per block, *threads = block size, *smem = dynamic bytes.
// want_w / want_n1: columns per CTA and first-pass length of the FFT split wanted (0: the default
// for the size, the first instantiation listed); *w, *n1, *threads, *smem: the kernel's shape
SignSbFn pick_sign_sb(int ndop, int ndb, int want_w, int want_n1, int* w, int* n1, int* threads, size_t* smem);

struct RotMmaParams;
struct DftMmaParams;
using DftMmaFn = void (*)(DftMmaParams);
using RotMmaFn = void (*)(RotMmaParams);
// tensor-core rotation combine for (coherent periods, blocks per period, candidates) at an
// ACQ_PREC_* precision other than FP32; nullptr when not instantiated; *smem = dynamic bytes.
RotMmaFn pick_rot_mma(int n_coh, int nb, int n_candidates, int combos, int prec, size_t* smem);


// coherent tile for an FFT size, transforming `rows` (1 or 2) rows per CTA
TileFsFn pick_tile_fs(int fft_size, int rows);
FusedFn pick_fused(int fft_size, int ndop);
ColFsFn pick_col_fs(int ndop);
ColTmaFn pick_col_tma(int ndop);
// TMA column stage that runs only the nb-point pass (the first pass applied by k_doppler_prepass)
ColTmaFn pick_col_tma_pre(int nb);
// the same stage with work items per Doppler group k1 (tile = nb rows x W columns, 128 threads)
ColTmaFn pick_col_tma_k1(int nb);
SignFsFn pick_sign_fs(int ndop);
RotFsFn pick_rot_fs(int ndop);

}  // namespace acq

// the checked build's bounds table, per translation unit (no-ops in the normal build)
cudaError_t acq_bounds_set_table_runtime(void* table);
cudaError_t acq_inst_tile_set_bounds_table(void* table);
cudaError_t acq_inst_col_set_bounds_table(void* table);
cudaError_t acq_inst_sign_set_bounds_table(void* table);
cudaError_t acq_inst_mma_set_bounds_table(void* table);
cudaError_t acq_inst_tile_upload_twiddles(const float2* host, size_t n);
cudaError_t acq_inst_col_upload_twiddles(const float2* host, size_t n);
cudaError_t acq_inst_sign_upload_twiddles(const float2* host, size_t n);
cudaError_t acq_inst_mma_upload_twiddles(const float2* host, size_t n);
