// acq_inst_tile.cu — coherent-tile and fused cluster kernels for the hot fft sizes.
#include "acq_inst.h"

namespace acq {

#define ACQ_TILE_CASE(F)                                                                     \
    case F:                                                                                  \
        return rows == 2 ? named(&k_tile_fs<best_split_n1(F), F / best_split_n1(F), 2>, "k_tile_fs<" #F ",2>") \
                         : named(&k_tile_fs<best_split_n1(F), F / best_split_n1(F), 1>, "k_tile_fs<" #F ",1>");

TileFsFn pick_tile_fs(int F, int rows) {
    if (rows != 1 && rows != 2) return nullptr;
    switch (F) {
        ACQ_TILE_CASE(128) ACQ_TILE_CASE(256) ACQ_TILE_CASE(500) ACQ_TILE_CASE(512) ACQ_TILE_CASE(1000)
        ACQ_TILE_CASE(1024) ACQ_TILE_CASE(1250) ACQ_TILE_CASE(1280) ACQ_TILE_CASE(1600) ACQ_TILE_CASE(2500)
        ACQ_TILE_CASE(2560)
        default: return nullptr;
    }
}

#define ACQ_FUSED_CASE(F, D) \
    if (fft == F && ndop == D)   \
        return named(&k_fused_simple<best_split_n1(F), F / best_split_n1(F), best_split_n1(D), D / best_split_n1(D)>, \
                     "k_fused_simple<" #F "," #D ">");

FusedFn pick_fused(int fft, int ndop) {
    // transform lengths as chosen by the runtime (powers of two, or five times one, where possible)
    ACQ_FUSED_CASE(512, 200) ACQ_FUSED_CASE(512, 16) ACQ_FUSED_CASE(512, 20) ACQ_FUSED_CASE(256, 16)
    ACQ_FUSED_CASE(256, 32) ACQ_FUSED_CASE(128, 32) ACQ_FUSED_CASE(1280, 75) ACQ_FUSED_CASE(2560, 20)
    ACQ_FUSED_CASE(1280, 320) ACQ_FUSED_CASE(1280, 16) ACQ_FUSED_CASE(512, 40) ACQ_FUSED_CASE(512, 400)
    return nullptr;
}

}  // namespace acq

cudaError_t acq_inst_tile_upload_twiddles(const float2* host, size_t n) {
    return cudaMemcpyToSymbol(acq::c_regtw, host, sizeof(float2) * n);
}

ACQ_BC_SET_TABLE_IMPL(acq_inst_tile_set_bounds_table)
