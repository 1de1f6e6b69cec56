// acq_inst_col.cu — simple-path Doppler column kernels (per step and TMA-staged) for hot ndop.
#include "acq_inst.h"

namespace acq {

#define ACQ_COL_CASE(N) \
    case N: return named(&k_col_simple_fs<best_split_n1(N), N / best_split_n1(N)>, "k_col_simple_fs<" #N ">");
#define ACQ_COLTMA_CASE(N) \
    case N: return named(&k_col_tma<best_split_n1(N), N / best_split_n1(N), false>, "k_col_tma<" #N ">");
#define ACQ_COLTMA_PRE_CASE(N) \
    case N: return named(&k_col_tma<1, N, true>, "k_col_tma_pre<" #N ">");

ColFsFn pick_col_fs(int ndop) {
    switch (ndop) {
        ACQ_COL_CASE(16) ACQ_COL_CASE(20) ACQ_COL_CASE(32) ACQ_COL_CASE(40) ACQ_COL_CASE(64) ACQ_COL_CASE(75)
        ACQ_COL_CASE(100) ACQ_COL_CASE(160) ACQ_COL_CASE(200) ACQ_COL_CASE(240) ACQ_COL_CASE(320) ACQ_COL_CASE(400)
        ACQ_COL_CASE(500) ACQ_COL_CASE(640) ACQ_COL_CASE(800) ACQ_COL_CASE(1280)
        default: return nullptr;
    }
}

ColTmaFn pick_col_tma_k1(int nb) {
    switch (nb) {
        case 8: return named(&k_col_tma_k1<8>, "k_col_tma_k1<8>");
        case 10: return named(&k_col_tma_k1<10>, "k_col_tma_k1<10>");
        case 16: return named(&k_col_tma_k1<16>, "k_col_tma_k1<16>");
        case 20: return named(&k_col_tma_k1<20>, "k_col_tma_k1<20>");
        case 25: return named(&k_col_tma_k1<25>, "k_col_tma_k1<25>");
        case 32: return named(&k_col_tma_k1<32>, "k_col_tma_k1<32>");
        case 40: return named(&k_col_tma_k1<40>, "k_col_tma_k1<40>");
        case 50: return named(&k_col_tma_k1<50>, "k_col_tma_k1<50>");
        case 64: return named(&k_col_tma_k1<64>, "k_col_tma_k1<64>");
        default: return nullptr;
    }
}

ColTmaFn pick_col_tma_pre(int nb) {
    switch (nb) {
        ACQ_COLTMA_PRE_CASE(8) ACQ_COLTMA_PRE_CASE(10) ACQ_COLTMA_PRE_CASE(16) ACQ_COLTMA_PRE_CASE(20)
        ACQ_COLTMA_PRE_CASE(25) ACQ_COLTMA_PRE_CASE(32) ACQ_COLTMA_PRE_CASE(40) ACQ_COLTMA_PRE_CASE(50)
        ACQ_COLTMA_PRE_CASE(64)
        default: return nullptr;
    }
}

ColTmaFn pick_col_tma(int ndop) {
    switch (ndop) {
        ACQ_COLTMA_CASE(16) ACQ_COLTMA_CASE(20) ACQ_COLTMA_CASE(32) ACQ_COLTMA_CASE(40) ACQ_COLTMA_CASE(64)
        ACQ_COLTMA_CASE(75) ACQ_COLTMA_CASE(100) ACQ_COLTMA_CASE(160) ACQ_COLTMA_CASE(200) ACQ_COLTMA_CASE(240)
        ACQ_COLTMA_CASE(320) ACQ_COLTMA_CASE(400) ACQ_COLTMA_CASE(500)
        default: return nullptr;
    }
}

}  // namespace acq

cudaError_t acq_inst_col_upload_twiddles(const float2* host, size_t n) {
    return cudaMemcpyToSymbol(acq::c_regtw, host, sizeof(float2) * n);
}

ACQ_BC_SET_TABLE_IMPL(acq_inst_col_set_bounds_table)
