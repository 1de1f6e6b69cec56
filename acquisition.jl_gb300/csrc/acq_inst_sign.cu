// acq_inst_sign.cu — data-bit / bit-edge and secondary-code rotation stages for hot ndop.
#include <cstdlib>

#include "acq_inst.h"

namespace acq {

#define ACQ_SIGN_CASE(N) \
    case N: return named(&k_col_sign_fs<best_split_n1(N), N / best_split_n1(N)>, "k_col_sign_fs<" #N ">");
#define ACQ_ROT_CASE(N) \
    case N: return named(&k_col_rot_fs<best_split_n1(N), N / best_split_n1(N)>, "k_col_rot_fs<" #N ">");

SignFsFn pick_sign_fs(int ndop) {
    switch (ndop) {
        ACQ_SIGN_CASE(40) ACQ_SIGN_CASE(200) ACQ_SIGN_CASE(400) ACQ_SIGN_CASE(500) ACQ_SIGN_CASE(640)
        ACQ_SIGN_CASE(800) ACQ_SIGN_CASE(1280)
        default: return nullptr;
    }
}

RotFsFn pick_rot_fs(int ndop) {
    switch (ndop) {
        ACQ_ROT_CASE(40) ACQ_ROT_CASE(100) ACQ_ROT_CASE(120) ACQ_ROT_CASE(160) ACQ_ROT_CASE(200)
        ACQ_ROT_CASE(240) ACQ_ROT_CASE(250) ACQ_ROT_CASE(400) ACQ_ROT_CASE(500) ACQ_ROT_CASE(1000)
        default: return nullptr;
    }
}

// W = 16 for tiles up to 384 rows, 8 above (the default); ACQ_RSB_W_CASE adds another width
#define ACQ_RSB_W_CASE(NC, NB, W)                                           \
    if (n_coh == NC && nb == NB && want_w == W) {                           \
        *w = W;                                                             \
        *threads = rot_sb_block(NC, NB, W);                                 \
        return named(&k_col_rot_sb<NC, NB, W>, "k_col_rot_sb<" #NC "," #NB "," #W ">"); \
    }
#define ACQ_RSB_CASE(NC, NB)                                                \
    if (n_coh == NC && nb == NB && (want_w == 0 || want_w == ((NC * NB <= 384) ? 16 : 8))) { \
        constexpr int kW = (NC * NB <= 384) ? 16 : 8;                       \
        *w = kW;                                                            \
        *threads = rot_sb_block(NC, NB, kW);                                \
        return named(&k_col_rot_sb<NC, NB, kW>,                             \
                     kW == 16 ? "k_col_rot_sb<" #NC "," #NB ",16>"          \
                              : "k_col_rot_sb<" #NC "," #NB ",8>");         \
    }

RotSbFn pick_rot_sb(int n_coh, int nb, int want_w, int* w, int* threads) {
    ACQ_RSB_CASE(20, 25) ACQ_RSB_CASE(10, 20) ACQ_RSB_CASE(20, 12) ACQ_RSB_CASE(10, 16) ACQ_RSB_CASE(10, 4)
    ACQ_RSB_CASE(20, 20) ACQ_RSB_CASE(10, 25) ACQ_RSB_CASE(20, 16) ACQ_RSB_CASE(10, 12) ACQ_RSB_CASE(20, 10)
    ACQ_RSB_W_CASE(20, 25, 4)
    return nullptr;
}

#define ACQ_SSB_CASE(N1, N2, W, NDB)                                                                 \
    if (ndop == N1 * N2 && ndb == NDB && (want_w == 0 || want_w == W) && (want_n1 == 0 || want_n1 == N1)) { \
        *w = W;                                                                                      \
        *n1 = N1;                                                                                    \
        *threads = (1 << (NDB - 1)) * N1 * W;                                                         \
        *smem = sizeof(float2) * ((size_t)(1 + NDB) * N1 * N2 * W + N1 * N2) + 64;                    \
        return named(&k_col_sign_sb<N1, N2, W, NDB>,                                                  \
                     "k_col_sign_sb<" #N1 "," #N2 "," #W "," #NDB ">");                              \
    }

// two data bits: the half-spectrum form (same block shape and shared memory as k_col_sign_sb)
#define ACQ_SFOLD_CASE(N1, N2, W)                                                                    \
    if (ndop == N1 * N2 && ndb == 2 && (want_w == 0 || want_w == W) && (want_n1 == 0 || want_n1 == N1)) { \
        *w = W;                                                                                      \
        *n1 = N1;                                                                                    \
        *threads = 2 * N1 * W;                                                                       \
        *smem = sizeof(float2) * ((size_t)3 * N1 * N2 * W + N1 * N2) + 64;                            \
        return named(&k_col_sign_fold<N1, N2, W>, "k_col_sign_fold<" #N1 "," #N2 "," #W ">");        \
    }

SignSbFn pick_sign_sb(int ndop, int ndb, int want_w, int want_n1, int* w, int* n1, int* threads, size_t* smem) {
    // the first instantiation listed for a size is its default (ndop 800: 32 x 25, four columns,
    // two CTAs per SM); the others are the autotuner's alternatives (ACQ_OPT_SEARCH_WIDTH / _SPLIT)
    ACQ_SFOLD_CASE(32, 25, 4) ACQ_SFOLD_CASE(32, 25, 8) ACQ_SFOLD_CASE(32, 25, 2) ACQ_SFOLD_CASE(40, 20, 2)
    ACQ_SFOLD_CASE(40, 20, 4) ACQ_SFOLD_CASE(32, 20, 8) ACQ_SFOLD_CASE(32, 40, 4) ACQ_SFOLD_CASE(20, 20, 8)
    ACQ_SFOLD_CASE(20, 10, 16)
    ACQ_SSB_CASE(16, 25, 8, 1)
    return nullptr;
}

}  // namespace acq

cudaError_t acq_inst_sign_upload_twiddles(const float2* host, size_t n) {
    return cudaMemcpyToSymbol(acq::c_regtw, host, sizeof(float2) * n);
}

ACQ_BC_SET_TABLE_IMPL(acq_inst_sign_set_bounds_table)
