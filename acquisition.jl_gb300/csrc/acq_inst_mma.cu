// acq_inst_mma.cu — tensor-core rotation combine (k_rot_mma) for the instantiated geometries.
#include "acqgb300.h"
#include "acq_inst.h"
#include "acq_mma.cuh"

namespace acq {

namespace {
template <int NC, int NB, int QP, int CB>
RotMmaFn pick_prec(int prec, size_t* smem, const char* const name[4]) {
    using S = RotMmaShape<NC, NB, QP>;
    switch (prec) {
        case ACQ_PREC_FP16: *smem = S::smem_bytes(1); return named(&k_rot_mma<NC, NB, QP, CB, 0, 1>, name[0]);
        case ACQ_PREC_BF16: *smem = S::smem_bytes(1); return named(&k_rot_mma<NC, NB, QP, CB, 1, 1>, name[1]);
        case ACQ_PREC_FP16_SPLIT: *smem = S::smem_bytes(2); return named(&k_rot_mma<NC, NB, QP, CB, 0, 2>, name[2]);
        case ACQ_PREC_BF16_SPLIT: *smem = S::smem_bytes(2); return named(&k_rot_mma<NC, NB, QP, CB, 1, 2>, name[3]);
        default: return nullptr;
    }
}
}  // namespace

#define ACQ_MMA_NAME(NC, NB, QP, CB, F, S) "k_rot_mma<" #NC "," #NB "," #QP "," #CB "," F "," S ">"
#define ACQ_MMA_CASE(NC, NB, QP, CB)                                                                      \
    if (n_coh == NC && nb == NB && qp == QP && combos == CB) {                                           \
        static const char* const name[4] = {                                                            \
            ACQ_MMA_NAME(NC, NB, QP, CB, "fp16", "1"), ACQ_MMA_NAME(NC, NB, QP, CB, "bf16", "1"),        \
            ACQ_MMA_NAME(NC, NB, QP, CB, "fp16", "2"), ACQ_MMA_NAME(NC, NB, QP, CB, "bf16", "2")};       \
        return pick_prec<NC, NB, QP, CB>(prec, smem, name);                                              \
    }

RotMmaFn pick_rot_mma(int n_coh, int nb, int n_candidates, int combos, int prec, size_t* smem) {
    const int qp = (n_candidates + 7) / 8 * 8;
    ACQ_MMA_CASE(20, 25, 24, 2) ACQ_MMA_CASE(10, 20, 16, 1) ACQ_MMA_CASE(20, 12, 24, 2) ACQ_MMA_CASE(10, 16, 16, 1)
    ACQ_MMA_CASE(10, 4, 16, 1) ACQ_MMA_CASE(20, 20, 24, 2)
    return nullptr;
}

}  // namespace acq

cudaError_t acq_inst_mma_upload_twiddles(const float2* host, size_t n) {
    return cudaMemcpyToSymbol(acq::c_regtw, host, sizeof(float2) * n);
}

ACQ_BC_SET_TABLE_IMPL(acq_inst_mma_set_bounds_table)
