// acq_inst_sign.cu — data-bit / bit-edge and secondary-code rotation stages for hot ndop.
#include "acq_inst.h"

namespace acq {

#define ACQ_SIGN_CASE(N) \
    case N: return &k_col_sign_fs<best_split_n1(N), N / best_split_n1(N)>;
#define ACQ_ROT_CASE(N) \
    case N: return &k_col_rot_fs<best_split_n1(N), N / best_split_n1(N)>;

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

}  // namespace acq

cudaError_t acq_inst_sign_upload_twiddles(const float2* host, size_t n) {
    return cudaMemcpyToSymbol(acq::c_regtw, host, sizeof(float2) * n);
}
