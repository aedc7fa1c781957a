// Block SVD / QR (placeholder until the batched Jacobi / Householder kernels land).
#include "ctrct.h"

using namespace qltg;

struct qltg_decomp {};

extern "C" {

int qltg_svd(qltg_ctx*, const qltg_tensor_desc*, const void*, int32_t, const int32_t*, double, int64_t, int64_t,
             void*, qltg_decomp**) {
  return guarded([&] { throw Error(QLTG_ERR_UNSUPPORTED, "qltg_svd not built yet"); });
}
int qltg_qr(qltg_ctx*, const qltg_tensor_desc*, const void*, int32_t, const int32_t*, void*, qltg_decomp**) {
  return guarded([&] { throw Error(QLTG_ERR_UNSUPPORTED, "qltg_qr not built yet"); });
}
int qltg_decomp_info(const qltg_decomp*, double*, int64_t*) { return QLTG_ERR_UNSUPPORTED; }
int qltg_decomp_tensor_info(const qltg_decomp*, int32_t, int64_t*) { return QLTG_ERR_UNSUPPORTED; }
int qltg_decomp_tensor_export(const qltg_decomp*, int32_t, int32_t*, int32_t*, int32_t*, int64_t*, int64_t*,
                              int64_t*, const void**) {
  return QLTG_ERR_UNSUPPORTED;
}
int qltg_decomp_destroy(qltg_decomp* d) { delete d; return QLTG_OK; }

}
