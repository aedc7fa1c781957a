// Split-precision grouped GEMM (placeholder until the tcgen05 kernel lands).
#include "split.h"

namespace qltg {

void launch_gemm_split(CtrctPlan&, const void*, const void*, void*, cudaStream_t) {
  throw Error(QLTG_ERR_UNSUPPORTED, "split-precision mode is not built yet");
}

}  // namespace qltg
