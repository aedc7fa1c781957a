// Split-precision (BF16-slice emulated FP64) grouped GEMM on the tcgen05 tensor cores.
#pragma once

#include "ctrct.h"

namespace qltg {

void launch_gemm_split(CtrctPlan& p, const void* a, const void* b, void* c, cudaStream_t s);

}  // namespace qltg
