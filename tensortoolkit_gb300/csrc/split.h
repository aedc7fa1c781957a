// Split-precision (BF16-slice emulated FP64) grouped GEMM on the tcgen05 tensor cores.
#pragma once

#include "ctrct.h"

namespace qltg {

// pack = false skips slicing the operands (they must have been packed by an earlier call).
void launch_gemm_split(CtrctPlan& p, const Operands& op, void* c, cudaStream_t s, bool pack = true);
// Build the slice schedule of a plan (allocates; call before any stream capture).
void prepare_split(CtrctPlan& p, cudaStream_t s);
// Pack an operand that stays constant for the plan's lifetime once, now (either may be NULL).
void split_prepack_static(CtrctPlan& p, const void* a_static, const void* b_static, cudaStream_t s);
// Kernel launches of one split-mode execution of the GEMM stage.
int64_t split_launches(const CtrctPlan& p);
// Device error word of the split GEMM (1 = a bounded tensor-core wait expired).
int split_device_error(const CtrctPlan& p, cudaStream_t s);
// One warp's bounded wait on an mbarrier nothing arrives on: 1 when it gave up after
// limit_cycles (expected), 0 if it completed.
int wait_selftest(int64_t limit_cycles, cudaStream_t s);

}  // namespace qltg
