// Contraction plan: device-built task list, transpose work lists and the grouped-GEMM
// schedule for one C = A . B.
#pragma once

#include "qltg_internal.h"

namespace qltg {

// One block permutation for the batched transpose kernel (dst-order dims after
// squeezing unit dims and merging runs that stay adjacent).
struct PermDesc {
  int64_t src_off, dst_off;
  int64_t sstride[kMaxRank];   // source stride of each destination dim
  int32_t dims[kMaxRank];      // destination-order dims
  int32_t rank;
  int32_t p;                   // destination dim that is innermost in the source
  int32_t tiles_p, tiles_q;    // 32-wide tiles along p and along the innermost dst dim
  int64_t nouter;              // product of the remaining dims
  int64_t tile_begin;          // first global tile of this block
  double sign;
};

struct TransposeList {
  std::vector<PermDesc> host;
  DevBuf dev;
  int64_t ntiles = 0;
  int64_t nblocks = 0;
  void build(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
             const std::vector<int64_t>* dst_offsets, cudaStream_t s);
  // host-side descriptors only (fills host / ntiles / nblocks, no device memory)
  void describe(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
                const std::vector<int64_t>* dst_offsets);
  void launch(const void* src, void* dst, int elem_bytes, cudaStream_t s) const;
};

// Grouped GEMM schedule. C blocks own contiguous task ranges; tiles reference C blocks.
struct GemmCBlk {
  int64_t c_off;
  int32_t m, n;
  int32_t t0, t1;              // task range
};
struct GemmTask {
  int64_t a_off, b_off;        // offsets of the (transposed) operand blocks
  int32_t k;
  int32_t sign;                // fermion exchange sign
};
struct GemmTile {
  int32_t cblk;
  int16_t tm, tn;
};

struct GemmSchedule {
  std::vector<GemmCBlk> cblk;
  std::vector<GemmTask> task;
  std::vector<GemmTile> tile;
  DevBuf d_cblk, d_task, d_tile;
  int bm = 64, bn = 64;
};

struct CtrctPlan {
  qltg_ctx* ctx = nullptr;
  Meta a, b, c;
  std::vector<int64_t> axa, axb, sa, sb;
  bool a_trans = false, b_trans = false;
  std::vector<int> a_order, b_order;
  // tasks in the reference's generation order: a, b, c_blk_idx, m, k, n, sign, beta
  std::vector<int64_t> tasks_gen;
  double flops = 0, bytes = 0;
  TransposeList a_tl, b_tl;
  DevBuf a_t, b_t;             // transposed operand scratch
  GemmSchedule sched;
  int64_t launches_per_exec = 0;
};

void plan_contraction(CtrctPlan& p, cudaStream_t s);
void exec_contraction(CtrctPlan& p, const void* a, const void* b, void* c, int mode, cudaStream_t s, int stage = 0);

// grouped GEMM launchers (gemm_f64.cu)
void launch_gemm_f64(const GemmSchedule& g, const void* a, const void* b, void* c, bool cplx, int num_sms,
                     cudaStream_t s);

// Block order, destination offsets and fermionic block signs of QLTensor::Transpose.
void transpose_layout(const Meta& m, const std::vector<int>& order, std::vector<double>& signs,
                      std::vector<int64_t>& dst_off);

// Allocation-free permute: descriptors go to a fixed device table (at most
// kNoAllocPermBlocks blocks per call), see transpose.cu.
constexpr int kNoAllocPermBlocks = 4096;
void launch_permute_noalloc(int device, const TransposeList& tl, const void* src, void* dst, int elem_bytes,
                            cudaStream_t s);

// Fermionic exchange sign of one block pair (host copy of the device routine).
int host_exchange_sign(const bool* pa, int ra, const bool* pb, int rb, const int64_t* axa, const int64_t* axb,
                       int nax, const int32_t* a_ctrct_dirs);

}  // namespace qltg

struct qltg_ctrct_plan {
  qltg::CtrctPlan p;
};
