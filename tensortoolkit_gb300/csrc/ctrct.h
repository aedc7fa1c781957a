// Contraction plan: device-built task list, transpose work lists and the grouped-GEMM
// schedule for one C = A . B.
#pragma once

#include <memory>

#include "qltg_internal.h"

namespace qltg {

// One block permutation for the batched transpose kernel (dst-order dims after
// squeezing unit dims and merging runs that stay adjacent).
struct PermDesc {
  int64_t src_off, dst_off;
  int64_t sstride[kMaxRank];   // source stride of each destination dim
  int32_t dims[kMaxRank];      // destination-order dims
  int32_t rank;
  int32_t p;                   // destination dim that is innermost in the source (-1: gather mode)
  int32_t tp, tq;              // tile extents along p and along the innermost dst dim
  int32_t tiles_p, tiles_q;    // tiles along p and along the innermost dst dim
  int32_t u, tu, tiles_u;      // batched outer dim (-1: none), its tile extent and tile count
  int64_t nouter;              // product of the remaining dims (gather mode: block size)
  int64_t tile_begin;          // first global work item of this block
  uint64_t sign_mask;          // 0, or the sign bit: the block's +-1 sign applied by XOR
};

struct TransposeList {
  std::vector<PermDesc> host;
  std::vector<uint8_t> identity;   // per block: its data layout is unchanged by the permutation
  DevBuf dev;
  int64_t ntiles = 0;
  int64_t nblocks = 0;
  // skip_identity: blocks whose layout the permutation leaves unchanged get no work (the
  // caller reads them from the source)
  void build(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
             const std::vector<int64_t>* dst_offsets, cudaStream_t s, bool skip_identity = false,
             const std::vector<uint8_t>* skip = nullptr);
  // host-side descriptors only (fills host / ntiles / nblocks, no device memory)
  void describe(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
                const std::vector<int64_t>* dst_offsets, bool skip_identity = false,
                const std::vector<uint8_t>* skip = nullptr);
  void launch(const void* src, void* dst, int elem_bytes, cudaStream_t s) const;
};

// Grouped GEMM schedule. C blocks own contiguous task ranges; tiles reference C blocks.
struct GemmCBlk {
  int64_t c_off;
  int32_t m, n;
  int32_t t0, t1;              // task range
};
struct GemmTask {
  int64_t a_off, b_off;        // offsets of the (transposed) operand blocks, | kFromSrc
  int32_t k;
  int32_t sign;                // fermion exchange sign
  int32_t a_rs, a_cs;          // skinny tasks: A element (row, kk) at row a_rs + kk a_cs
};
// Operand offset flag: the block is read from the untransposed operand, whose layout for
// this block already matches the transposed one (same offset in both buffers).
constexpr int64_t kFromSrc = (int64_t)1 << 62;
template <typename T>
__host__ __device__ __forceinline__ const T* operand_block(const T* scratch, const T* src, int64_t off) {
  return (off & kFromSrc) ? src + (off & ~kFromSrc) : scratch + off;
}
struct GemmTile {
  int32_t cblk;
  int16_t tm, tn;
};
struct GemmRowChunk {          // skinny output blocks: 256 consecutive rows of one block
  int32_t cblk;
  int32_t chunk;
};

// Row-scale fields of a later split-mode contraction's A operand, folded by the skinny kernel
// that writes that operand (the matvec's second MPO step writing the last step's A): per
// skinny output block, the first field of its rows in that operand and the operand's row
// length k3 (a multiple of the block's n); exp_base < 0: not folded.
struct SkinnyFuse {
  int32_t exp_base;
  int32_t k3;
};

struct GemmSchedule {
  std::vector<GemmCBlk> cblk;
  std::vector<GemmTask> task;
  std::vector<GemmTile> tile;           // 64 x 64 tiles (DMMA / DFMA kernels)
  std::vector<GemmRowChunk> skinny;     // row chunks of skinny blocks (n, k <= 8)
  DevBuf d_cblk, d_task, d_tile, d_skinny, d_counter;
  int bm = 32, bn = 32;
  int skinny_maxn = 8;                  // largest n of the skinny blocks (kernel variant)
};

// Split-precision schedule (gemm_split.cu): operand blocks to slice and pack, per-task
// packed-tile addresses, output tiles of 128 x 32.
//
// Row stacking: output blocks whose task lists pair the same B blocks with the same k and
// signs (the blocks of one "stack") are computed as one taller GEMM - their A blocks are
// packed one under the other into shared 128-row tiles (each A block at a row offset of a
// stacked operand), and each output row of a tile finds its place in C through a row map.
// Short blocks then share tiles instead of each padding its own to 128 rows.
struct SplitOperand {
  int64_t src_off;        // element offset of the (transposed) FP64 block
  int64_t pack_off;       // byte offset of its packed slice tiles (A: of its stacked operand)
  int32_t rows, cols;     // A: m x k; B: k x n
  int32_t ktiles;         // 64-wide k tiles
  int32_t exp_off;        // offset of its row (A) / column (B) exponent fields
  int64_t chunk_begin;    // A: prefix over operands of 8-element chunks (row-scale kernel)
  int64_t pchunk_begin;   // A: prefix over operands of rows x ceil(cols / 16) (pack kernel)
  int32_t cplx;           // B: complex block read as its real 2k x 2n form
  int32_t row_base;       // A: first row of this block in its stacked operand
};
// Schedule choices of one split-precision plan (picked by the tuner, or fixed).
struct SplitConfig {
  bool stack = true;      // row stacking of output blocks with the same task structure
  int max_stack_rows = 4096;
};
struct SplitTask {
  int64_t a_pack, b_pack;
  int32_t a_exp, b_exp;
  int32_t ktiles;
  int32_t sign;
};
// One (output tile, task) step of the split GEMM; the steps of one CTA are contiguous, in
// the order it processes them.
struct SplitWork {
  int64_t c_off;          // element offset of the first output block of the stack (reporting)
  int64_t a_pack, b_pack; // byte offsets of the operand blocks' packed slice tiles
  int32_t m, n;           // stacked output shape (rows of all blocks of the stack) x n
  int32_t a_exp, b_exp;   // exponent offsets of the operand blocks
  int32_t ktiles;         // 64-wide k tiles of the task
  int32_t k;              // contracted extent of the task
  int16_t tm, tn;         // 128-row / 32-column tile of the stacked output
  int8_t sign;            // sign of the task
  uint8_t flags;          // bit 0: first task of the tile, bit 1: last task of the tile
  uint8_t pad0[2];
  int32_t row_map;        // first entry of the stack's rows in the row map (C offset per row)
  uint8_t pad[4];
};
static_assert(sizeof(SplitWork) == 64, "SplitWork is one 64-byte record");
struct SplitPlan {
  bool built = false;
  bool a_static = false, b_static = false;   // operand packed once, unchanged afterwards
  bool a_ready = false, b_ready = false;
  std::vector<SplitOperand> a_ops, b_ops;
  SplitConfig cfg;
  std::vector<SplitTask> tasks;   // per stack, its task positions (stack_task0 offsets)
  std::vector<int32_t> stack_task0, stack_m, stack_n, stack_rowmap, stack_cblk0;   // per stack
  std::vector<int64_t> row_map;   // per stacked output row: its element offset in C
  std::vector<GemmTile> tiles;    // (stack, 128-row tile, 32-col tile), longest first
  std::vector<SplitWork> work;    // per CTA: tiles blockIdx.x, + grid, ...; each its tasks
  std::vector<int32_t> work_off;  // grid + 1 offsets into work
  int grid = 0;
  std::vector<int2> b_col_tiles;  // (B operand, 32-column tile) items of the B packing kernel
  int row_exp_grid = 1, pack_a_grid = 1, pack_b_grid = 1;   // one wave of resident CTAs of each
  int64_t n_a_chunks = 0, n_a_pchunks = 0, n_a_rows = 0;
  bool row_warp = false;          // A row scales one warp per row (long rows) or by chunks
  bool a_fields_external = false; // A row scales written by the kernel producing A (matvec)
  DevBuf d_a_ops, d_b_ops, d_work, d_work_off, a_packed, b_packed, a_exps, b_exps, error, d_b_col_tiles, d_row_map;
  // executed tensor work: 128 x 32 x 32 tile stages per launch, and the useful share of it
  int64_t tile_stages = 0;
  double useful_frac = 0.0;
  // a plan with skinny blocks and tiles runs the skinny kernel on a side stream (forked and
  // joined with events, capturable), beside the slicing kernels and the split GEMM
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  SplitPlan() = default;
  SplitPlan(const SplitPlan&) = delete;
  SplitPlan& operator=(const SplitPlan&) = delete;
  ~SplitPlan() {
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (side) cudaStreamDestroy(side);
  }
  void build(const struct CtrctPlan& p, cudaStream_t s);
  int64_t launches() const;
};

// A schedule choice of the tuner (tune.cu): FP64 tile rows and split-precision row stacking,
// with the timed GEMM stage of the chosen and of the slowest candidate.
struct TuneChoice {
  int f64_bm = 32;
  bool split_stack = true;
  float ms = 0.f, other_ms = 0.f;
};

struct CtrctPlan {
  qltg_ctx* ctx = nullptr;
  Meta a, b, c;
  std::vector<int64_t> axa, axb, sa, sb;
  // Optional order of the saved legs in C (empty: ascending, as Contract). A fermionic block
  // whose saved legs leave ascending order takes that reordering's sign (ContractContiguousAxes).
  std::vector<int64_t> sa_order, sb_order;
  bool a_trans = false, b_trans = false;
  std::vector<int> a_order, b_order;
  // tasks in the reference's generation order: a, b, c_blk_idx, m, k, n, sign, beta
  std::vector<int64_t> tasks_gen;
  double flops = 0, bytes = 0;
  TransposeList a_tl, b_tl;
  DevBuf a_t, b_t;             // transposed operand scratch
  GemmSchedule sched;
  std::unique_ptr<SplitPlan> split;   // built on first use of QLTG_MODE_SPLIT
  SplitConfig split_cfg;              // schedule choices the split plan is built with
  TuneChoice tuned[2];                // per mode (QLTG_MODE_FP64, QLTG_MODE_SPLIT): the tuner's choice
  bool is_tuned[2] = {false, false};
  DevBuf d_fuse;                      // split mode: SkinnyFuse per output block, or empty
  int32_t* fuse_fields = nullptr;     // the field array those blocks fold into
  int64_t launches_per_exec = 0;
};

void plan_contraction(CtrctPlan& p, cudaStream_t s);
// Schedule tuner (tune.cu): time the candidate GEMM schedules of `mode` on these operands
// and keep the fastest (cached per block-structure signature); *cached = taken from cache.
TuneChoice tune_plan(CtrctPlan& p, const void* a, const void* b, void* c, int mode, cudaStream_t s, bool* cached);
void apply_choice(CtrctPlan& p, int mode, const TuneChoice& c, cudaStream_t s);
uint64_t plan_signature(const CtrctPlan& p, int mode);
void set_f64_tile(CtrctPlan& p, int bm, int bn, cudaStream_t s);
// Grouped-GEMM schedule, operand transposes and device buffers of a planned contraction.
void finalize_plan(CtrctPlan& p, cudaStream_t s);
int64_t exec_launches_split(const CtrctPlan& p);
void exec_contraction(CtrctPlan& p, const void* a, const void* b, void* c, int mode, cudaStream_t s, int stage = 0);

// grouped GEMM launchers (gemm_f64.cu)
bool skinny_cblk(const GemmSchedule& g, int32_t q);
int skinny_rows_per_item();
// Grid of the skinny kernel: one full wave of resident CTAs (the first call queries the
// occupancy; call it once outside any stream capture).
int skinny_grid(int items, bool cplx, int maxn, int num_sms);
// Operand buffers of one execution: scratch (transposed blocks) and source (the operands as
// passed in, for blocks flagged kFromSrc).
struct Operands {
  const void* a;
  const void* a_src;
  const void* b;
  const void* b_src;
};
void launch_gemm_f64(const GemmSchedule& g, const Operands& op, void* c, bool cplx, int num_sms, cudaStream_t s);
void launch_gemm_f64_skinny(const GemmSchedule& g, const Operands& op, void* c, bool cplx, int num_sms,
                            cudaStream_t s, const SkinnyFuse* fuse = nullptr, int32_t* fields = nullptr);

// FP64 rate self-test (gemm_f64.cu): DFMA and mma.sync f64 throughput of this GPU, TFLOP/s.
void fp64_rates(int num_sms, cudaStream_t s, double* dfma_tflops, double* dmma_tflops);

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

struct qltg_transpose_plan {
  qltg_ctx* ctx = nullptr;
  int elem_bytes = 8;
  qltg::TransposeList tl;
};

struct qltg_ctrct_plan {
  qltg::CtrctPlan p;
};
