/*
 * qltg.h - C ABI of the GB300-native block-sparse hot path of TensorToolkit (qlten).
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an int
 * status (QLTG_OK = 0) and never exits the process. Device buffers are raw CUDA device
 * pointers holding a tensor's raw data in the reference's BlockSparseDataTensor layout:
 * blocks in ascending block index, each block row-major over its degeneracy dims, at
 * cumulative offsets (reference qltensor/blk_spar_data_ten/blk_spar_data_ten.h:53-572,
 * data_blk_operations.h:137-145). Complex data is interleaved (re, im) doubles, i.e.
 * std::complex<double>. Streams are passed as `void*` (a cudaStream_t, NULL = legacy
 * default stream).
 *
 * Ownership: callers own every tensor buffer they pass in. The library owns plans,
 * workspaces, CUDA graphs and the outputs of decompositions (freed with the matching
 * *_destroy call). Calls on one context are not thread-safe; use one context per thread.
 */
#ifndef QLTG_H_
#define QLTG_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define QLTG_API __attribute__((visibility("default")))
#else
#define QLTG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum {
  QLTG_OK = 0,
  QLTG_ERR_INVALID = 1,      /* malformed descriptor, axes or argument */
  QLTG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  QLTG_ERR_OOM = 3,          /* device allocation failed */
  QLTG_ERR_TIMEOUT = 4,      /* a bounded device-side wait expired */
  QLTG_ERR_NOCONV = 5,       /* an iterative decomposition did not converge */
  QLTG_ERR_EMPTY_SVD = 6,    /* no block fits lqndiv: reference EmptySVDResultError */
  QLTG_ERR_UNSUPPORTED = 7,  /* valid input outside what the library implements */
  QLTG_ERR_LAYOUT = 8        /* accumulate: the output's indexes differ from the contraction
                                result, or it lacks result blocks and expansion is off
                                (reference ContractAccumulateLayoutMismatch) */
};

enum { QLTG_F64 = 0, QLTG_C128 = 1 };     /* element types */
enum { QLTG_IN = 0, QLTG_OUT = 1 };       /* TenIndexDirType */

/* Arithmetic of a contraction.
 * QLTG_MODE_FP64:  plain FP64 on the FP64 pipe, the reference's precision.
 * QLTG_MODE_SPLIT: FP64 emulated with BF16 slices on the tcgen05 tensor cores: every row
 *                  of A / column of B is scaled by a power of two and cut into seven 7-bit
 *                  integer slices, the 28 slice products of weight >= 2^-56 accumulate
 *                  exactly (FP32 integers in tensor memory, drained every 256 k into int64),
 *                  and each task's sum is rounded to FP64 once. Per element the error is
 *                  below 2^-48 * sum_k |a_ik| |b_kj| scaled by the row / column maxima
 *                  (about 1e-14 relative for random data); the tests and the benchmark
 *                  state the measured relative error against the FP64 result. Real and
 *                  complex128 tensors (a complex product runs as the real product of A's
 *                  interleaved parts with B's 2 x 2 real form); output blocks with n, k <= 8
 *                  stay on the FP64 pipe. */
enum { QLTG_MODE_FP64 = 0, QLTG_MODE_SPLIT = 1 };

/* ---------------------------------------------------------------- descriptors */
/* Metadata of one block-sparse tensor (QLTensor indexes + block map). All arrays are
 * host memory borrowed for the duration of the call.
 * Mirrors: Index / QNSector (reference qltensor/index.h:45-229, qltensor/qnsct.h:34-139)
 * and the block map of BlockSparseDataTensor (blk_spar_data_ten.h:53-572). */
typedef struct qltg_tensor_desc {
  int32_t rank;
  int32_t dtype;            /* QLTG_F64 or QLTG_C128 */
  int32_t qn_ncomp;         /* integer components of one quantum number (U1QN: 1, fU1U1QN: 2) */
  int32_t parity_comp;      /* QN component whose oddness is the fermion parity; -1 = bosonic */
  const int32_t* dirs;      /* [rank]  QLTG_IN / QLTG_OUT */
  const int32_t* nsct;      /* [rank]  sectors per leg */
  const int32_t* qns;       /* [sum(nsct) * qn_ncomp] sector quantum numbers, leg by leg */
  const int64_t* dims;      /* [sum(nsct)] sector degeneracies, leg by leg */
  int64_t nblk;             /* stored blocks */
  const int64_t* coords;    /* [nblk * rank] sector coordinates, ascending block index */
} qltg_tensor_desc;

/* ---------------------------------------------------------------- context */
typedef struct qltg_ctx qltg_ctx;

/* Bind a context to CUDA device `device`. Replaces the reference's process-wide
 * cuBLAS/cuSOLVER/cuTENSOR handle singletons (framework/hp_numeric/gpu_set.h:30-192). */
QLTG_API int qltg_create(int device, qltg_ctx** ctx);
QLTG_API int qltg_destroy(qltg_ctx* ctx);

/* Message of the last failing call on this thread (never NULL). */
QLTG_API const char* qltg_last_error(void);

/* Failure-path self-test of the device-side bounded waits the tensor-core kernels use: one
 * warp waits on an mbarrier nothing arrives on, with a limit of limit_cycles (1 .. 2^31 SM
 * cycles). Returns QLTG_ERR_TIMEOUT when the wait gave up as designed (the expected result;
 * the context stays usable), QLTG_OK if it had completed. Synchronises `stream`. */
QLTG_API int qltg_selftest_bounded_wait(qltg_ctx* ctx, int64_t limit_cycles, void* stream);

/* Measured FP64 throughput of the device in TFLOP/s: a DFMA loop and an mma.sync m8n8k4 f64
 * (DMMA) loop over the whole GPU, timed with CUDA events (the reason the FP64 GEMM kernels use
 * DFMA: equal rates, and DMMA pads blocks to 8 x 8 x 4 fragments). No counterpart in the
 * reference. Synchronises `stream`. */
QLTG_API int qltg_selftest_fp64_rates(qltg_ctx* ctx, double* dfma_tflops, double* dmma_tflops, void* stream);

/* ---------------------------------------------------------------- contraction */
typedef struct qltg_ctrct_plan qltg_ctrct_plan;

/* Plan C = A . B over axes_a[i] <-> axes_b[i] (i < naxes). Replaces the constructor of
 * TensorContractionExecutor (reference tensor_manipulation/ten_ctrct.h:177-217): saved
 * axes, transpose orders, result legs = saved A legs ++ saved B legs, and the sector
 * pairing / task list of BlockSparseDataTensor::DataBlkGenForTenCtrct
 * (qltensor/blk_spar_data_ten/data_blk_operations.h:411-578), computed on the device.
 * Contracted legs must be inverse to each other (same sectors, opposite direction). */
QLTG_API int qltg_ctrct_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b,
                           const int64_t* axes_a, const int64_t* axes_b, int32_t naxes,
                           qltg_ctrct_plan** plan);

/* Result topology: rank, number of blocks and raw-data size (elements) of C. */
QLTG_API int qltg_ctrct_plan_result(const qltg_ctrct_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size);

/* C's block coordinates [nblk * rank] and offsets [nblk] (either may be NULL). The legs of
 * C are the saved legs of A followed by the saved legs of B, in order. */
QLTG_API int qltg_ctrct_plan_result_blocks(const qltg_ctrct_plan* plan, int64_t* coords, int64_t* offsets);

/* The task list in the reference's generation order (A blocks outer, B blocks inner),
 * 8 int64 per task: a_blk_idx, b_blk_idx, c_blk_idx, m, k, n, fermion sign (+-1),
 * beta (0 for the task that creates its output block). `tasks` may be NULL to query
 * *ntasks only. Mirrors RawDataCtrctTask (raw_data_operation_tasks.h:196-248). */
QLTG_API int qltg_ctrct_plan_tasks(const qltg_ctrct_plan* plan, int64_t* ntasks, int64_t* tasks);

/* Algorithmic FLOPs (sum of 2mkn, 8mkn for complex) and the bytes of A, B and C. */
QLTG_API int qltg_ctrct_plan_stats(const qltg_ctrct_plan* plan, double* flops, double* bytes);

/* Execute: c_dev (C's raw buffer, size from qltg_ctrct_plan_result) = A . B.
 * Replaces BlockSparseDataTensor::CtrctTwoBSDTAndAssignIn (global_operations.h:895-992):
 * per-block transposes, then one persistent grouped GEMM over all tasks, each output tile
 * accumulating all of its tasks before a single store. Asynchronous on `stream`. */
QLTG_API int qltg_ctrct_exec(qltg_ctrct_plan* plan, const void* a_dev, const void* b_dev, void* c_dev,
                    int32_t mode, void* stream);

/* The stages of qltg_ctrct_exec, separately, for profiling: stage 1 runs only the operand
 * transposes into the plan's scratch, stage 2 only the grouped GEMM (reading the operands
 * left by the last stage-1 call on this plan; in split mode this includes slicing the
 * operands), stage 3 only the GEMM kernels (split mode: on the slices packed by the last
 * stage-2 call; QLTG_ERR_INVALID before any), stage 0 all of it. */
QLTG_API int qltg_ctrct_exec_stage(qltg_ctrct_plan* plan, const void* a_dev, const void* b_dev, void* c_dev,
                                   int32_t mode, int32_t stage, void* stream);

/* Wait for `stream`, then report the device-side status of the plan's kernels: QLTG_OK, or
 * QLTG_ERR_TIMEOUT if a bounded tensor-core wait expired (the kernel then stopped early and
 * its output is not valid). */
QLTG_API int qltg_ctrct_plan_device_status(qltg_ctrct_plan* plan, void* stream);

QLTG_API int qltg_ctrct_plan_destroy(qltg_ctrct_plan* plan);

/* Schedule of a plan's grouped GEMM stage. No counterpart in the reference, which issues one
 * cublasDgemm per task (framework/hp_numeric/blas_level3.h:797-856) and has no schedule.
 * f64_tile_rows: rows of the FP64 output tiles, 32 or 64 (x 32 columns); 0 keeps it.
 * split_stack: split-precision row stacking (output blocks with the same task structure share
 * 128-row tiles), 1 on, 0 off, -1 keeps it. Rebuilds the affected schedule (allocates and
 * synchronises `stream`; not inside a stream capture). Results are the same under every
 * schedule (to rounding). */
QLTG_API int qltg_ctrct_plan_set_schedule(qltg_ctrct_plan* plan, int32_t f64_tile_rows, int32_t split_stack,
                                          void* stream);
/* The current schedule and, per mode (index QLTG_MODE_FP64 / QLTG_MODE_SPLIT), whether the
 * tuner chose it (tuned[mode] = 1) and the GEMM-stage times it measured for the chosen and
 * the slowest candidate (ms[2 mode], ms[2 mode + 1]). Any out-pointer may be NULL. */
QLTG_API int qltg_ctrct_plan_get_schedule(const qltg_ctrct_plan* plan, int32_t* f64_tile_rows, int32_t* split_stack,
                                          int32_t* tuned, float* ms);
/* Autotune the schedule of `mode`: every candidate (FP64: 32 x 32 and 64 x 32 tiles; split:
 * stacking on and off) runs on these operands (c_dev is overwritten), timed with CUDA events
 * on `stream`, and the fastest is kept. The choice is cached per device and block-structure
 * signature for the life of the process; a plan with the same signature takes it without
 * timing (*from_cache = 1). Synchronises `stream`; not inside a stream capture. */
QLTG_API int qltg_ctrct_plan_tune(qltg_ctrct_plan* plan, const void* a_dev, const void* b_dev, void* c_dev,
                                  int32_t mode, void* stream, int32_t* from_cache);
/* Executed tensor work of the plan's split-precision GEMM (after its first split-mode use):
 * 128 x 32 output-tile stages of 32 k per launch, and the share of them that is not padding
 * (m n k summed over tasks / (stages 128 32 32)). Zero before the split schedule exists. */
QLTG_API int qltg_ctrct_plan_split_stats(const qltg_ctrct_plan* plan, int64_t* tile_stages, double* useful_frac);

/* ------------------------------------------------ contiguous-axes contraction, accumulation */
enum { QLTG_SIDE_HEAD = 0, QLTG_SIDE_TAIL = 1 };

/* Plan for ContractContiguousAxes<ASide, BSide>(A, B, a_start, b_start, n, C) (reference
 * tensor_manipulation/contract_contiguous_axes.h:849-868): A's axes (a_start + i) mod rank_A
 * against B's (b_start + i) mod rank_B, i < n; C's legs are A's saved legs then B's, each in
 * cyclic order from the end of its contracted range (a fermionic block whose saved legs leave
 * ascending order takes that reordering's sign, as the reference's residue sign,
 * qltensor/blk_spar_data_ten/data_blk_operations.h:580-611). a_side / b_side
 * (QLTG_SIDE_HEAD / QLTG_SIDE_TAIL) are the reference's layout hints; the result does not
 * depend on them. The returned plan is a contraction plan: query and execute it with
 * qltg_ctrct_plan_result / _result_blocks / qltg_ctrct_exec. */
QLTG_API int qltg_ctrct_plan_create_contiguous(qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b,
                                               int64_t a_start, int64_t b_start, int32_t n, int32_t a_side,
                                               int32_t b_side, qltg_ctrct_plan** plan);

typedef struct qltg_accum_plan qltg_accum_plan;

/* Plan for C = beta C + alpha A.B with the tail/head contiguous contraction of
 * ContractTailHeadContiguousAccumulate (allow_expand = 1) or
 * TryContractTailHeadContiguousAccumulate (allow_expand = 0)
 * (contract_contiguous_axes.h:953-1040; executor :333-472, :557-783).
 * c_in NULL: C is default (exec then needs beta == 0) and the output is the contraction's
 * topology. Otherwise c_in's legs must equal the contraction result's (else
 * QLTG_ERR_LAYOUT); its blocks may be a superset. If it lacks result blocks the output is
 * the union topology (*expanded = 1) or, with allow_expand = 0, QLTG_ERR_LAYOUT and no plan
 * (the reference's Try form returning false). */
QLTG_API int qltg_accum_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b,
                                    int64_t a_start, int64_t b_start, int32_t n, const qltg_tensor_desc* c_in,
                                    int32_t allow_expand, qltg_accum_plan** plan, int32_t* expanded);
/* Output topology: rank, blocks, elements (scalar outputs: 1 element). */
QLTG_API int qltg_accum_plan_result(const qltg_accum_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size);
QLTG_API int qltg_accum_plan_result_blocks(const qltg_accum_plan* plan, int64_t* coords, int64_t* offsets);
/* c_out_dev = beta c_in_dev + alpha A.B (alpha, beta: {re, im}; imaginary parts must be 0
 * for FP64 tensors). Blocks of the old C the contraction does not touch are scaled by beta,
 * new blocks get alpha A.B; beta == 0 never reads c_in_dev. c_out_dev may be c_in_dev unless
 * the output was expanded. mode: QLTG_MODE_FP64 or QLTG_MODE_SPLIT (real tensors). */
QLTG_API int qltg_accum_exec(qltg_accum_plan* plan, const void* a_dev, const void* b_dev, const void* c_in_dev,
                             void* c_out_dev, const double* alpha, const double* beta, int32_t mode, void* stream);
QLTG_API int qltg_accum_plan_device_status(qltg_accum_plan* plan, void* stream);
QLTG_API int qltg_accum_plan_destroy(qltg_accum_plan* plan);

/* ---------------------------------------------------------------- transpose */
/* dst = A transposed to leg order `perm` (new leg i = old leg perm[i]), blocks reordered to
 * ascending block index of the permuted tensor, each block multiplied by its fermionic
 * exchange sign when the tensor is fermionic. Mirrors QLTensor::Transpose /
 * BlockSparseDataTensor::Transpose (qltensor/qltensor_impl.h:448-464,
 * global_operations.h:393-441) with DataBlk sign from FermionicInplaceReorder
 * (utility/utils_inl.h:52-75). dst must hold the same number of elements as src. */
QLTG_API int qltg_transpose(qltg_ctx* ctx, const qltg_tensor_desc* a, const void* src_dev,
                   const int32_t* perm, void* dst_dev, void* stream);

/* Reusable permute plan: the per-block work list of qltg_transpose for one tensor layout and
 * permutation is built and uploaded once; each exec is one asynchronous kernel launch
 * (no host work, no allocation). Replaces building an HPTT / cuTENSOR plan per block per
 * call (framework/hp_numeric/ten_trans.h:56-114, :245-349). Same result as qltg_transpose
 * (fermionic block signs included). */
typedef struct qltg_transpose_plan qltg_transpose_plan;
QLTG_API int qltg_transpose_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* a, const int32_t* perm, void* stream,
                                        qltg_transpose_plan** plan);
QLTG_API int qltg_transpose_plan_exec(qltg_transpose_plan* plan, const void* src_dev, void* dst_dev, void* stream);
QLTG_API int qltg_transpose_plan_destroy(qltg_transpose_plan* plan);

/* Same result as qltg_transpose, but allocates nothing: no cudaMalloc / cudaFree and no
 * allocating library call. No counterpart in the reference. It is for callers that cannot
 * allocate device memory while they run: a host whose device memory is all handed out up
 * front to another framework's pool (a cudaMalloc there fails or evicts that pool's cache),
 * or a latency-critical loop that cannot afford cudaMalloc / cudaFree, which synchronise the
 * device. The per-block work list goes to a fixed table of at most 4096 blocks compiled into
 * the library (about 600 KB, held by every GPU that loads the library until the process
 * exits); larger tensors are rejected with QLTG_ERR_INVALID. The first call on a device looks
 * up that table's device address (once per device, with the device current) and keeps it for
 * the life of the process, so the library must not outlive a cudaDeviceReset; make that first
 * call before any stream capture. All calls share the table and it keeps the last call's
 * descriptors: calls that overlap on the GPU race. The call copies its descriptors from host
 * memory and synchronises `stream` before it returns. */
QLTG_API int qltg_transpose_noalloc(qltg_ctx* ctx, const qltg_tensor_desc* a, const void* src_dev,
                                    const int32_t* perm, void* dst_dev, void* stream);

/* ---------------------------------------------------------------- dmrg axis primitives
 * The reference's bosonic qlten::dmrg axis operations (tensor_manipulation/dmrg/axis_ops.h);
 * fermionic tensors are rejected with QLTG_ERR_UNSUPPORTED, as there. */

/* out = beta out + alpha D(in): ApplyAxisDiagonal (axis_ops.h:2370-2547); with out_dev ==
 * in_dev, alpha 1, beta 0 it is ApplyAxisDiagonalInPlace (:2549-2582). values: one per
 * degeneracy of `axis`, sectors in index order (AxisDiagonalOp::values flattened; complex
 * interleaved). beta == 0 never reads out_dev. The output has the input's topology. */
QLTG_API int qltg_axis_diagonal(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis, const double* values,
                                const void* in_dev, void* out_dev, const double* alpha, const double* beta,
                                void* stream);
/* out = in with every block times the value of its sector on `axis`:
 * ApplyAxisSectorScalarsPreserveOrder (axis_ops.h:2655-2744). out_dev may be in_dev. */
QLTG_API int qltg_axis_sector_scalars(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis,
                                      const double* values_by_sector, const void* in_dev, void* out_dev,
                                      void* stream);

typedef struct qltg_axis_plan qltg_axis_plan;
/* ApplyRank2ToAxisPreserveOrder (axis_ops.h:2862-2993): `axis` of t contracted with op's index
 * 0 (op index 0 must be the inverse of t's leg), op's index 1 takes the axis' place. */
QLTG_API int qltg_axis_rank2_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, const qltg_tensor_desc* op,
                                         int32_t axis, qltg_axis_plan** plan);
/* ApplyTwoRank2ToAxesPreserveOrder (axis_ops.h:2995-3126): op1 on axis1, then op2 on axis2. */
QLTG_API int qltg_axis_two_rank2_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, const qltg_tensor_desc* op1,
                                             int32_t axis1, const qltg_tensor_desc* op2, int32_t axis2,
                                             qltg_axis_plan** plan);
/* ApplyAxisMonomial (axis_ops.h:2746-2860): `axis` of t replaced by the output index
 * (out_nsct sectors: out_qns, out_dims; t's direction); entries[4 e .. 4 e + 3] = (in_sector,
 * in_offset, out_sector, out_offset) with coefs[e] (complex: interleaved), each satisfying
 * output qn = input qn + flux. Output blocks: t's blocks mapped through every matching entry.
 * Execute with qltg_axis_monomial_exec. */
QLTG_API int qltg_axis_monomial_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis, int32_t out_nsct,
                                            const int32_t* out_qns, const int64_t* out_dims, const int32_t* flux,
                                            int64_t nentries, const int64_t* entries, const double* coefs,
                                            qltg_axis_plan** plan);
/* ProjectAxis (axis_ops.h:2469-2532): kept_counts[s] degeneracies kept from input sector s,
 * their offsets concatenated in `kept` (each in range and unique within its sector; at least
 * one kept overall). Sectors keeping none leave the output index; the others keep their
 * quantum number and order, degeneracies in the listed order. Execute with
 * qltg_axis_monomial_exec (alpha 1, beta 0). */
QLTG_API int qltg_axis_project_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis,
                                           const int64_t* kept_counts, const int64_t* kept, qltg_axis_plan** plan);
/* out = beta out + alpha M(in) over the generated topology (beta == 0 never reads out_dev). */
QLTG_API int qltg_axis_monomial_exec(qltg_axis_plan* plan, const void* in_dev, void* out_dev, const double* alpha,
                                     const double* beta, void* stream);
QLTG_API int qltg_axis_plan_result(const qltg_axis_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size);
QLTG_API int qltg_axis_plan_result_blocks(const qltg_axis_plan* plan, int64_t* coords, int64_t* offsets);
/* out_dev (the result topology) from in_dev and the operators (op2_dev: two-operator plans). */
QLTG_API int qltg_axis_plan_exec(qltg_axis_plan* plan, const void* in_dev, const void* op1_dev, const void* op2_dev,
                                 void* out_dev, int32_t mode, void* stream);
QLTG_API int qltg_axis_plan_device_status(qltg_axis_plan* plan, void* stream);
QLTG_API int qltg_axis_plan_destroy(qltg_axis_plan* plan);

/* ---------------------------------------------------------------- linear combination
 * out = sum_i coefs[i] T_i + beta res over the union of the blocks of the contributing
 * tensors (coefs[i] != 0; res when beta != 0, or always with keep_res), ascending block
 * index: LinearCombine (tensor_manipulation/ten_linear_combine.h:33-197); AddScaledAssign
 * (:211-221) is ({alpha}, {x}, beta 1, res y). All tensors share the indexes of T_0
 * (QLTG_ERR_LAYOUT otherwise); 1 to 64 tensors of rank >= 1; coefs and beta interleaved for
 * complex tensors. beta != 0 needs res. */
typedef struct qltg_lincomb_plan qltg_lincomb_plan;
QLTG_API int qltg_lincomb_plan_create(qltg_ctx* ctx, int32_t n, const qltg_tensor_desc* const* tens,
                                      const double* coefs, const qltg_tensor_desc* res, const double* beta,
                                      int32_t keep_res, qltg_lincomb_plan** plan);
QLTG_API int qltg_lincomb_plan_result(const qltg_lincomb_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size);
QLTG_API int qltg_lincomb_plan_result_blocks(const qltg_lincomb_plan* plan, int64_t* coords, int64_t* offsets);
/* out_dev may be a T_i's or res's buffer only when that tensor has the output's topology. */
QLTG_API int qltg_lincomb_exec(qltg_lincomb_plan* plan, const void* const* tens_dev, const void* res_dev,
                               void* out_dev, void* stream);
QLTG_API int qltg_lincomb_plan_destroy(qltg_lincomb_plan* plan);

/* ---------------------------------------------------------------- .qlten stream I/O
 * The reference's QLTensor serialisation (qltensor/qltensor_impl.h:799-830, index.h:170-188,
 * qnsct.h:106-115, special_qn/u1qn.h / u1u1qn.h, blk_spar_data_ten.h:791-830,
 * raw_data_operations.h:583-640): text header (rank; per index its sectors with quantum
 * numbers, degeneracies and hashes, direction, dimension, hash; the block coordinates), then
 * the raw buffer. Quantum number types: qn_ncomp 1 = U1QN, 2 = U1U1QN (parity_comp -1) or
 * fU1U1QN (parity_comp 0). */
typedef struct qltg_qlten_file qltg_qlten_file;

/* Parse a file's header; every stored hash is checked (a wrong quantum number type fails). */
QLTG_API int qltg_qlten_open(const char* path, int32_t qn_ncomp, int32_t parity_comp, int32_t elem_type,
                             qltg_qlten_file** file);
/* rank, sum of sector counts over the legs, blocks (a scalar: 1), elements. */
QLTG_API int qltg_qlten_info(const qltg_qlten_file* file, int32_t* rank, int64_t* total_sectors, int64_t* nblk,
                             int64_t* size);
/* Descriptor arrays (as qltg_tensor_desc; qns / dims leg by leg). */
QLTG_API int qltg_qlten_meta(const qltg_qlten_file* file, int32_t* dirs, int32_t* nsct, int32_t* qns,
                             int64_t* dims, int64_t* coords);
/* The raw buffer into device memory (dst_is_device = 1: through a pinned staging buffer,
 * copied on `stream`, complete on return) or host memory. */
QLTG_API int qltg_qlten_read_data(qltg_qlten_file* file, void* dst, int32_t dst_is_device, void* stream);
QLTG_API int qltg_qlten_close(qltg_qlten_file* file);
/* Write tensor `t` with raw buffer `data` (device or host memory) as a .qlten stream that the
 * reference reads with operator>>; byte-identical to what the reference writes. */
QLTG_API int qltg_qlten_write(const char* path, const qltg_tensor_desc* t, const void* data, int32_t data_is_device,
                              void* stream);

/* ---------------------------------------------------------------- two-site matvec */
typedef struct qltg_matvec qltg_matvec;

/* Plan and capture (one CUDA graph) the two-site effective-Hamiltonian product
 *   t1 = lenv.psi {{0},{0}};  t2 = t1.mpo1 {{0,2},{0,1}};
 *   t3 = t2.mpo2 {{4,1},{0,1}};  out = t3.renv {{4,1},{1,0}}
 * exactly as the reference's chain (tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257).
 * The operator buffers must stay valid and unchanged while the matvec lives. */
QLTG_API int qltg_matvec_create(qltg_ctx* ctx, const qltg_tensor_desc* lenv, const void* lenv_dev,
                       const qltg_tensor_desc* psi, const qltg_tensor_desc* mpo1, const void* mpo1_dev,
                       const qltg_tensor_desc* mpo2, const void* mpo2_dev,
                       const qltg_tensor_desc* renv, const void* renv_dev, int32_t mode, void* stream,
                       qltg_matvec** mv);

/* Topology of the result (rank 4: a', s1', s2', r'). */
QLTG_API int qltg_matvec_result(const qltg_matvec* mv, int64_t* nblk, int64_t* size);
QLTG_API int qltg_matvec_result_blocks(const qltg_matvec* mv, int64_t* coords, int64_t* offsets);

/* Algorithmic FLOPs of one product and the number of kernel launches in its graph. */
QLTG_API int qltg_matvec_stats(const qltg_matvec* mv, double* flops, int64_t* launches);

/* out_dev = H_eff . psi_dev (one graph launch on `stream`). */
QLTG_API int qltg_matvec_apply(qltg_matvec* mv, const void* psi_dev, void* out_dev, void* stream);
/* The same with host buffers, both page-locked (cudaMallocHost / cudaHostAlloc): psi copied
 * in, the product, the result copied out, all on `stream`. Asynchronous: the result is in
 * out_host once `stream` has completed. */
QLTG_API int qltg_matvec_apply_host(qltg_matvec* mv, const void* psi_host, void* out_host, void* stream);

/* Device-side status of the four captured contractions (see qltg_ctrct_plan_device_status). */
QLTG_API int qltg_matvec_device_status(qltg_matvec* mv, void* stream);

/* The form of the matvec's MPO part. No counterpart in the reference, whose chain is four
 * Contract calls. With W12 = W1 . W2 contracted over the middle MPO bond once at creation,
 * the two MPO steps become one, t3 = t1 . W12: the same result to rounding, without the
 * intermediate t2. qltg_matvec_create times both forms and keeps the faster one.
 * qltg_matvec_mpo_form reports: *fused (1 = the fused form runs), *fusable (0 when W12 cannot
 * replace the two steps) and ms[0], ms[1] = the MPO part timed at creation in the two-step and
 * the fused form. qltg_matvec_set_mpo_form forces a form (QLTG_ERR_UNSUPPORTED when not
 * fusable); only before the matvec's first apply and before a Lanczos is created on it. */
QLTG_API int qltg_matvec_mpo_form(const qltg_matvec* mv, int32_t* fused, int32_t* fusable, float* ms);
QLTG_API int qltg_matvec_set_mpo_form(qltg_matvec* mv, int32_t fused, void* stream);

/* The GEMM schedule the tuner chose for contraction `step` (0..3) of the matvec when it was
 * created, as qltg_ctrct_plan_get_schedule reports it, and that step's split-precision tile
 * stages and useful share (qltg_ctrct_plan_split_stats; zero in plain FP64 mode). */
QLTG_API int qltg_matvec_schedule(const qltg_matvec* mv, int32_t step, int32_t* f64_tile_rows, int32_t* split_stack,
                                  int32_t* tuned, float* ms, int64_t* tile_stages, double* useful_frac);

QLTG_API int qltg_matvec_destroy(qltg_matvec* mv);

/* ---------------------------------------------------------------- Lanczos (device vectors)
 * Lanczos on a matvec's effective Hamiltonian (real FP64 or complex128, either precision
 * mode of the matvec) with every vector operation on the device in FP64: the reference's
 * BSDT vector primitives (Dot / Norm / ScaleByFactor / LinearCombine on the raw buffer:
 * framework/hp_numeric/blas_level1.h, complex forms :381-1080,
 * tensor_manipulation/ten_linear_combine.h:186-459, raw_data_operations.h:225-272) applied to
 * Krylov vectors that share ψ's block topology. Step j: w = H v_j, two passes of classical
 * Gram-Schmidt against v_0..v_j with <x, y> = Σ conj(x) y (alpha_j = Re <v_j, H v_j> with
 * both corrections; real for a Hermitian H),
 * beta_{j+1} = ||w||, v_{j+1} = w / beta_{j+1}; deterministic reductions. Each step is one
 * CUDA graph (built on the step's first use; later starts reuse it). alpha and beta stay on
 * the device until qltg_lanczos_coeffs. The eigenvalues of the tridiagonal matrix are left
 * to the caller (a small dense FP64 problem). */
typedef struct qltg_lanczos qltg_lanczos;

/* Krylov space of up to max_iter + 1 vectors (max_iter 1..63) for matvec `mv`, which must
 * outlive the Lanczos object. */
QLTG_API int qltg_lanczos_create(qltg_matvec* mv, int32_t max_iter, qltg_lanczos** lz);
/* v_0 = psi0 / ||psi0|| (psi0 in ψ's raw layout); beta_0 = ||psi0||; resets the step count. */
QLTG_API int qltg_lanczos_start(qltg_lanczos* lz, const void* psi0_dev, void* stream);
/* One step (asynchronous on `stream`). QLTG_ERR_INVALID after max_iter steps. */
QLTG_API int qltg_lanczos_step(qltg_lanczos* lz, void* stream);
/* Copies alpha_0..alpha_{n-1} and beta_0..beta_n (n = steps taken, written to *nsteps);
 * synchronises `stream`. A beta of 0 means the Krylov space became invariant. */
QLTG_API int qltg_lanczos_coeffs(qltg_lanczos* lz, int32_t* nsteps, double* alpha, double* beta, void* stream);
/* Device address of Krylov vector v_i (0 <= i <= steps), ψ's raw layout. */
QLTG_API int qltg_lanczos_vector(const qltg_lanczos* lz, int32_t i, const void** v_dev);
QLTG_API int qltg_lanczos_destroy(qltg_lanczos* lz);

/* ---------------------------------------------------------------- decompositions */
typedef struct qltg_decomp qltg_decomp;

/* Truncated block SVD: T (legs 0..ldims-1 | ldims..rank-1) = U S Vt, mirroring
 * qlten::SVD (tensor_manipulation/ten_decomp/ten_svd.h:244-263): block-matrices grouped by
 * (left flux, right flux) (ten_decomp/ten_decomp_basic.h:68-106), all block-matrices
 * decomposed in one batched one-sided Jacobi launch, truncation keeping from Dmin while
 * the kept weight <= (1 - trunc_err) of the total and <= Dmax (ten_svd.h:281-372) - on the
 * device, over all values in descending order with ties by block-matrix, then rank -,
 * U with a new OUT leg, S = (IN, OUT) diagonal, Vt with a new IN leg (ten_svd.h:467-582).
 * `lqndiv` has qn_ncomp components. Returns QLTG_ERR_EMPTY_SVD when nothing is kept. */
QLTG_API int qltg_svd(qltg_ctx* ctx, const qltg_tensor_desc* t, const void* t_dev, int32_t ldims,
             const int32_t* lqndiv, double trunc_err, int64_t dmin, int64_t dmax, void* stream,
             qltg_decomp** out);

/* Block QR: T = Q R (Householder, one batched launch), mirroring qlten::QR
 * (tensor_manipulation/ten_decomp/ten_qr.h:152-162): mid leg dim min(rows, cols) per
 * block-matrix, Q with a new OUT leg, R with a new IN leg, LAPACK sign convention. */
QLTG_API int qltg_qr(qltg_ctx* ctx, const qltg_tensor_desc* t, const void* t_dev, int32_t ldims,
            const int32_t* lqndiv, void* stream, qltg_decomp** out);

/* SVD: actual truncation error and kept dimension D (QR: 0 and the mid dimension). */
QLTG_API int qltg_decomp_info(const qltg_decomp* d, double* trunc_err, int64_t* kept_dim);

/* Result tensors: SVD which = 0 U, 1 S, 2 Vt; QR which = 0 Q, 1 R.
 * info[0..5] = rank, qn_ncomp, dtype, nblk, size, total sectors. */
QLTG_API int qltg_decomp_tensor_info(const qltg_decomp* d, int32_t which, int64_t* info);

/* Copy the metadata of a result tensor into caller arrays sized from the info call and
 * return its library-owned device buffer in *dev (valid until qltg_decomp_destroy). */
QLTG_API int qltg_decomp_tensor_export(const qltg_decomp* d, int32_t which, int32_t* dirs, int32_t* nsct,
                              int32_t* qns, int64_t* dims, int64_t* coords, int64_t* offsets,
                              const void** dev);

QLTG_API int qltg_decomp_destroy(qltg_decomp* d);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* QLTG_H_ */
