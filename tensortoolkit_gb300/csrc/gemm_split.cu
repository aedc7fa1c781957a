// Split-precision grouped GEMM: FP64 emulated with BF16 slices on the tcgen05 tensor
// cores, FP32 accumulation in tensor memory, exact integer recombination, one FP64
// rounding per output element.
//
// Slicing (per operand block, integer arithmetic only - the FP64 pipe of this GPU runs at
// about 1 TFLOP/s, so nothing here touches it):
//   every row i of A (column j of B) gets a scale 2^e with max |x| < 2^e, and each element
//   x = s 2^e y, |y| < 1, is cut into S = 7 base-2^7 digits of Y = floor(|y| 2^49):
//   x ~= 2^e sum_p a_p 2^(-7p) with integer slices a_p = s d_p in [-127, 127], exact in BF16.
//   Truncation error < 2^-49 of the row (column) maximum.
// Products (the Ozaki scheme, restated): C_ij = 2^(ea_i + eb_j) sum_l 2^(-7l) D_l with
//   D_l = sum_{p+q=l} (A_p B_q)_ij over the 28 slice pairs with p + q <= 8 (levels 2..8).
//   Every product a_p b_q is an integer of magnitude < 2^14; level l sums l-1 pairs, so over
//   at most 128 k the FP32 accumulation of every level is exact (7 * 128 * 127^2 < 2^24).
//   Each level has its own 128 x 32 FP32 accumulator in tensor memory (7 x 32 = 224
//   columns); every 128 k the levels are drained to two int64 registers per output
//   (levels 2-4 -> hi, 5-8 -> lo, both < 2^53), and at the end of a task
//   C += sign * 2^(ea+eb-56) (hi 2^28 + lo) with one FMA-rounding.
//
// Layout for the tensor cores: both operands K-major, no swizzle, in 8 x 16-byte core
// matrices (leading-byte offset 128 B between the two core matrices of a 16-wide k step,
// stride-byte offset 256 B between 8-row groups). The pack kernels write each (row tile,
// k tile, slice) as one contiguous tile in exactly that layout, zero-padded, so the GEMM
// stages operands with plain 16-byte copies and points the MMA descriptors at them.
//
// GEMM (one CTA of 128 threads per 128 x 32 output tile at a time, dynamic tile queue):
//   for each task of the output block, for each 64-wide k tile: all threads stage the 7 A
//   slices (7 x 16 KB) and 7 B slices (7 x 4 KB) into shared memory; one thread issues the
//   4 x 28 tcgen05.mma (M=128, N=32, K=16) and commits them to an mbarrier; after every
//   second k tile (and at the end of a task) the four warps read their 32 lanes of the 7
//   level accumulators with tcgen05.ld and fold them into the int64 pair.
// Every wait on the mbarrier is bounded; on expiry the CTA sets the plan's error word,
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "split.h"

namespace qltg {
namespace {

constexpr int kS = 7;                      // slices
constexpr int kPairs = 28;                 // p + q <= kS + 1
constexpr int kLevels = 7;                 // levels 2..8
constexpr int kTM = 128, kTN = 32, kTK = 64;
constexpr int kATile = kTM * kTK * 2;      // bytes of one (row tile, k tile, slice): 16 KB
constexpr int kBTile = kTN * kTK * 2;      // 4 KB
constexpr int kThreads = 128;
constexpr int kDrainK = 128;               // k between drains (exactness bound)
constexpr uint32_t kTmemCols = 256;        // >= 7 * 32, power of two

// ------------------------------------------------------------------ slicing
// Row / column scale exponents: e with max |x| < 2^e (0 for an all-zero row).
__device__ __forceinline__ int exp_of_bits(uint64_t absbits) {
  if (absbits == 0) return 0;
  const int ef = (int)(absbits >> 52);
  return ef == 0 ? -1021 : ef - 1022;     // subnormals: treat as 2^-1022 scale
}

// A (m x k row-major): one warp per row.
__global__ void k_row_exp(const double* __restrict__ src, const SplitOperand* __restrict__ ops, int nops,
                          int32_t* __restrict__ exps, int64_t total_rows) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t rg = warp; rg < total_rows; rg += nw) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (ops[mid].vec_begin <= rg) lo = mid; else hi = mid - 1; }
    const SplitOperand o = ops[lo];
    const int64_t r = rg - o.vec_begin;
    const double* row = src + o.src_off + r * o.cols;
    uint64_t mx = 0;
    for (int c = lane; c < o.cols; c += 32) {
      const uint64_t b = (uint64_t)__double_as_longlong(row[c]) & 0x7FFFFFFFFFFFFFFFull;
      mx = b > mx ? b : mx;
    }
    for (int sft = 16; sft > 0; sft >>= 1) {
      const uint64_t y = __shfl_xor_sync(0xffffffffu, mx, sft);
      mx = y > mx ? y : mx;
    }
    if (lane == 0) exps[o.exp_off + r] = exp_of_bits(mx);
  }
}

// B (k x n row-major): the scale of a column only depends on the largest exponent field in
// it, so threads take (column, 32-row chunk) items and fold into the column with atomicMax
// on the biased exponent (the array starts at zero); k_col_exp_finish turns fields into
// scale exponents.
__global__ void k_col_exp(const double* __restrict__ src, const SplitOperand* __restrict__ ops, int nops,
                          int32_t* __restrict__ exps, int64_t total_items) {
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < total_items;
       it += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (ops[mid].item_begin <= it) lo = mid; else hi = mid - 1; }
    const SplitOperand o = ops[lo];
    const int64_t l = it - o.item_begin;
    const int64_t c = l % o.cols, r0 = (l / o.cols) * 32;
    int mx = 0;
    const int64_t r1 = min((int64_t)o.rows, r0 + 32);
    for (int64_t r = r0; r < r1; ++r) {
      const uint64_t b = (uint64_t)__double_as_longlong(src[o.src_off + r * o.cols + c]) & 0x7FFFFFFFFFFFFFFFull;
      const int f = b == 0 ? 0 : max(1, (int)(b >> 52));
      mx = max(mx, f);
    }
    if (mx) atomicMax(&exps[o.exp_off + c], mx);
  }
}

__global__ void k_col_exp_finish(int32_t* __restrict__ exps, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    exps[i] = exps[i] == 0 ? 0 : exps[i] - 1022;
}

// Seven 7-bit digits of x / 2^e (sign-magnitude), as BF16 bit patterns.
__device__ __forceinline__ void slice7(double x, int e, uint16_t* out) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const uint64_t ab = bits & 0x7FFFFFFFFFFFFFFFull;
  uint64_t Y = 0;
  if (ab != 0) {
    const int ex = (int)(ab >> 52);
    const uint64_t mant = (ab & 0xFFFFFFFFFFFFFull) | (ex ? (1ull << 52) : 0ull);
    const int ee = ex ? ex : 1;
    // |x| = mant 2^(ee - 1075); Y = floor(|x| 2^(49 - e)) = mant >> (1075 + e - 49 - ee)
    const int sh = 1026 + e - ee;
    Y = sh >= 64 ? 0 : (mant >> sh);
  }
  const uint16_t sgn = (uint16_t)((bits >> 48) & 0x8000u);
#pragma unroll
  for (int p = 0; p < kS; ++p) {
    const uint32_t d = (uint32_t)((Y >> (7 * (kS - 1 - p))) & 127u);
    // bf16 of the integer d (exact): float bits >> 16
    const uint32_t f = __float_as_uint((float)d);
    out[p] = d ? (uint16_t)((f >> 16) | sgn) : (uint16_t)0;
  }
}

// Pack A operand tiles. One thread per 16-byte chunk (8 consecutive k of one row) per
// (row tile, k tile); writes the chunk of every slice plane.
__global__ void k_pack_a(const double* __restrict__ src, const SplitOperand* __restrict__ ops, int nops,
                         const int32_t* __restrict__ exps, uint8_t* __restrict__ pack, int64_t total_chunks) {
  for (int64_t ch = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ch < total_chunks;
       ch += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (ops[mid].chunk_begin <= ch) lo = mid; else hi = mid - 1; }
    const SplitOperand o = ops[lo];
    const int64_t l = ch - o.chunk_begin;
    // chunk order inside a (rt, kt) tile: ks (4), m_core (16), k_core (2), r8 (8) = 1024 chunks
    const int64_t tile = l >> 10;
    const int w = (int)(l & 1023);
    const int ks = w >> 8, m_core = (w >> 4) & 15, k_core = (w >> 3) & 1, r8 = w & 7;
    const int64_t rt = tile / o.ktiles, kt = tile % o.ktiles;
    const int64_t r = rt * kTM + m_core * 8 + r8;
    const int64_t k0 = kt * kTK + ks * 16 + k_core * 8;
    uint16_t sl[8][kS];
    const int e = r < o.rows ? exps[o.exp_off + r] : 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const double x = (r < o.rows && k0 + j < o.cols) ? src[o.src_off + r * o.cols + k0 + j] : 0.0;
      slice7(x, e, sl[j]);
    }
    const int64_t within = (int64_t)ks * 4096 + m_core * 256 + k_core * 128 + r8 * 16;
#pragma unroll
    for (int p = 0; p < kS; ++p) {
      uint4 v;
      v.x = (uint32_t)sl[0][p] | ((uint32_t)sl[1][p] << 16);
      v.y = (uint32_t)sl[2][p] | ((uint32_t)sl[3][p] << 16);
      v.z = (uint32_t)sl[4][p] | ((uint32_t)sl[5][p] << 16);
      v.w = (uint32_t)sl[6][p] | ((uint32_t)sl[7][p] << 16);
      *reinterpret_cast<uint4*>(pack + o.pack_off + (tile * kS + p) * (int64_t)kATile + within) = v;
    }
  }
}

// Pack B operand tiles (k x n row-major source, K-major tiles of 32 columns).
__global__ void k_pack_b(const double* __restrict__ src, const SplitOperand* __restrict__ ops, int nops,
                         const int32_t* __restrict__ exps, uint8_t* __restrict__ pack, int64_t total_chunks) {
  for (int64_t ch = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ch < total_chunks;
       ch += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (ops[mid].chunk_begin <= ch) lo = mid; else hi = mid - 1; }
    const SplitOperand o = ops[lo];
    const int64_t l = ch - o.chunk_begin;
    // chunk order inside a (ct, kt) tile: ks (4), n_core (4), k_core (2), n8 (8) = 256 chunks
    const int64_t tile = l >> 8;
    const int w = (int)(l & 255);
    const int ks = w >> 6, n_core = (w >> 4) & 3, k_core = (w >> 3) & 1, n8 = w & 7;
    const int64_t ct = tile / o.ktiles, kt = tile % o.ktiles;
    const int64_t c = ct * kTN + n_core * 8 + n8;        // output column (B column)
    const int64_t k0 = kt * kTK + ks * 16 + k_core * 8;  // B row
    uint16_t sl[8][kS];
    const int e = c < o.cols ? exps[o.exp_off + c] : 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const double x = (c < o.cols && k0 + j < o.rows) ? src[o.src_off + (k0 + j) * o.cols + c] : 0.0;
      slice7(x, e, sl[j]);
    }
    const int64_t within = (int64_t)ks * 1024 + n_core * 256 + k_core * 128 + n8 * 16;
#pragma unroll
    for (int p = 0; p < kS; ++p) {
      uint4 v;
      v.x = (uint32_t)sl[0][p] | ((uint32_t)sl[1][p] << 16);
      v.y = (uint32_t)sl[2][p] | ((uint32_t)sl[3][p] << 16);
      v.z = (uint32_t)sl[4][p] | ((uint32_t)sl[5][p] << 16);
      v.w = (uint32_t)sl[6][p] | ((uint32_t)sl[7][p] << 16);
      *reinterpret_cast<uint4*>(pack + o.pack_off + (tile * kS + p) * (int64_t)kBTile + within) = v;
    }
  }
}

// ------------------------------------------------------------------ tcgen05 helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  // start >> 4 | LBO (128 B) >> 4 << 16 | SBO (256 B) >> 4 << 32 | fixed 0b001 << 46; no swizzle
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = 32.
__device__ __forceinline__ uint32_t idesc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTN >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(id), "r"(acc));
}

// Wait for the mbarrier phase with a bounded spin: about 1 s of SM clock (2^31 cycles at
// the 2.07 GHz maximum), checked every 256 polls so the fast path is a bare try_wait.
constexpr long long kWaitCycles = 1ll << 31;

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  uint32_t done = 0;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mbar), "r"(phase));
  if (done) return true;
  const long long t0 = clock64();
  while (true) {
    for (int i = 0; i < 256; ++i) {
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(mbar), "r"(phase));
      if (done) return true;
    }
    if (clock64() - t0 > kWaitCycles) return false;
  }
}

// 2^n as a double built from its bit pattern (integer ops only), with an ldexp fallback
// outside the normal range.
__device__ __forceinline__ double pow2(int n) {
  if (n >= -1022 && n <= 1023) return __longlong_as_double((long long)(n + 1023) << 52);
  return ldexp(1.0, n);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

// Operand pipeline: a stage holds one 32-wide k slab of all 7 A slices (7 x 8 KB) and all
// 7 B slices (7 x 2 KB) = 70 KB; 3 stages = 210 KB of shared memory.
constexpr int kStages = 3;
constexpr int kKS = 32;                         // k per stage (2 MMA k-steps)
constexpr int kAStage = kTM * kKS * 2;          // 8 KB per A slice per stage
constexpr int kBStage = kTN * kKS * 2;          // 2 KB per B slice per stage
constexpr int kStageBytes = kS * (kAStage + kBStage);
constexpr int kSmemBytes = kStages * kStageBytes + 1024;
constexpr int kPeriod = kDrainK / kKS;          // stages between drains (4)
constexpr int kRoleThreads = 192;               // warp 0 producer, warp 1 MMA, warps 2-5 drain
constexpr uint32_t kTmemAlloc = 512;            // two buffers of 7 levels x 32 columns

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes));
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar));
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

// Bounded wait that also gives up as soon as another role has aborted.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t mbar, uint32_t phase, volatile int* abort_flag) {
  uint32_t done = 0;
  const long long t0 = clock64();
  while (true) {
    for (int i = 0; i < 256; ++i) {
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(mbar), "r"(phase));
      if (done) return true;
    }
    if (*abort_flag || clock64() - t0 > kWaitCycles) return false;
  }
}

// Warp-specialised split GEMM. All roles walk the same static sequence of work items
// (output tiles ti = blockIdx.x, blockIdx.x + gridDim.x, ...; for each its tasks; for each
// task its 32-wide k stages), so they agree on stage, period and buffer numbers without
// talking: the producer fills stage g % 3 once the MMAs of stage g - 3 released it; the
// MMA thread consumes stage g into TMEM buffer (period d) % 2 once the drain of period
// d - 2 released that buffer; the drain warps read a buffer after its MMAs completed and
// release it, and after a task's last period write the task's contribution to C.
__global__ void __launch_bounds__(kRoleThreads, 1)
    k_gemm_split(const GemmCBlk* __restrict__ cblk, const SplitTask* __restrict__ task,
                 const GemmTask* __restrict__ gtask, const GemmTile* __restrict__ tiles, int ntiles,
                 const uint8_t* __restrict__ apack, const uint8_t* __restrict__ bpack,
                 const int32_t* __restrict__ aexp, const int32_t* __restrict__ bexp, double* __restrict__ C,
                 int* __restrict__ err) {
  extern __shared__ uint8_t smem_dyn[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], accf_bar[2], acce_bar[2], fin_bar;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemAlloc));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) { mbar_init(smem_u32(&full_bar[s]), 1); mbar_init(smem_u32(&empty_bar[s]), 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(smem_u32(&accf_bar[b]), 1); mbar_init(smem_u32(&acce_bar[b]), 4); }
    mbar_init(smem_u32(&fin_bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_abort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint32_t sbase = smem_u32(smem);
  auto fail = [&]() {
    s_abort = 1;
    atomicExch(err, 1);
  };

  if (warp == 0 && lane == 0) {
    // ------------------------------------------------------------ producer
    uint32_t g = 0;
    for (int ti = blockIdx.x; ti < ntiles && !s_abort; ti += gridDim.x) {
      const GemmTile tl = tiles[ti];
      const GemmCBlk cb = cblk[tl.cblk];
      for (int t = cb.t0; t < cb.t1 && !s_abort; ++t) {
        const SplitTask tk = task[t];
        const int nst = (gtask[t].k + kKS - 1) / kKS;
        for (int j = 0; j < nst; ++j, ++g) {
          const int s = g % kStages;
          if (g >= (uint32_t)kStages &&
              !mbar_wait_or_abort(smem_u32(&empty_bar[s]), ((g / kStages) - 1) & 1, &s_abort)) { fail(); break; }
          const int kt = j >> 1, half = j & 1;
          const uint8_t* ga = apack + tk.a_pack + ((int64_t)tl.tm * tk.ktiles + kt) * kS * kATile + half * kAStage;
          const uint8_t* gb = bpack + tk.b_pack + ((int64_t)tl.tn * tk.ktiles + kt) * kS * kBTile + half * kBStage;
          const uint32_t sa = sbase + s * kStageBytes, sb = sa + kS * kAStage;
          const uint32_t fb = smem_u32(&full_bar[s]);
          mbar_expect_tx(fb, kStageBytes);
#pragma unroll
          for (int p = 0; p < kS; ++p) {
            bulk_g2s(sa + p * kAStage, ga + (int64_t)p * kATile, kAStage, fb);
            bulk_g2s(sb + p * kBStage, gb + (int64_t)p * kBTile, kBStage, fb);
          }
        }
      }
    }
    // copies still in flight are waited for by the MMA thread (every issued stage is
    // consumed on the normal path); on abort wait for the tail of issued stages here
    if (s_abort) {
      for (uint32_t x = (g > (uint32_t)kStages ? g - kStages : 0); x < g; ++x)
        mbar_wait_or_abort(smem_u32(&full_bar[x % kStages]), (x / kStages) & 1, &s_abort);
    }
  } else if (warp == 1 && lane == 0) {
    // ------------------------------------------------------------ MMA issuer
    const uint32_t id = idesc_bf16();
    // descriptor of stage 0, slice 1, k-step 0; every other operand is a fixed byte offset
    const uint64_t da0 = smem_desc(sbase), db0 = smem_desc(sbase + kS * kAStage);
    uint32_t g = 0, d = 0;
    for (int ti = blockIdx.x; ti < ntiles && !s_abort; ti += gridDim.x) {
      const GemmTile tl = tiles[ti];
      const GemmCBlk cb = cblk[tl.cblk];
      for (int t = cb.t0; t < cb.t1 && !s_abort; ++t) {
        const int nst = (gtask[t].k + kKS - 1) / kKS;
        for (int j = 0; j < nst; ++j, ++g) {
          const int s = g % kStages;
          const int buf = d & 1;
          const bool first = (j % kPeriod) == 0;
          const bool drain = (j % kPeriod) == kPeriod - 1 || j + 1 == nst;
          if (first && d >= 2 && !mbar_wait_or_abort(smem_u32(&acce_bar[buf]), ((d / 2) - 1) & 1, &s_abort)) {
            fail();
            break;
          }
          if (!mbar_wait_or_abort(smem_u32(&full_bar[s]), (g / kStages) & 1, &s_abort)) { fail(); break; }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t soff = (uint64_t)((s * kStageBytes) >> 4);
          const uint32_t dbuf = tmem + (uint32_t)(buf * kLevels * kTN);
#pragma unroll
          for (int ks = 0; ks < kKS / 16; ++ks) {
            int started = 0;
#pragma unroll
            for (int p = 1; p <= kS; ++p) {
#pragma unroll
              for (int q = 1; p + q <= kS + 1; ++q) {
                const int l = p + q - 2;
                const uint64_t adesc = da0 + soff + (uint64_t)(((p - 1) * kAStage + ks * 4096) >> 4);
                const uint64_t bdesc = db0 + soff + (uint64_t)(((q - 1) * kBStage + ks * 1024) >> 4);
                const uint32_t acc = (first && ks == 0 && !(started >> l & 1)) ? 0u : 1u;
                mma_bf16(dbuf + (uint32_t)(l * kTN), adesc, bdesc, id, acc);
                started |= 1 << l;
              }
            }
          }
          tc_commit(smem_u32(&empty_bar[s]));
          if (drain) { tc_commit(smem_u32(&accf_bar[buf])); ++d; }
        }
      }
    }
    // all MMAs issued by this thread complete before the tensor memory is released
    tc_commit(smem_u32(&fin_bar));
    mbar_wait_or_abort(smem_u32(&fin_bar), 0, &s_abort);
  } else if (warp >= 2) {
    // ------------------------------------------------------------ drain / epilogue
    const int quad = warp & 3;                       // TMEM lanes 32 * quad .. + 31
    const int row_in_tile = quad * 32 + lane;
    uint32_t d = 0;
    for (int ti = blockIdx.x; ti < ntiles && !s_abort; ti += gridDim.x) {
      const GemmTile tl = tiles[ti];
      const GemmCBlk cb = cblk[tl.cblk];
      const int row = tl.tm * kTM + row_in_tile;
      bool stop = false;
      for (int t = cb.t0; t < cb.t1 && !stop; ++t) {
        const SplitTask tk = task[t];
        const int nst = (gtask[t].k + kKS - 1) / kKS;
        long long hi[kTN], lo[kTN];
#pragma unroll
        for (int c = 0; c < kTN; ++c) hi[c] = lo[c] = 0;
        for (int j = 0; j < nst; ++j) {
          const bool drain = (j % kPeriod) == kPeriod - 1 || j + 1 == nst;
          if (!drain) continue;
          const int buf = d & 1;
          if (!mbar_wait_or_abort(smem_u32(&accf_bar[buf]), (d / 2) & 1, &s_abort)) {
            if (lane == 0) fail();
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * kLevels * kTN);
#pragma unroll 1
          for (int l = 0; l < kLevels; ++l) {
            uint32_t r[kTN];
            tmem_ld32(lane_base + (uint32_t)(l * kTN), r);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            const int wsh = l < 3 ? 7 * (2 - l) : 7 * (6 - l);
#pragma unroll
            for (int c = 0; c < kTN; ++c) {
              // exact integer below 2^24: the 32-bit conversion suffices
              const long long v = (long long)__float2int_rn(__uint_as_float(r[c])) * (1ll << wsh);
              if (l < 3) hi[c] += v; else lo[c] += v;
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;");
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&acce_bar[buf]));
          ++d;
        }
        if (stop) break;
        // C (+)= sign 2^(ea + eb - 56) (hi 2^28 + lo)
        if (row < cb.m) {
          const int ea = aexp[tk.a_exp + row];
          double* out = C + cb.c_off + (int64_t)row * cb.n;
#pragma unroll
          for (int c = 0; c < kTN; ++c) {
            const int col = tl.tn * kTN + c;
            if (col < cb.n) {
              const int eb = bexp[tk.b_exp + col];
              const double v = fma((double)hi[c], 268435456.0, (double)lo[c]);
              const double sc = tk.sign < 0 ? -pow2(ea + eb - 56) : pow2(ea + eb - 56);
              if (t == cb.t0) out[col] = v * sc; else out[col] = fma(v, sc, out[col]);
            }
          }
        }
      }
      if (stop) break;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemAlloc));
}

unsigned grid_for(int64_t n, int bs = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + bs - 1) / bs, 152 * 32));
}

}  // namespace

// ------------------------------------------------------------------ host side
void SplitPlan::build(const CtrctPlan& p, cudaStream_t s) {
  built = false;
  const GemmSchedule& g = p.sched;
  // operand blocks used by non-skinny output blocks
  std::vector<int32_t> a_of(p.a.nblk, -1), b_of(p.b.nblk, -1);
  a_ops.clear();
  b_ops.clear();
  tasks.clear();
  tiles.clear();
  int64_t a_pack = 0, b_pack = 0, a_exp = 0, b_exp = 0, a_vec = 0, b_vec = 0, a_chunks = 0, b_chunks = 0, b_items = 0;
  auto a_index = [&](int64_t a_off) {   // block ordinal from its offset
    return (int64_t)(std::lower_bound(p.a.offsets.begin(), p.a.offsets.end(), a_off) - p.a.offsets.begin());
  };
  auto b_index = [&](int64_t b_off) {
    return (int64_t)(std::lower_bound(p.b.offsets.begin(), p.b.offsets.end(), b_off) - p.b.offsets.begin());
  };
  tasks.resize(g.task.size());
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q) {
    const GemmCBlk& cb = g.cblk[q];
    if (skinny_cblk(g, q)) continue;
    for (int32_t t = cb.t0; t < cb.t1; ++t) {
      const GemmTask& gt = g.task[t];
      const int64_t ia = a_index(gt.a_off), ib = b_index(gt.b_off);
      const int k = gt.k;
      const int ktiles = (k + kTK - 1) / kTK;
      if (a_of[ia] < 0) {
        SplitOperand o{};
        o.src_off = gt.a_off;
        o.rows = cb.m;
        o.cols = k;
        o.ktiles = ktiles;
        o.exp_off = (int32_t)a_exp;
        o.vec_begin = a_vec;
        o.chunk_begin = a_chunks;
        o.pack_off = a_pack;
        const int64_t rtiles = (cb.m + kTM - 1) / kTM;
        a_exp += cb.m;
        a_vec += cb.m;
        a_chunks += rtiles * ktiles * 1024;
        a_pack += rtiles * ktiles * kS * (int64_t)kATile;
        a_of[ia] = (int32_t)a_ops.size();
        a_ops.push_back(o);
      }
      if (b_of[ib] < 0) {
        SplitOperand o{};
        o.src_off = gt.b_off;
        o.rows = k;
        o.cols = cb.n;
        o.ktiles = ktiles;
        o.exp_off = (int32_t)b_exp;
        o.vec_begin = b_vec;
        o.item_begin = b_items;
        o.chunk_begin = b_chunks;
        o.pack_off = b_pack;
        const int64_t ctiles = (cb.n + kTN - 1) / kTN;
        b_exp += cb.n;
        b_vec += cb.n;
        b_items += (int64_t)cb.n * ((k + 31) / 32);
        b_chunks += ctiles * ktiles * 256;
        b_pack += ctiles * ktiles * kS * (int64_t)kBTile;
        b_of[ib] = (int32_t)b_ops.size();
        b_ops.push_back(o);
      }
      const SplitOperand& oa = a_ops[a_of[ia]];
      const SplitOperand& ob = b_ops[b_of[ib]];
      QLTG_CHECK(oa.rows == cb.m && oa.cols == k && ob.rows == k && ob.cols == cb.n, QLTG_ERR_INVALID,
                 "internal: inconsistent operand shapes in the split schedule");
      tasks[t] = SplitTask{oa.pack_off, ob.pack_off, oa.exp_off, ob.exp_off, ktiles, gt.sign};
    }
    const int rtiles = (cb.m + kTM - 1) / kTM, ctiles = (cb.n + kTN - 1) / kTN;
    for (int i = 0; i < rtiles; ++i)
      for (int j = 0; j < ctiles; ++j) tiles.push_back(GemmTile{q, (int16_t)i, (int16_t)j});
  }
  QLTG_CHECK(tiles.size() < ((size_t)1 << 31), QLTG_ERR_UNSUPPORTED, "too many split tiles");
  // longest first: tiles of blocks with more k tiles
  std::vector<int64_t> cost(g.cblk.size(), 0);
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q)
    for (int32_t t = g.cblk[q].t0; t < g.cblk[q].t1; ++t) cost[q] += (g.task[t].k + 31) / 32;
  std::stable_sort(tiles.begin(), tiles.end(), [&](const GemmTile& x, const GemmTile& y) { return cost[x.cblk] > cost[y.cblk]; });
  n_a_vec = a_vec;
  n_b_vec = b_vec;
  n_a_chunks = a_chunks;
  n_b_chunks = b_chunks;
  n_b_items = b_items;
  d_a_ops = upload(a_ops, s);
  d_b_ops = upload(b_ops, s);
  d_tasks = upload(tasks, s);
  d_tiles = upload(tiles, s);
  a_packed.alloc(std::max<int64_t>(a_pack, 16));
  b_packed.alloc(std::max<int64_t>(b_pack, 16));
  a_exps.alloc(std::max<int64_t>(a_exp, 1) * 4);
  b_exps.alloc(std::max<int64_t>(b_exp, 1) * 4);
  counter.alloc(sizeof(int));
  error.alloc(sizeof(int));
  QLTG_CUDA(cudaMemsetAsync(error.get(), 0, sizeof(int), s));
  static bool attr_set = false;
  if (!attr_set) {
    QLTG_CUDA(cudaFuncSetAttribute(k_gemm_split, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    attr_set = true;
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
  built = true;
}

int64_t SplitPlan::launches() const {
  if (tiles.empty()) return 0;
  return (a_static ? 0 : 2) + (b_static ? 0 : 4) + 1;   // per side: (memset,) exps, (finish,) pack; GEMM
}

// Scale exponents and slice tiles of one operand side (A: rows, B: columns).
void pack_split_operand(SplitPlan& sp, bool side_a, const void* src, cudaStream_t s) {
  const double* X = static_cast<const double*>(src);
  if (side_a) {
    if (sp.a_ops.empty()) return;
    k_row_exp<<<grid_for(sp.n_a_vec * 32), 256, 0, s>>>(X, sp.d_a_ops.as<SplitOperand>(), (int)sp.a_ops.size(),
                                                        sp.a_exps.as<int32_t>(), sp.n_a_vec);
    k_pack_a<<<grid_for(sp.n_a_chunks), 256, 0, s>>>(X, sp.d_a_ops.as<SplitOperand>(), (int)sp.a_ops.size(),
                                                     sp.a_exps.as<int32_t>(), sp.a_packed.as<uint8_t>(),
                                                     sp.n_a_chunks);
  } else {
    if (sp.b_ops.empty()) return;
    QLTG_CUDA(cudaMemsetAsync(sp.b_exps.get(), 0, sp.n_b_vec * sizeof(int32_t), s));
    k_col_exp<<<grid_for(sp.n_b_items), 256, 0, s>>>(X, sp.d_b_ops.as<SplitOperand>(), (int)sp.b_ops.size(),
                                                     sp.b_exps.as<int32_t>(), sp.n_b_items);
    k_col_exp_finish<<<grid_for(sp.n_b_vec), 256, 0, s>>>(sp.b_exps.as<int32_t>(), sp.n_b_vec);
    k_pack_b<<<grid_for(sp.n_b_chunks), 256, 0, s>>>(X, sp.d_b_ops.as<SplitOperand>(), (int)sp.b_ops.size(),
                                                     sp.b_exps.as<int32_t>(), sp.b_packed.as<uint8_t>(),
                                                     sp.n_b_chunks);
  }
  QLTG_CUDA(cudaGetLastError());
  (side_a ? sp.a_ready : sp.b_ready) = true;
}

void split_prepack_static(CtrctPlan& p, const void* a_static, const void* b_static, cudaStream_t s) {
  if (!p.split || !p.split->built) return;
  const int eb = (int)p.a.elem_bytes();
  if (a_static) {
    const void* src = a_static;
    if (p.a_trans && p.a.size) { p.a_tl.launch(a_static, p.a_t.get(), eb, s); src = p.a_t.get(); }
    p.split->a_static = true;
    pack_split_operand(*p.split, true, src, s);
  }
  if (b_static) {
    const void* src = b_static;
    if (p.b_trans && p.b.size) { p.b_tl.launch(b_static, p.b_t.get(), eb, s); src = p.b_t.get(); }
    p.split->b_static = true;
    pack_split_operand(*p.split, false, src, s);
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
}

void launch_gemm_split(CtrctPlan& p, const void* a, const void* b, void* c, cudaStream_t s) {
  QLTG_CHECK(p.a.dtype == QLTG_F64, QLTG_ERR_UNSUPPORTED, "split-precision mode supports FP64 tensors");
  if (!p.split) {
    // first split-mode execution of this plan: build the slice schedule (allocates; not
    // allowed inside a stream capture - the matvec builds it before capturing)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    QLTG_CUDA(cudaStreamIsCapturing(s, &cs));
    QLTG_CHECK(cs == cudaStreamCaptureStatusNone, QLTG_ERR_INVALID,
               "split-precision schedule must be prepared before stream capture (run the plan once first)");
    prepare_split(p, s);
  }
  SplitPlan& sp = *p.split;
  // skinny output blocks stay on the FP64 skinny kernel (k, n <= 8: the tensor cores would
  // pad them 8x); everything else goes through the slices
  launch_gemm_f64_skinny(p.sched, a, b, c, false, p.ctx->num_sms, s);
  if (sp.tiles.empty()) return;
  if (!(sp.a_static && sp.a_ready)) pack_split_operand(sp, true, a, s);
  if (!(sp.b_static && sp.b_ready)) pack_split_operand(sp, false, b, s);
  const int grid = (int)std::min<int64_t>((int64_t)sp.tiles.size(), p.ctx->num_sms);
  k_gemm_split<<<grid, kRoleThreads, kSmemBytes, s>>>(
      p.sched.d_cblk.as<GemmCBlk>(), sp.d_tasks.as<SplitTask>(), p.sched.d_task.as<GemmTask>(), sp.d_tiles.as<GemmTile>(),
      (int)sp.tiles.size(),
      sp.a_packed.as<uint8_t>(), sp.b_packed.as<uint8_t>(), sp.a_exps.as<int32_t>(), sp.b_exps.as<int32_t>(),
      static_cast<double*>(c), sp.error.as<int>());
  QLTG_CUDA(cudaGetLastError());
}

void prepare_split(CtrctPlan& p, cudaStream_t s) {
  if (p.split && p.split->built) return;
  if (p.a.dtype != QLTG_F64) return;   // complex operands stay on the FP64 path
  p.split = std::make_unique<SplitPlan>();
  p.split->build(p, s);
}

int64_t split_launches(const CtrctPlan& p) {
  int64_t n = p.sched.skinny.empty() ? 0 : 1;
  if (p.split) n += p.split->launches();
  return n;
}

int split_device_error(const CtrctPlan& p, cudaStream_t s) {
  if (!p.split || !p.split->built) return 0;
  int e = 0;
  QLTG_CUDA(cudaMemcpyAsync(&e, p.split->error.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  QLTG_CUDA(cudaStreamSynchronize(s));
  return e;
}

}  // namespace qltg
