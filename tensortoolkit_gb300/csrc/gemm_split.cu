// Split-precision grouped GEMM: FP64 emulated with BF16 slices on the tcgen05 tensor
// cores, FP32 accumulation in tensor memory, integer recombination, one FP64 rounding per
// output element (per task of the output block).
//
// Slicing (per operand block, integer arithmetic only - the FP64 pipe of this GPU runs at
// about 1 TFLOP/s, so nothing on the hot path leans on it):
//   every row i of A (column j of B) gets a scale 2^e with max |x| < 2^e, and each element
//   x = s 2^e y, |y| < 1, is cut into S = 7 base-2^7 digits of Y = floor(|y| 2^49):
//   x ~= 2^e sum_p a_p 2^(-7p), digits a_p = s d_p in [-127, 127]. Slice p is stored as
//   the BF16 number a_p 2^(-7p) (exact: 7 significant bits). Truncation error < 2^-49 of
//   the row (column) maximum.
// Products (the Ozaki scheme, restated): C_ij = 2^(ea_i + eb_j) sum over the 28 slice pairs
//   p + q <= 8 of (A_p B_q)_ij. Level L = p + q sums L - 1 pairs, each an integer multiple
//   of 2^(-7L) below 2^14 of those units. Each level has its own 128 x 32 FP32 accumulator
//   in tensor memory (levels 2..8: 224 columns per set, two sets). Over 256 k the sums of
//   levels 2..5 stay below 2^24 and are exact; levels 6..8 may round in FP32, at most
//   2^-24 of a quantity 2^-28 below the leading level. Every 256 k the drain warps read the
//   levels and fold them into one int64 per output (units 2^-49); at the end of a task
//   C (+)= sign 2^(ea + eb - 49) z, rounded to FP64 with integer operations.
//
// Layout for the tensor cores: both operands K-major, no swizzle, in 8 x 16-byte core
// matrices (leading-byte offset 128 B between the two core matrices of a 16-wide k step,
// stride-byte offset 256 B between 8-row groups). The pack kernels write each (row tile,
// k tile, slice) as one contiguous tile in exactly that layout, zero-padded, so the GEMM
// stages operands with bulk copies and points the descriptors at them.
//
// GEMM: one persistent CTA per SM, warp-specialised (see k_gemm_split): a producer warp
// streams 32-wide k slabs of all A and B slices into shared memory, an MMA warp issues per
// 16-wide k step 7 MMAs (A slice p against B slices 1..8-p concatenated along N), sixteen
// drain warps fold the accumulators. Output rows reach C through a row map, so the A blocks
// of several output blocks can share one 128-row tile (row stacking).
// Every wait on an mbarrier is bounded; on expiry the CTA sets the plan's error word,
// waits (bounded) for its own copies and tensor-core work, frees its tensor memory and
// returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <queue>

#include "scaled_int.h"
#include "split.h"

namespace qltg {
namespace {

constexpr int kS = 7;                      // slices
constexpr int kLevels = 7;                 // accumulators: levels 2..8
constexpr int kTM = 128, kTN = 32, kTK = 64;
constexpr int kATile = kTM * kTK * 2;      // bytes of one (row tile, k tile, slice): 16 KB
constexpr int kBTile = kTN * kTK * 2;      // 4 KB
constexpr int kDrainK = 256;               // k between drains (exactness bound of levels 2..5)

// ------------------------------------------------------------------ slicing
// Work distribution of the slicing kernels: CTA b takes the contiguous item range
// [b per, (b + 1) per); a thread finds the operand owning its first item once and walks
// forward from there (items only grow).
// Row / column scales are kept as exponent fields F: 0 for an all-zero row (column), else
// max(1, largest biased exponent field of |x|), so that atomicMax can fold them. The scale
// exponent is e = F - 1022 (max |x| < 2^e; subnormal-only rows use 2^-1021), 0 for F = 0.
__device__ __forceinline__ int field_of_bits(uint64_t absbits) {
  // 32-bit halves only: 64-bit compares and shifts cost extra issue slots
  const uint32_t hi = (uint32_t)(absbits >> 32), lo = (uint32_t)absbits;
  return (hi | lo) ? max(1, (int)(hi >> 20)) : 0;
}
__device__ __forceinline__ int exp_of_field(int f) { return f ? f - 1022 : 0; }

// |x| / 2^e as the 49-bit integer Y = floor(|x| 2^(49 - e)) and the sign as a BF16 sign bit,
// in 32-bit halves: Y = (hidden bit : fraction) >> sh with sh = 1026 + e - max(ex, 1) >= 4
// (|x| < 2^e); zero has no hidden bit and a zero fraction, so it gives Y = 0.
__device__ __forceinline__ uint64_t scaled_y(double x, int e, uint32_t& sgn) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  sgn = (hi >> 16) & 0x8000u;
  const uint32_t ex = (hi >> 20) & 0x7FFu;
  const uint32_t mhi = (hi & 0xFFFFFu) | (ex ? 0x100000u : 0u);
  const int sh = 1026 + e - (int)max(ex, 1u);
  const bool small = sh < 32;
  const uint32_t yl = small ? __funnelshift_r(lo, mhi, sh) : (mhi >> min(sh - 32, 31));
  const uint32_t yh = small ? (mhi >> sh) : 0u;
  return ((uint64_t)yh << 32) | yl;
}
// Slice p of two elements as one word of two BF16 values: digit d = bits 7 (kS - 1 - p) ..
// + 6 of Y, value d 2^(-7(p+1)) with the element's sign. The digit is or-ed into the
// mantissa of 2^23 (float 2^23 + d), one FMA scales and removes the 2^23 exactly (d has at
// most 7 significant bits, so the float's low 16 bits are zero and its high half is the
// exact BF16), one byte permute takes both high halves.
template <int P>
__device__ __forceinline__ uint32_t digit_magic(uint64_t y) {
  const uint32_t hi = (uint32_t)(y >> 32), lo = (uint32_t)y;
  constexpr int sh = 7 * (kS - 1 - P);
  uint32_t x;
  if constexpr (sh >= 32) x = hi >> (sh - 32);
  else if constexpr (sh + 7 > 32) x = __funnelshift_r(lo, hi, sh);
  else x = lo >> sh;
  return (x & 127u) | 0x4B000000u;
}
template <int P>
__device__ __forceinline__ uint32_t plane_pair(uint64_t y0, uint64_t y1, uint32_t sgn_pair) {
  const float scale = __uint_as_float((uint32_t)(127 - 7 * (P + 1)) << 23);
  const float f0 = __fmaf_rn(__uint_as_float(digit_magic<P>(y0)), scale, -8388608.0f * scale);
  const float f1 = __fmaf_rn(__uint_as_float(digit_magic<P>(y1)), scale, -8388608.0f * scale);
  return __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632) | sgn_pair;
}
// The 7 slice planes of 8 consecutive elements, written as 16-byte words at dst + p stride.
__device__ __forceinline__ void store_planes(const uint64_t* y, const uint32_t* sg, uint8_t* dst, int stride) {
  const uint32_t s01 = sg[0] | (sg[1] << 16), s23 = sg[2] | (sg[3] << 16), s45 = sg[4] | (sg[5] << 16),
                 s67 = sg[6] | (sg[7] << 16);
#define QLTG_PLANE(P)                                                                           \
  {                                                                                             \
    uint4 v;                                                                                    \
    v.x = plane_pair<P>(y[0], y[1], s01);                                                       \
    v.y = plane_pair<P>(y[2], y[3], s23);                                                       \
    v.z = plane_pair<P>(y[4], y[5], s45);                                                       \
    v.w = plane_pair<P>(y[6], y[7], s67);                                                       \
    *reinterpret_cast<uint4*>(dst + P * stride) = v;                                            \
  }
  QLTG_PLANE(0) QLTG_PLANE(1) QLTG_PLANE(2) QLTG_PLANE(3) QLTG_PLANE(4) QLTG_PLANE(5) QLTG_PLANE(6)
#undef QLTG_PLANE
}

// Row scales of A as exponent fields: every thread takes 8 consecutive elements of one
// operand block (blocks are dense row-major m x k), folds the exponent fields of each row it
// touches and adds them with atomicMax (one or two per thread unless the rows are short).
// Operand blocks are laid end to end in units of 8-element chunks (chunk_begin).
__global__ void __launch_bounds__(256) k_row_field(const double* __restrict__ scr, const double* __restrict__ src,
                                                   const SplitOperand* __restrict__ ops, int nops,
                                                   int64_t total_chunks, int32_t* __restrict__ fields) {
  // contiguous chunk range per CTA, so a thread's chunks stay in one operand block or move
  // to the next ones: one binary search, then a forward scan
  const int64_t per = (total_chunks + gridDim.x - 1) / gridDim.x;
  const int64_t cbeg = (int64_t)blockIdx.x * per, cend = min(total_chunks, cbeg + per);
  int lo = 0;
  {
    int hi = nops - 1;
    const int64_t first = cbeg + threadIdx.x;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ops[mid].chunk_begin <= first) lo = mid; else hi = mid - 1;
    }
  }
  // uniform trip count across the CTA: the warp-wide match below needs all 32 lanes
  for (int64_t base = cbeg; base < cend; base += blockDim.x) {
    const int64_t ch = base + threadIdx.x;
    const bool valid = ch < cend;
    int k1 = -1, v1 = 0, k2 = -2, v2 = 0;
    if (valid) {
      while (lo + 1 < nops && ops[lo + 1].chunk_begin <= ch) ++lo;
      const SplitOperand o = ops[lo];
      const int n = o.rows * o.cols;   // one block: below 2^31 elements (checked on the host)
      const int e0 = (int)(ch - o.chunk_begin) * 8;
      const double* blk = operand_block(scr, src, o.src_off);
      uint64_t v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = e0 + j < n ? (uint64_t)__double_as_longlong(__ldg(blk + e0 + j)) : 0ull;
      int r = e0 / o.cols;
      int c = e0 - r * o.cols;
      // the chunk's first row (r0, f0) and last row (r, f); rows strictly between (blocks
      // with fewer than 8 columns) are added directly
      const int r0 = r;
      int f = 0, f0 = -1;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (e0 + j < n) {
          if (c == o.cols) {
            if (f0 < 0) f0 = f;
            else if (f) atomicMax(fields + o.exp_off + r, f);
            f = 0;
            ++r;
            c = 0;
          }
          f = max(f, field_of_bits(v[j] & 0x7FFFFFFFFFFFFFFFull));
          ++c;
        }
      }
      k1 = o.exp_off + r0;
      v1 = f0 < 0 ? f : f0;
      if (f0 >= 0) {
        k2 = o.exp_off + r;
        v2 = f;
      }
    }
    // warp aggregation: lanes adding to the same row combine first, one lane adds
    const int lane = threadIdx.x & 31;
    const unsigned m1 = __match_any_sync(0xffffffffu, k1);
    const int x1 = (int)__reduce_max_sync(m1, (unsigned)v1);
    if (k1 >= 0 && x1 && lane == __ffs(m1) - 1) atomicMax(fields + k1, x1);
    const unsigned m2 = __match_any_sync(0xffffffffu, k2);
    const int x2 = (int)__reduce_max_sync(m2, (unsigned)v2);
    if (k2 >= 0 && x2 && lane == __ffs(m2) - 1) atomicMax(fields + k2, x2);
  }
}

// Row scales of A for long rows: one warp per row (rows of all A operands end to end, in
// exponent-offset order), loads along the row coalesced across the warp, a warp max, one
// store per row (no zero fill, no atomics).
__global__ void __launch_bounds__(256) k_row_field_rows(const double* __restrict__ scr, const double* __restrict__ src,
                                                        const SplitOperand* __restrict__ ops, int nops, int64_t nrows,
                                                        int32_t* __restrict__ fields) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < nrows; g += nwarps) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ops[mid].exp_off <= g) lo = mid; else hi = mid - 1;
    }
    const SplitOperand o = ops[lo];
    const double* row = operand_block(scr, src, o.src_off) + (g - o.exp_off) * (int64_t)o.cols;
    uint32_t mx = 0, nz = 0;
#pragma unroll 4
    for (int c = lane; c < o.cols; c += 32) {
      const uint64_t b = (uint64_t)__double_as_longlong(__ldg(row + c)) & 0x7FFFFFFFFFFFFFFFull;
      mx = max(mx, (uint32_t)(b >> 32));
      nz |= (uint32_t)b | (uint32_t)(b >> 32);
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    nz = __reduce_or_sync(0xffffffffu, nz);
    if (lane == 0) fields[g] = nz ? max(1, (int)(mx >> 20)) : 0;
  }
}

// Slices of A: one thread per 16-wide k step of one row that holds operand data (its two
// 16-byte chunks, 8 consecutive k each), numbered per operand in (128-row tile, k step, row)
// order, so consecutive threads take consecutive rows and their 16-byte plane words land
// side by side. CTA b takes the contiguous range [b per, (b + 1) per) of all operands' items.
__global__ void __launch_bounds__(256) k_pack_a(const double* __restrict__ scr, const double* __restrict__ src,
                                                const SplitOperand* __restrict__ ops, int nops, int64_t total,
                                                const int32_t* __restrict__ exps, uint8_t* __restrict__ pack) {
  const int64_t per = (total + gridDim.x - 1) / gridDim.x;
  const int64_t cbeg = (int64_t)blockIdx.x * per, cend = min(total, cbeg + per);
  int lo = 0;
  {
    int hi = nops - 1;
    const int64_t first = cbeg + threadIdx.x;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ops[mid].pchunk_begin <= first) lo = mid; else hi = mid - 1;
    }
  }
  for (int64_t ch = cbeg + threadIdx.x; ch < cend; ch += blockDim.x) {
    while (lo + 1 < nops && ops[lo + 1].pchunk_begin <= ch) ++lo;
    const SplitOperand o = ops[lo];
    const int npair = (o.cols + 15) >> 4;        // 16-wide k steps of a row
    const int l = (int)(ch - o.pchunk_begin);   // below 2^31: one block has < 2^31 elements
    const int rt = l / (kTM * npair);
    const int l2 = l - rt * kTM * npair;
    const int rows_rt = min(kTM, o.rows - rt * kTM);
    const int kp = l2 / rows_rt;
    const int r = l2 - kp * rows_rt;
    const int64_t row = (int64_t)rt * kTM + r;
    const int k0 = kp * 16;
    const int e = exp_of_field(__ldg(exps + o.exp_off + row));
    const double* src_row = operand_block(scr, src, o.src_off) + row * o.cols;
    // the row's place in its stacked operand: 128-row tile vt, row vr inside it
    const int vrow = o.row_base + (int)row;
    const int vt = vrow / kTM, vr = vrow - vt * kTM;
    // tile layout [ks][slice][m_core][k_core][8 rows x 16 B]: the 7 slices of a 16-wide k
    // step are contiguous, so a 32-wide stage is one 56 KB copy
    const int kt = k0 / kTK, ks = (k0 % kTK) >> 4;
    const int64_t tile = (int64_t)vt * o.ktiles + kt;
    uint8_t* dst = pack + o.pack_off + tile * (int64_t)(kS * kATile) + (int64_t)ks * (kS * 4096) + (vr >> 3) * 256 +
                   (vr & 7) * 16;
#pragma unroll
    for (int half = 0; half < 2; ++half) {   // k_core 0 and 1: the two 8-wide chunks of the step
      const int kb = k0 + 8 * half;
      if (kb >= o.cols) break;
      uint64_t y[8];
      uint32_t sg[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) y[j] = scaled_y((kb + j < o.cols) ? __ldg(src_row + kb + j) : 0.0, e, sg[j]);
      store_planes(y, sg, dst + half * 128, 4096);
    }
  }
}

// Element (r, c) of a B operand block: the block itself (k x n row-major), or for a complex
// block (k x n complex, interleaved) its real 2k x 2n form of 2 x 2 blocks [[Re, Im], [-Im, Re]].
template <bool CPLX>
__device__ __forceinline__ double b_elem(const double* __restrict__ blk, int64_t r, int c, int cols) {
  if constexpr (!CPLX) return __ldg(blk + r * cols + c);
  const double v = __ldg(blk + (r >> 1) * cols + (c & ~1) + ((r ^ c) & 1));
  return ((r & 1) && !(c & 1)) ? -v : v;
}

// Column scales and slices of B (k x n row-major), one CTA per (operand block, 32-column
// tile). Phase 1: thread (row group g, column c) folds rows g, g + 8, ... of its column (a
// warp reads 32 consecutive columns of one row); the 8 partial maxima per column meet in
// shared memory. Phase 2: one thread per 16-byte chunk (8 consecutive k of one column) of
// every 64-wide k tile writes the chunk of every slice plane.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_pack_b_cols(const double* __restrict__ scr, const double* __restrict__ src,
                                                     const SplitOperand* __restrict__ ops,
                                                     const int2* __restrict__ col_tiles, int ntiles,
                                                     int32_t* __restrict__ exps, uint8_t* __restrict__ pack) {
  __shared__ uint32_t smx[8][kTN], snz[8][kTN];
  __shared__ int se[kTN];
  const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    const int2 tt = col_tiles[ti];
    const SplitOperand o = ops[tt.x];
    const double* blk = operand_block(scr, src, o.src_off);
    const int c0 = tt.y * kTN;
    const int nc = min(kTN, o.cols - c0);
    uint32_t mx = 0, nz = 0;   // largest high word of |x|, any nonzero bit
    if (lane < nc) {
      const double* col = blk + c0 + lane;
      for (int r = g; r < o.rows; r += 32) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if constexpr (CPLX)
            v[u] = r + 8 * u < o.rows ? b_elem<true>(blk, r + 8 * u, c0 + lane, o.cols) : 0.0;
          else
            v[u] = r + 8 * u < o.rows ? __ldg(col + (int64_t)(r + 8 * u) * o.cols) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const uint32_t h = (uint32_t)__double2hiint(v[u]) & 0x7FFFFFFFu;
          mx = max(mx, h);
          nz |= h | (uint32_t)__double2loint(v[u]);
        }
      }
    }
    smx[g][lane] = mx;
    snz[g][lane] = nz;
    __syncthreads();
    if (threadIdx.x < kTN) {
      uint32_t m = 0, z = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        m = max(m, smx[q][threadIdx.x]);
        z |= snz[q][threadIdx.x];
      }
      const int f = z ? max(1, (int)(m >> 20)) : 0;
      se[threadIdx.x] = exp_of_field(f);
      if ((int)threadIdx.x < nc) exps[o.exp_off + c0 + threadIdx.x] = f;
    }
    __syncthreads();
    const int nch = o.ktiles * 256;
    for (int l = threadIdx.x; l < nch; l += blockDim.x) {
      // chunk order inside a (column tile, k tile): ks (4), n_core (4), k_core (2), n8 (8)
      const int kt = l >> 8, w = l & 255;
      const int ks = w >> 6, n_core = (w >> 4) & 3, k_core = (w >> 3) & 1, n8 = w & 7;
      const int cc = n_core * 8 + n8;
      const int64_t k0 = (int64_t)kt * kTK + ks * 16 + k_core * 8;
      if (cc >= nc || k0 >= o.rows) continue;   // padding: the buffer was zeroed once
      const int e = se[cc];
      const double* col = blk + c0 + cc;
      uint64_t y[8];
      uint32_t sg[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        double x = 0.0;
        if (k0 + j < o.rows) {
          if constexpr (CPLX) x = b_elem<true>(blk, k0 + j, c0 + cc, o.cols);
          else x = col[(k0 + j) * o.cols];
        }
        y[j] = scaled_y(x, e, sg[j]);
      }
      // tile layout [ks][slice][n_core][k_core][8 columns x 16 B]: the 7 slices of a 16-wide k
      // step form one 224-row K-major operand (slice q = rows 32 (q-1) .. 32 q - 1)
      const int64_t tile = (int64_t)tt.y * o.ktiles + kt;
      store_planes(y, sg, pack + o.pack_off + tile * (int64_t)(kS * kBTile) + (int64_t)ks * (kS * 1024) + n_core * 256 +
                              k_core * 128 + n8 * 16, 1024);
    }
    __syncthreads();   // smx / se are rewritten by the next column tile
  }
}

// ------------------------------------------------------------------ tcgen05 helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  // start >> 4 | LBO (128 B) >> 4 << 16 | SBO (256 B) >> 4 << 32 | fixed 0b001 << 46; no swizzle
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);
}

// Bounded waits spin for about 1 s of SM clock (2^31 cycles at the 2.07 GHz maximum),
// checking the clock every 256 polls so the fast path is a bare try_wait.
constexpr long long kWaitCycles = 1ll << 31;

// Operand pipeline: a stage holds one 32-wide k slab of all 7 A slices (56 KB) and all 7 B
// slices (14 KB), each as it lies in the packed tile ([16-wide k step][slice][...]); 3
// stages = 210 KB of shared memory. Per 16-wide k step the A slices are 4 KB apart and the
// B slices form one 224-row operand.
constexpr int kStages = 3;
constexpr int kKS = 32;                         // k per stage (2 MMA k-steps)
constexpr int kAStep = kS * kTM * 16 * 2;       // 28 KB: 7 A slices of one k step
constexpr int kBStep = kS * kTN * 16 * 2;       // 7 KB: 7 B slices of one k step
constexpr int kABytes = 2 * kAStep, kBBytes = 2 * kBStep;
constexpr int kStageBytes = kABytes + kBBytes;  // 70 KB
constexpr int kSmemBytes = kStages * kStageBytes + 1024;
constexpr int kPeriod = kDrainK / kKS;          // stages between drains (4)
constexpr int kDrainWarps = 16;                 // four per tensor-memory lane quadrant
constexpr int kDrainCols = kTN / 4;             // columns per drain thread
constexpr int kRoleThreads = 64 + 32 * kDrainWarps;   // warp 0 producer, warp 1 MMA, warps 2-17 drain
// Tensor memory: two accumulator sets, each 7 levels x 32 columns (level L at 32 (L - 2)).
constexpr int kAccCols = kLevels * kTN;         // 224
// Then the tile's running FP64 sum over its tasks: 32 doubles per lane as 64 32-bit columns.
constexpr int kSumCol = 2 * kAccCols;           // 448
constexpr uint32_t kTmemAlloc = 512;
static_assert(kSumCol + 2 * kTN <= (int)kTmemAlloc, "tensor memory budget");
constexpr int kFlushDrains = 32;                // the int64 sum of a chunk stays below 2^63
constexpr float kMagic = 12582912.0f;           // 1.5 * 2^23: x + kMagic has the integer x in its low bits
constexpr int kMagicBits = 0x4B400000;          // for |x| < 2^22

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
// One lane of the calling warp (the same one every time for a full warp).
__device__ __forceinline__ bool elect_one() {
  uint32_t pred = 0;
  asm volatile("{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\tselp.u32 %0, 1, 0, p;\n\t}\n" : "=r"(pred));
  return pred != 0;
}
// The tensor-core helpers below are called by a whole warp; the elected lane issues.
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  if (elect_one())
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}
// The same, issued by the calling thread alone (the caller elects it).
__device__ __forceinline__ void tc_commit_issue(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}
__device__ __forceinline__ void mma_bf16_issue(uint32_t d, uint64_t da, uint64_t db, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(da), "l"(db), "r"(id), "r"(acc));
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

// 16 lanes x 256 bits: thread t gets 32-bit columns 2 (t % 4) and 2 (t % 4) + 1 of lanes t / 4
// (r[0], r[1]) and t / 4 + 8 (r[2], r[3]) - one FP64 value of each of two rows
__device__ __forceinline__ void tmem_ld_16x256b(uint32_t taddr, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.16x256b.x1.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]));
}

// Bounded wait that also gives up as soon as another role has aborted.
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t mbar, uint32_t phase, const volatile int* abort_flag,
                                                   long long limit = kWaitCycles) {
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
    if (*abort_flag || clock64() - t0 > limit) return false;
  }
}

// Warp-uniform forms for warps whose lanes run the same loop: the abort flag as lane 0 saw
// it, and a bounded wait that succeeds only if it succeeded in every lane.
__device__ __forceinline__ bool aborted(volatile int* abort_flag) {
  return __shfl_sync(0xffffffffu, *abort_flag, 0) != 0;
}
__device__ __forceinline__ bool wait_warp(uint32_t mbar, uint32_t phase, volatile int* abort_flag) {
  return __all_sync(0xffffffffu, mbar_wait_or_abort(mbar, phase, abort_flag));
}
// Bounded wait that ignores the abort flag: for the copies and tensor-core work a CTA issued
// itself, which must land before it frees or leaves the memory they write.
__device__ __forceinline__ bool wait_warp_own(uint32_t mbar, uint32_t phase) {
  const int never = 0;
  return __all_sync(0xffffffffu, mbar_wait_or_abort(mbar, phase, &never));
}

// The bounded wait itself, checked on the device: one warp waits on an mbarrier nothing
// arrives on, with a limit of `limit` cycles, and reports 1 when the wait gave up (the
// expected outcome) or 0 had it completed. Nothing else runs; the context stays usable.
__global__ void __launch_bounds__(32) k_wait_selftest(long long limit, int* __restrict__ status) {
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  __syncwarp();
  const int never = 0;
  const bool ok = __all_sync(0xffffffffu, mbar_wait_or_abort(smem_u32(&bar), 0, &never, limit));
  if (threadIdx.x == 0) *status = ok ? 0 : 1;
}

// Fold one drained accumulator set into the int64 sums z (units 2^-49) of this thread's
// row and 8 columns. Over 256 k, level L sums (L - 1) slice pairs of 256 products below
// 127^2 each, integers times 2^(-7L): levels 2..5 stay below 2^24 and are exact in FP32;
// levels 6..8 may pass 2^24 and carry an FP32 rounding there, at most 2^-24 of a quantity
// 2^-28 below the leading level (2^-52 of the result: below the 2^-49 slice truncation).
// Level 2 stays below 2^22 and converts with the magic-number add, the others with F2I;
// level 8 is rounded to units of 2^-49.
__device__ __forceinline__ void drain_set(uint32_t lb, long long (&z)[kDrainCols]) {
  // levels are read two at a time, one wait per pair
  uint32_t r[kDrainCols], q[kDrainCols];
  int32_t u[kDrainCols];
  tmem_ld8(lb, r);                                       // level 2
  tmem_ld8(lb + kTN, q);                                 // level 3
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int c = 0; c < kDrainCols; ++c) {
    u[c] = (__float_as_int(fmaf(__uint_as_float(r[c]), 0x1p14f, kMagic)) - kMagicBits) * 128;
    u[c] += __float2int_rn(__uint_as_float(q[c]) * 0x1p21f);
    z[c] += (long long)u[c] << 28;
  }
  tmem_ld8(lb + 2 * kTN, r);                             // level 4
  tmem_ld8(lb + 3 * kTN, q);                             // level 5
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int c = 0; c < kDrainCols; ++c) {
    u[c] = __float2int_rn(__uint_as_float(r[c]) * 0x1p28f) * 128;
    u[c] += __float2int_rn(__uint_as_float(q[c]) * 0x1p35f);
    z[c] += (long long)u[c] << 14;
  }
  tmem_ld8(lb + 4 * kTN, r);                             // level 6 (in int64: it may pass 2^24)
  tmem_ld8(lb + 5 * kTN, q);                             // level 7
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int c = 0; c < kDrainCols; ++c) {
    z[c] += (long long)__float2int_rn(__uint_as_float(r[c]) * 0x1p42f) * 128;
    u[c] = __float2int_rn(__uint_as_float(q[c]) * 0x1p49f);
  }
  tmem_ld8(lb + 6 * kTN, r);                             // level 8
  asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
  for (int c = 0; c < kDrainCols; ++c)
    z[c] += (long long)(u[c] + ((__float2int_rn(__uint_as_float(r[c]) * 0x1p56f) + 64) >> 7));
}

// sum (+)= sign 2^(ea + eb - 49) z, each term rounded once to FP64; the tile's running sum
// of this thread's 8 columns lives in tensor memory at tsum (16 columns). The first
// contribution to a tile sets it, later ones add.
__device__ __forceinline__ void fold_sums(const long long (&z)[kDrainCols], int ea, const int (&eb)[kDrainCols],
                                          bool neg, uint32_t tsum, bool& written) {
  uint32_t v[2 * kDrainCols];
  if (written) {                                   // warp-uniform: later tasks of the tile add
    tmem_ld16(tsum, v);
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int c = 0; c < kDrainCols; ++c) {
      const double x = scaled_i64(z[c], ea + eb[c] - 49, neg) + __hiloint2double((int)v[2 * c + 1], (int)v[2 * c]);
      v[2 * c] = (uint32_t)__double2loint(x);
      v[2 * c + 1] = (uint32_t)__double2hiint(x);
    }
  } else {
#pragma unroll
    for (int c = 0; c < kDrainCols; ++c) {
      const double x = scaled_i64(z[c], ea + eb[c] - 49, neg);
      v[2 * c] = (uint32_t)__double2loint(x);
      v[2 * c + 1] = (uint32_t)__double2hiint(x);
    }
  }
  tmem_st16(tsum, v);
  asm volatile("tcgen05.wait::st.sync.aligned;");
  written = true;
}

// Warp-specialised split GEMM. All roles walk the same static sequence of work items
// (output tiles ti = blockIdx.x, blockIdx.x + gridDim.x, ...; for each its tasks; for each
// task its 32-wide k stages), so they agree on stage, period and buffer numbers without
// talking:
//  * warp 0 fills shared-memory stage g % 3 with two bulk copies once the MMAs of stage
//    g - 3 released it;
//  * warp 1 issues, per 16-wide k step, 7 MMAs into accumulator set (period d) % 2 once
//    the drain warps released it: MMA p multiplies A slice p by B slices 1..8-p
//    concatenated along N (N = 32 (8 - p)) into the levels p+1..8, i.e. accumulator
//    columns 32 (p - 1) .. 223, so every slice pair with p + q <= 8 lands on its level
//    with no padding and the tensor core sees few wide instructions instead of 28 narrow
//    ones;
//  * warps 2-17 (four per tensor-memory lane quadrant, 8 columns each) read a set after its
//    MMAs completed, fold it into int64 sums and release it; after a task's last period
//    (or every 64 periods) they write the contribution to C.
// Warps 0 and 1 run their loops as whole warps (warp-uniform state and descriptors); one
// elected lane issues each copy / tensor-core instruction.
__global__ void __launch_bounds__(kRoleThreads, 1)
    k_gemm_split(const SplitWork* __restrict__ items, const int32_t* __restrict__ item_off,
                 const uint8_t* __restrict__ apack, const uint8_t* __restrict__ bpack,
                 const int32_t* __restrict__ aexp, const int32_t* __restrict__ bexp,
                 const int64_t* __restrict__ row_map, double* __restrict__ C, int* __restrict__ err) {
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
    for (int b = 0; b < 2; ++b) { mbar_init(smem_u32(&accf_bar[b]), 1); mbar_init(smem_u32(&acce_bar[b]), kDrainWarps); }
    mbar_init(smem_u32(&fin_bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_abort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint32_t sbase = smem_u32(smem);
  const int beg = item_off[blockIdx.x], end = item_off[blockIdx.x + 1];
  auto fail = [&]() {
    s_abort = 1;
    atomicExch(err, 1);
  };

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    uint32_t g = 0;
    SplitWork nx;
    if (beg < end) nx = items[beg];
    for (int it = beg; it < end && !aborted(&s_abort); ++it) {
      const SplitWork w = nx;
      if (it + 1 < end) nx = items[it + 1];            // prefetch the next step
      const int nst = (w.k + kKS - 1) / kKS;
      bool ok = true;
      for (int j = 0; j < nst; ++j, ++g) {
        const int s = g % kStages;
        if (g >= (uint32_t)kStages && !wait_warp(smem_u32(&empty_bar[s]), ((g / kStages) - 1) & 1, &s_abort)) {
          if (lane == 0) fail();
          ok = false;
          break;
        }
        const int kt = j >> 1, half = j & 1;
        const uint8_t* ga = apack + w.a_pack + ((int64_t)w.tm * w.ktiles + kt) * (kS * kATile) + half * kABytes;
        const uint8_t* gb = bpack + w.b_pack + ((int64_t)w.tn * w.ktiles + kt) * (kS * kBTile) + half * kBBytes;
        const uint32_t sa = sbase + s * kStageBytes;
        const uint32_t fb = smem_u32(&full_bar[s]);
        if (elect_one()) {
          mbar_expect_tx(fb, kStageBytes);
          bulk_g2s(sa, ga, kABytes, fb);
          bulk_g2s(sa + kABytes, gb, kBBytes, fb);
        }
        __syncwarp();
      }
      if (!ok) break;
    }
    // copies still in flight are waited for by the MMA warp (every issued stage is consumed
    // on the normal path); on abort wait for the tail of issued stages here
    if (aborted(&s_abort)) {
      for (uint32_t x = (g > (uint32_t)kStages ? g - kStages : 0); x < g; ++x)
        wait_warp_own(smem_u32(&full_bar[x % kStages]), (x / kStages) & 1);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ tensor-core issuer
    // descriptor of stage 0 at byte 0; every operand is a fixed byte offset from it
    const uint64_t sd0 = smem_desc(sbase);
    uint32_t g = 0, d = 0;
    bool ok = true;
    int nst_next = beg < end ? items[beg].k : 0;
    for (int it = beg; it < end && ok && !aborted(&s_abort); ++it) {
      const int nst = (nst_next + kKS - 1) / kKS;
      if (it + 1 < end) nst_next = items[it + 1].k;   // prefetch the next step
      {
        for (int j = 0; j < nst; ++j, ++g) {
          const int s = g % kStages;
          const int buf = d & 1;
          const bool first = (j % kPeriod) == 0;
          const bool drain = (j % kPeriod) == kPeriod - 1 || j + 1 == nst;
          if (first && d >= 2 && !wait_warp(smem_u32(&acce_bar[buf]), ((d / 2) - 1) & 1, &s_abort)) {
            ok = false;
            break;
          }
          if (!wait_warp(smem_u32(&full_bar[s]), (g / kStages) & 1, &s_abort)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t soff = (uint64_t)((s * kStageBytes) >> 4);
          const uint32_t dbuf = tmem + (uint32_t)(buf * kAccCols);
          // one elected lane issues the stage's 14 MMAs and its commits: the warp shares its
          // scheduler with four busy drain warps, so the fewer instructions between two MMAs,
          // the less the tensor pipe waits for the next one
          if (elect_one()) {
#pragma unroll
            for (int ks = 0; ks < kKS / 16; ++ks) {
              const uint64_t bdesc = sd0 + soff + (uint64_t)((kABytes + ks * kBStep) >> 4);
#pragma unroll
              for (int p = 1; p <= kS; ++p) {
                const uint64_t adesc = sd0 + soff + (uint64_t)((ks * kAStep + (p - 1) * kTM * 32) >> 4);
                // the first MMA of a period (p = 1, all 224 columns) overwrites the set
                const uint32_t acc = (first && ks == 0 && p == 1) ? 0u : 1u;
                mma_bf16_issue(dbuf + (uint32_t)((p - 1) * kTN), adesc, bdesc, idesc_bf16(kTN * (kS + 1 - p)), acc);
              }
            }
            tc_commit_issue(smem_u32(&empty_bar[s]));
            if (drain) tc_commit_issue(smem_u32(&accf_bar[buf]));
          }
          __syncwarp();
          if (drain) ++d;
        }
      }
    }
    if (!ok && lane == 0) fail();
    // all tensor-core work issued by this warp completes before the memory is released
    tc_commit(smem_u32(&fin_bar));
    wait_warp_own(smem_u32(&fin_bar), 0);
  } else if (warp >= 2) {
    // ------------------------------------------------------------ drain / epilogue
    const int quad = warp & 3;                       // tensor-memory lanes 32 * quad .. + 31
    const int cpart = (warp - 2) >> 2;               // columns 8 * cpart .. + 7 of the tile
    const int row_in_tile = quad * 32 + lane;
    uint32_t d = 0;
    bool stop = false, written = false;
    // outputs of the tile that a non-finite operand row or column reaches (bit c: column c);
    // they are stored as NaN (FP64 gives NaN or an infinity there; the slices cannot carry it)
    uint32_t poison = 0;
    const uint32_t tsum = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(kSumCol + 2 * cpart * kDrainCols);
    for (int it = beg; it < end && !stop && !aborted(&s_abort); ++it) {
      const SplitWork w = items[it];
      const int row = w.tm * kTM + row_in_tile;
      const int col0 = w.tn * kTN + cpart * kDrainCols;
      const int nst = (w.k + kKS - 1) / kKS;
      if (w.flags & 1) {
        written = false;
        poison = 0;
      }
      // this row's place in C, fetched early for the tile's store
      const long long rmap = (w.flags & 2) && row < w.m ? __ldg(row_map + w.row_map + row) : -1ll;
      // scale exponents, fetched while the first period is still on the tensor cores
      const int fa = row < w.m ? aexp[w.a_exp + row] : 0;
      const int ea = exp_of_field(fa);
      if (fa == 2047) poison = (1u << kDrainCols) - 1;
      int eb[kDrainCols];
#pragma unroll
      for (int c = 0; c < kDrainCols; ++c) {
        const int fb = col0 + c < w.n ? bexp[w.b_exp + col0 + c] : 0;
        eb[c] = exp_of_field(fb);
        if (fb == 2047) poison |= 1u << c;
      }
      long long z[kDrainCols];
      // the task's periods in chunks of kFlushDrains, each folded on its own, so the int64
      // sums stay in range for any k
      for (int j0 = 0; j0 < nst && !stop; j0 += kFlushDrains * kPeriod) {
        const int j1 = min(nst, j0 + kFlushDrains * kPeriod);
#pragma unroll
        for (int c = 0; c < kDrainCols; ++c) z[c] = 0;
        for (int j = j0; j < j1; ++j) {
          const bool drain = (j % kPeriod) == kPeriod - 1 || j + 1 == nst;
          if (!drain) continue;
          const int buf = d & 1;
          if (!wait_warp(smem_u32(&accf_bar[buf]), (d / 2) & 1, &s_abort)) {
            if (lane == 0) fail();
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          drain_set(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * kAccCols + cpart * kDrainCols), z);
          asm volatile("tcgen05.fence::before_thread_sync;");
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&acce_bar[buf]));
          ++d;
        }
        if (stop) break;
        fold_sums(z, ea, eb, w.sign < 0, tsum, written);
      }
      // one store per tile after its last task (a C tile belongs to exactly one CTA). The sums
      // are read back in the 16 x 256-bit shape, so that four consecutive lanes hold four
      // consecutive columns of one row and each store instruction writes 32-byte pieces of 8
      // rows (a lane-per-row store would write 32 separate 8-byte pieces). Row places and
      // non-finite masks come from the lane that owns the row.
      if (!stop && (w.flags & 2)) {
        uint32_t v[4 * kDrainCols];
        const uint32_t tb = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(kSumCol + 2 * cpart * kDrainCols);
        tmem_ld_16x256b(tb, v);
        tmem_ld_16x256b(tb + 8u, v + 4);
        tmem_ld_16x256b(tb + (16u << 16), v + 8);
        tmem_ld_16x256b(tb + (16u << 16) + 8u, v + 12);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        const int cq = lane & 3, rq = lane >> 2;
#pragma unroll
        for (int lh = 0; lh < 2; ++lh)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int rl = 16 * lh + 8 * h + rq;       // the row's lane in this warp
            const long long rm = __shfl_sync(0xffffffffu, rmap, rl);
            const uint32_t pz = __shfl_sync(0xffffffffu, poison, rl);
            if (rm >= 0) {
#pragma unroll
              for (int ch = 0; ch < 2; ++ch) {
                const int c = 4 * ch + cq;
                if (col0 + c < w.n) {
                  const uint32_t* x = v + 8 * lh + 4 * ch + 2 * h;
                  C[rm + col0 + c] = (pz >> c) & 1u ? __longlong_as_double(0x7FF8000000000000ll)
                                                    : __hiloint2double((int)x[1], (int)x[0]);
                }
              }
            }
          }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemAlloc));
}


}  // namespace

// ------------------------------------------------------------------ host side
// Row tiles of every stack fit the 16-bit tile index of a work record.
static bool rtiles_fit(const std::vector<int32_t>& m) {
  for (const int32_t x : m)
    if ((x + kTM - 1) / kTM > 32767) return false;
  return true;
}

void SplitPlan::build(const CtrctPlan& p, cudaStream_t s) {
  built = false;
  cfg = p.split_cfg;
  const GemmSchedule& g = p.sched;
  a_ops.clear();
  b_ops.clear();
  tasks.clear();
  tiles.clear();
  stack_task0.clear();
  stack_m.clear();
  stack_n.clear();
  stack_rowmap.clear();
  stack_cblk0.clear();
  row_map.clear();
  auto a_index = [&](int64_t a_off) {   // block ordinal from its offset
    return (int64_t)(std::lower_bound(p.a.offsets.begin(), p.a.offsets.end(), a_off) - p.a.offsets.begin());
  };
  auto b_index = [&](int64_t b_off) {
    return (int64_t)(std::lower_bound(p.b.offsets.begin(), p.b.offsets.end(), b_off) - p.b.offsets.begin());
  };
  // complex operands as real ones: A (m x k complex) is the real m x 2k matrix of its
  // interleaved parts, C likewise m x 2n, and B becomes the real 2k x 2n matrix of 2 x 2
  // blocks [[Re, Im], [-Im, Re]] (built by the B slicing kernel), so C' = A' B'
  const int cw = p.a.dtype == QLTG_C128 ? 2 : 1;
  auto real_off = [cw](int64_t off) { return ((off & ~kFromSrc) * cw) | (off & kFromSrc); };

  // ---- stacks: output blocks with the same n and the same (B block, k, sign) task sequence.
  // Within a stack, the A blocks of task position t form one stacked operand (rows in the
  // stack's block order). An A block can sit in one stacked operand only (its slices are
  // packed once), so a stack whose A blocks would also be stacked differently elsewhere is
  // split back into single blocks, until every A block has one place.
  std::vector<int32_t> cand;
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q)
    if (!skinny_cblk(g, q)) cand.push_back(q);
  std::vector<std::vector<int32_t>> stacks;
  if (cfg.stack) {
    std::map<std::vector<int64_t>, int32_t> key_of;
    for (const int32_t q : cand) {
      const GemmCBlk& cb = g.cblk[q];
      std::vector<int64_t> key{cb.n};
      for (int32_t t = cb.t0; t < cb.t1; ++t) {
        key.push_back(b_index(g.task[t].b_off & ~kFromSrc));
        key.push_back(g.task[t].k);
        key.push_back(g.task[t].sign);
      }
      auto it = key_of.find(key);
      if (it == key_of.end()) {
        key_of.emplace(std::move(key), (int32_t)stacks.size());
        stacks.push_back({q});
      } else {
        stacks[it->second].push_back(q);
      }
    }
    // cap the rows of one stack (greedy in block order; equal keys split identically)
    std::vector<std::vector<int32_t>> capped;
    for (auto& st : stacks) {
      std::vector<int32_t> cur;
      int64_t rows = 0;
      for (const int32_t q : st) {
        if (!cur.empty() && rows + g.cblk[q].m > cfg.max_stack_rows) {
          capped.push_back(cur);
          cur.clear();
          rows = 0;
        }
        cur.push_back(q);
        rows += g.cblk[q].m;
      }
      if (!cur.empty()) capped.push_back(cur);
    }
    stacks.swap(capped);
    // demote stacks whose A blocks have more than one stacked place, to a fixed point
    for (bool changed = true; changed;) {
      changed = false;
      std::map<int64_t, std::vector<int64_t>> place;   // A block -> its stacked operand (A blocks)
      std::vector<uint8_t> bad(stacks.size(), 0);
      std::map<int64_t, std::vector<int32_t>> users;   // A block -> stacks using it
      for (int32_t si = 0; si < (int32_t)stacks.size(); ++si) {
        const auto& st = stacks[si];
        const int32_t nt = g.cblk[st[0]].t1 - g.cblk[st[0]].t0;
        for (int32_t pos = 0; pos < nt; ++pos) {
          std::vector<int64_t> tuple;
          for (const int32_t q : st) tuple.push_back(a_index(g.task[g.cblk[q].t0 + pos].a_off & ~kFromSrc));
          for (const int64_t ia : tuple) {
            users[ia].push_back(si);
            auto it = place.find(ia);
            if (it == place.end()) place.emplace(ia, tuple);
            else if (it->second != tuple) bad[si] = 1;
          }
        }
      }
      // a conflict marks every stack that uses a conflicting block
      for (auto& [ia, tuple] : place) {
        bool conflict = false;
        for (const int32_t si : users[ia]) conflict |= bad[si] != 0;
        if (conflict)
          for (const int32_t si : users[ia]) bad[si] = 1;
      }
      std::vector<std::vector<int32_t>> next;
      for (int32_t si = 0; si < (int32_t)stacks.size(); ++si) {
        if (bad[si] && stacks[si].size() > 1) {
          changed = true;
          for (const int32_t q : stacks[si]) next.push_back({q});
        } else {
          next.push_back(stacks[si]);
        }
      }
      stacks.swap(next);
    }
  } else {
    for (const int32_t q : cand) stacks.push_back({q});
  }

  // ---- stacked A operands (one per distinct tuple of A blocks), B operands per block
  int64_t a_pack = 0, b_pack = 0, a_exp = 0, b_exp = 0, a_chunks = 0, a_pchunks = 0;
  std::map<std::vector<int64_t>, std::pair<int64_t, int32_t>> stacked_op;   // tuple -> (pack, exp)
  std::vector<int32_t> b_of(p.b.nblk, -1);
  tile_stages = 0;
  double useful = 0.0;
  for (const auto& st : stacks) {
    const GemmCBlk& c0 = g.cblk[st[0]];
    const int32_t nt = c0.t1 - c0.t0;
    int64_t m = 0;
    for (const int32_t q : st) m += g.cblk[q].m;
    QLTG_CHECK(m < ((int64_t)1 << 22), QLTG_ERR_UNSUPPORTED, "stacked output too tall");
    const int cn = cw * c0.n;
    stack_cblk0.push_back(st[0]);
    stack_task0.push_back((int32_t)tasks.size());
    stack_m.push_back((int32_t)m);
    stack_n.push_back(cn);
    stack_rowmap.push_back((int32_t)row_map.size());
    QLTG_CHECK(row_map.size() + (size_t)m < ((size_t)1 << 31), QLTG_ERR_UNSUPPORTED, "too many stacked rows");
    for (const int32_t q : st) {
      const GemmCBlk& cb = g.cblk[q];
      for (int32_t r = 0; r < cb.m; ++r) row_map.push_back(cw * cb.c_off + (int64_t)r * cn);
    }
    const int64_t rtiles = (m + kTM - 1) / kTM, ctiles = (cn + kTN - 1) / kTN;
    for (int32_t pos = 0; pos < nt; ++pos) {
      const GemmTask& gt0 = g.task[c0.t0 + pos];
      const int k = cw * gt0.k;
      const int ktiles = (k + kTK - 1) / kTK;
      std::vector<int64_t> tuple;
      for (const int32_t q : st) tuple.push_back(a_index(g.task[g.cblk[q].t0 + pos].a_off & ~kFromSrc));
      auto it = stacked_op.find(tuple);
      if (it == stacked_op.end()) {
        const std::pair<int64_t, int32_t> where{a_pack, (int32_t)a_exp};
        int32_t row_base = 0;
        for (size_t i = 0; i < st.size(); ++i) {
          const GemmCBlk& cb = g.cblk[st[i]];
          const GemmTask& gt = g.task[cb.t0 + pos];
          QLTG_CHECK((int64_t)cb.m * k < ((int64_t)1 << 31) - 8, QLTG_ERR_UNSUPPORTED, "operand block too large");
          SplitOperand o{};
          o.src_off = real_off(gt.a_off);
          o.rows = cb.m;
          o.cols = k;
          o.ktiles = ktiles;
          o.exp_off = (int32_t)(a_exp + row_base);
          o.pack_off = a_pack;
          o.chunk_begin = a_chunks;
          o.pchunk_begin = a_pchunks;
          o.row_base = row_base;
          a_chunks += ((int64_t)cb.m * k + 7) / 8;
          a_pchunks += (int64_t)cb.m * ((k + 15) / 16);
          row_base += cb.m;
          a_ops.push_back(o);
        }
        a_exp += m;
        a_pack += rtiles * ktiles * kS * (int64_t)kATile;
        it = stacked_op.emplace(tuple, where).first;
      }
      const int64_t ib = b_index(gt0.b_off & ~kFromSrc);
      if (b_of[ib] < 0) {
        SplitOperand o{};
        o.src_off = real_off(gt0.b_off);
        o.rows = k;
        o.cols = cn;
        o.ktiles = ktiles;
        o.exp_off = (int32_t)b_exp;
        o.pack_off = b_pack;
        o.cplx = cw == 2 ? 1 : 0;
        b_exp += cn;
        b_pack += ctiles * ktiles * kS * (int64_t)kBTile;
        b_of[ib] = (int32_t)b_ops.size();
        b_ops.push_back(o);
      }
      const SplitOperand& ob = b_ops[b_of[ib]];
      QLTG_CHECK(ob.rows == k && ob.cols == cn, QLTG_ERR_INVALID, "internal: inconsistent operand shapes in the split schedule");
      tasks.push_back(SplitTask{it->second.first, ob.pack_off, it->second.second, ob.exp_off, ktiles, gt0.sign});
      tile_stages += rtiles * ctiles * ((k + kKS - 1) / kKS);
      useful += (double)m * cn * k;
    }
    for (int64_t i = 0; i < rtiles; ++i)
      for (int64_t j = 0; j < ctiles; ++j)
        tiles.push_back(GemmTile{(int32_t)(stack_m.size() - 1), (int16_t)i, (int16_t)j});
  }
  useful_frac = tile_stages ? useful / ((double)tile_stages * kTM * kTN * kKS) : 0.0;
  QLTG_CHECK(tiles.size() < ((size_t)1 << 31), QLTG_ERR_UNSUPPORTED, "too many split tiles");
  QLTG_CHECK(rtiles_fit(stack_m), QLTG_ERR_UNSUPPORTED, "stacked output has too many row tiles");
  // Per-CTA work lists by longest processing time first: tiles in decreasing cost, each to
  // the CTA with the least work so far. Cost of a tile: 2 per 32-wide k stage plus 1 per
  // task (the drain and rounding that end a task).
  const int32_t nstacks = (int32_t)stack_m.size();
  std::vector<int64_t> cost(nstacks, 0);
  for (int32_t si = 0; si < nstacks; ++si) {
    const GemmCBlk& c0 = g.cblk[stack_cblk0[si]];
    for (int32_t t = c0.t0; t < c0.t1; ++t) cost[si] += 2 * ((cw * g.task[t].k + 31) / 32) + 1;
  }
  std::stable_sort(tiles.begin(), tiles.end(), [&](const GemmTile& x, const GemmTile& y) { return cost[x.cblk] > cost[y.cblk]; });
  grid = (int)std::min<int64_t>((int64_t)tiles.size(), std::max(1, p.ctx->num_sms));
  std::vector<std::vector<int32_t>> owned(grid);
  {
    using Load = std::pair<int64_t, int>;   // (work so far, CTA)
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int b = 0; b < grid; ++b) heap.push({0, b});
    for (size_t ti = 0; ti < tiles.size(); ++ti) {
      Load l = heap.top();
      heap.pop();
      owned[l.second].push_back((int32_t)ti);
      l.first += cost[tiles[ti].cblk];
      heap.push(l);
    }
  }
  // Each CTA's tiles alternate long and short (its list is in decreasing cost): a short
  // tile's drain, fold and store then overlap a long tile's MMAs instead of the short tiles
  // all coming last, where the drain warps would set the pace.
  for (auto& v : owned) {
    std::vector<int32_t> mixed;
    mixed.reserve(v.size());
    for (size_t i = 0, j = v.size(); i < j;) {
      mixed.push_back(v[i++]);
      if (i < j) mixed.push_back(v[--j]);
    }
    v.swap(mixed);
  }
  work.clear();
  work_off.assign(grid + 1, 0);
  for (int b = 0; b < grid; ++b) {
    work_off[b] = (int32_t)work.size();
    for (const int32_t ti : owned[b]) {
      const GemmTile& tl = tiles[ti];
      const int32_t si = tl.cblk;
      const GemmCBlk& c0 = g.cblk[stack_cblk0[si]];
      const int32_t nt = c0.t1 - c0.t0;
      for (int32_t pos = 0; pos < nt; ++pos) {
        const SplitTask& tk = tasks[stack_task0[si] + pos];
        SplitWork w{};
        w.c_off = cw * c0.c_off;
        w.a_pack = tk.a_pack;
        w.b_pack = tk.b_pack;
        w.m = stack_m[si];
        w.n = stack_n[si];
        w.a_exp = tk.a_exp;
        w.b_exp = tk.b_exp;
        w.ktiles = tk.ktiles;
        w.k = cw * g.task[c0.t0 + pos].k;
        w.tm = tl.tm;
        w.tn = tl.tn;
        w.sign = (int8_t)(tk.sign < 0 ? -1 : 1);
        w.flags = (uint8_t)((pos == 0 ? 1 : 0) | (pos + 1 == nt ? 2 : 0));
        w.row_map = stack_rowmap[si];
        work.push_back(w);
      }
    }
    QLTG_CHECK(work.size() < ((size_t)1 << 31), QLTG_ERR_UNSUPPORTED, "too many split work items");
  }
  work_off[grid] = (int32_t)work.size();
  b_col_tiles.clear();
  for (int i = 0; i < (int)b_ops.size(); ++i)
    for (int ct = 0; ct * kTN < b_ops[i].cols; ++ct) b_col_tiles.push_back(make_int2(i, ct));
  d_b_col_tiles = upload(b_col_tiles, s);
  n_a_chunks = a_chunks;
  n_a_pchunks = a_pchunks;
  // long rows (the matvec's t2 . renv: k up to 528) are folded one warp per row; short ones
  // by 8-element chunks with atomics
  row_warp = a_exp > 0 && a_chunks * 8 >= (int64_t)32 * a_exp;
  {
    int per_sm = 0;
    if (row_warp) {
      QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_row_field_rows, 256, 0));
      row_exp_grid = (int)std::max<int64_t>(1, std::min<int64_t>((a_exp + 7) / 8,
                                                                 (int64_t)std::max(1, per_sm) * p.ctx->num_sms));
    } else {
      QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_row_field, 256, 0));
      row_exp_grid = (int)std::max<int64_t>(1, std::min<int64_t>((n_a_chunks + 255) / 256,
                                                                 (int64_t)std::max(1, per_sm) * p.ctx->num_sms));
    }
    QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pack_a, 256, 0));
    pack_a_grid = (int)std::max<int64_t>(1, std::min<int64_t>((n_a_pchunks + 255) / 256,
                                                              (int64_t)std::max(1, per_sm) * p.ctx->num_sms));
    if (p.a.dtype == QLTG_C128)
      QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pack_b_cols<true>, 256, 0));
    else
      QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pack_b_cols<false>, 256, 0));
    pack_b_grid = std::max(1, std::min((int)b_col_tiles.size(), std::max(1, per_sm) * p.ctx->num_sms));
  }
  d_a_ops = upload(a_ops, s);
  d_b_ops = upload(b_ops, s);
  d_work = upload(work, s);
  d_work_off = upload(work_off, s);
  d_row_map = upload(row_map, s);
  a_packed.alloc(std::max<int64_t>(a_pack, 16));
  b_packed.alloc(std::max<int64_t>(b_pack, 16));
  // tile padding (rows or columns past the block, k past the task) stays zero: the pack
  // kernels only write the chunks that hold operand data
  QLTG_CUDA(cudaMemsetAsync(a_packed.get(), 0, std::max<int64_t>(a_pack, 16), s));
  QLTG_CUDA(cudaMemsetAsync(b_packed.get(), 0, std::max<int64_t>(b_pack, 16), s));
  n_a_rows = a_exp;
  a_exps.alloc(std::max<int64_t>(a_exp, 1) * 4);
  b_exps.alloc(std::max<int64_t>(b_exp, 1) * 4);
  error.alloc(sizeof(int));
  QLTG_CUDA(cudaMemsetAsync(error.get(), 0, sizeof(int), s));
  // per device (the attribute belongs to the current device's copy of the kernel)
  QLTG_CUDA(cudaFuncSetAttribute(k_gemm_split, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
  if (!g.skinny.empty() && !tiles.empty() && !side) {
    QLTG_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    QLTG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    QLTG_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
  built = true;
}

int64_t SplitPlan::launches() const {
  if (tiles.empty()) return 0;
  // A: (memset,) row scales, pack; B: pack; GEMM
  return (a_static ? 0 : (a_fields_external ? 1 : (row_warp ? 2 : 3))) + (b_static ? 0 : 1) + 1;
}

// Scale exponents and slice tiles of one operand side (A: rows, B: columns), reading each
// operand block from the scratch or, flagged kFromSrc, from the source.
void pack_split_operand(SplitPlan& sp, bool side_a, const void* scratch, const void* source, cudaStream_t s) {
  const double* X = static_cast<const double*>(scratch);
  const double* Xs = static_cast<const double*>(source);
  if (side_a) {
    if (sp.a_ops.empty()) {
      sp.a_ready = true;
      return;
    }
    if (sp.a_fields_external) {
      // the row scales were folded by the kernel that wrote this operand
    } else if (sp.row_warp) {
      k_row_field_rows<<<sp.row_exp_grid, 256, 0, s>>>(X, Xs, sp.d_a_ops.as<SplitOperand>(), (int)sp.a_ops.size(),
                                                       sp.n_a_rows, sp.a_exps.as<int32_t>());
    } else {
      QLTG_CUDA(cudaMemsetAsync(sp.a_exps.get(), 0, sp.n_a_rows * sizeof(int32_t), s));
      k_row_field<<<sp.row_exp_grid, 256, 0, s>>>(X, Xs, sp.d_a_ops.as<SplitOperand>(), (int)sp.a_ops.size(),
                                                  sp.n_a_chunks, sp.a_exps.as<int32_t>());
    }
    k_pack_a<<<sp.pack_a_grid, 256, 0, s>>>(X, Xs, sp.d_a_ops.as<SplitOperand>(), (int)sp.a_ops.size(),
                                            sp.n_a_pchunks, sp.a_exps.as<int32_t>(), sp.a_packed.as<uint8_t>());
  } else {
    if (sp.b_ops.empty()) {
      sp.b_ready = true;
      return;
    }
    const int nt = (int)sp.b_col_tiles.size();
    if (sp.b_ops[0].cplx)
      k_pack_b_cols<true><<<sp.pack_b_grid, 256, 0, s>>>(X, Xs, sp.d_b_ops.as<SplitOperand>(),
                                                         sp.d_b_col_tiles.as<int2>(), nt, sp.b_exps.as<int32_t>(),
                                                         sp.b_packed.as<uint8_t>());
    else
      k_pack_b_cols<false><<<sp.pack_b_grid, 256, 0, s>>>(X, Xs, sp.d_b_ops.as<SplitOperand>(),
                                                          sp.d_b_col_tiles.as<int2>(), nt, sp.b_exps.as<int32_t>(),
                                                          sp.b_packed.as<uint8_t>());
  }
  QLTG_CUDA(cudaGetLastError());
  (side_a ? sp.a_ready : sp.b_ready) = true;
}

void split_prepack_static(CtrctPlan& p, const void* a_static, const void* b_static, cudaStream_t s) {
  if (!p.split || !p.split->built) return;
  const int eb = (int)p.a.elem_bytes();
  if (a_static) {
    const void* scr = a_static;
    if (p.a_tl.ntiles) { p.a_tl.launch(a_static, p.a_t.get(), eb, s); scr = p.a_t.get(); }
    p.split->a_static = true;
    pack_split_operand(*p.split, true, scr, a_static, s);
  }
  if (b_static) {
    const void* scr = b_static;
    if (p.b_tl.ntiles) { p.b_tl.launch(b_static, p.b_t.get(), eb, s); scr = p.b_t.get(); }
    p.split->b_static = true;
    pack_split_operand(*p.split, false, scr, b_static, s);
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
}

void launch_gemm_split(CtrctPlan& p, const Operands& op, void* c, cudaStream_t s, bool pack) {
  const bool cplx = p.a.dtype == QLTG_C128;
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
  // pad them 8x, and exact integer emulation of these rows measured slower than the FP64
  // pipe); everything else goes through the slices. With both present the skinny kernel
  // runs on the side stream (it writes other output blocks) and joins after the split GEMM.
  const bool fork = !p.sched.skinny.empty() && !sp.tiles.empty() && sp.side;
  const SkinnyFuse* fuse = p.fuse_fields ? p.d_fuse.as<SkinnyFuse>() : nullptr;
  if (fork) {
    QLTG_CUDA(cudaEventRecord(sp.fork, s));
    QLTG_CUDA(cudaStreamWaitEvent(sp.side, sp.fork, 0));
    launch_gemm_f64_skinny(p.sched, op, c, cplx, p.ctx->num_sms, sp.side, fuse, p.fuse_fields);
    QLTG_CUDA(cudaEventRecord(sp.join, sp.side));
  } else {
    launch_gemm_f64_skinny(p.sched, op, c, cplx, p.ctx->num_sms, s, fuse, p.fuse_fields);
  }
  if (sp.tiles.empty()) return;
  struct Join {   // the main stream waits for the side stream on every way out
    bool on;
    SplitPlan& sp;
    cudaStream_t s;
    ~Join() {
      if (on) cudaStreamWaitEvent(s, sp.join, 0);
    }
  } join{fork, sp, s};
  if (pack) {
    if (!(sp.a_static && sp.a_ready)) pack_split_operand(sp, true, op.a, op.a_src, s);
    if (!(sp.b_static && sp.b_ready)) pack_split_operand(sp, false, op.b, op.b_src, s);
  } else {
    QLTG_CHECK(sp.a_ready && sp.b_ready, QLTG_ERR_INVALID, "GEMM-only stage before the operands were ever packed");
  }
  k_gemm_split<<<sp.grid, kRoleThreads, kSmemBytes, s>>>(
      sp.d_work.as<SplitWork>(), sp.d_work_off.as<int32_t>(), sp.a_packed.as<uint8_t>(), sp.b_packed.as<uint8_t>(),
      sp.a_exps.as<int32_t>(), sp.b_exps.as<int32_t>(), sp.d_row_map.as<int64_t>(),
      static_cast<double*>(c), sp.error.as<int>());
  QLTG_CUDA(cudaGetLastError());
}

void prepare_split(CtrctPlan& p, cudaStream_t s) {
  if (p.split && p.split->built) return;
  p.split = std::make_unique<SplitPlan>();
  p.split->build(p, s);
}

int64_t split_launches(const CtrctPlan& p) {
  int64_t n = p.sched.skinny.empty() ? 0 : 1;
  if (p.split) n += p.split->launches();
  return n;
}

int wait_selftest(int64_t limit_cycles, cudaStream_t s) {
  DevBuf st;
  st.alloc(sizeof(int));
  QLTG_CUDA(cudaMemsetAsync(st.get(), 0xFF, sizeof(int), s));
  k_wait_selftest<<<1, 32, 0, s>>>((long long)limit_cycles, st.as<int>());
  QLTG_CUDA(cudaGetLastError());
  int v = -1;
  QLTG_CUDA(cudaMemcpyAsync(&v, st.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  QLTG_CUDA(cudaStreamSynchronize(s));
  return v;
}

int split_device_error(const CtrctPlan& p, cudaStream_t s) {
  if (!p.split || !p.split->built) return 0;
  int e = 0;
  QLTG_CUDA(cudaMemcpyAsync(&e, p.split->error.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  QLTG_CUDA(cudaStreamSynchronize(s));
  return e;
}

}  // namespace qltg
