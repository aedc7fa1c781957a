// Grouped FP64 / complex128 GEMM over all tasks of one contraction.
//
// Replaces the reference's serial loop of one cblas_dgemm / cublasDgemm per task with
// beta = 0 for the first task of an output block and beta = 1 after it
// (global_operations.h:895-992 -> raw_data_operations.h:530-548 -> blas_level3.h:35-56,
// :797-856). Every output tile is owned by one CTA that loops over all tasks of its output
// block, accumulating sign_t * A_t[tile rows, :] B_t[:, tile cols] in registers, and stores
// the tile once: no read-modify-write of C, no atomics, deterministic.
//
// Two kernels, chosen per output block when the plan is built:
//  * k_gemm_dfma   - FP64 / complex128 (4 real FMAs per complex FMA) on 32 x 32 output tiles.
//                    On this GPU the FP64 tensor path (mma.sync m8n8k4 f64) runs at the same
//                    rate as DFMA (about 1.05 TFLOP/s each, measured) but pads every block to
//                    8 x 8 x 4 fragments (48 % useful on the matvec's block shapes), so the
//                    predicated DFMA tile is the faster FP64 kernel;
//  * k_gemm_skinny - output blocks with n <= 8 and k <= 8 (the MPO steps of the two-site
//                    matvec: m up to 3e4, k, n <= 3): one thread per output row, operand B
//                    in registers, memory-streaming.
#include <algorithm>

#include "ctrct.h"

namespace qltg {
namespace {

constexpr int NT = 256;

__device__ __forceinline__ void fma_acc(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void fma_acc(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ double zero_of(double) { return 0.0; }
__device__ __forceinline__ double2 zero_of(double2) { return make_double2(0.0, 0.0); }
// Multiply by a +-1 sign without touching the FP64 pipe: flip the IEEE sign bit(s).
__device__ __forceinline__ double flip(double x, unsigned long long m) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)m);
}
__device__ __forceinline__ double2 flip(double2 x, unsigned long long m) { return make_double2(flip(x.x, m), flip(x.y, m)); }
__device__ __forceinline__ unsigned long long sign_mask(int sign) { return sign < 0 ? 0x8000000000000000ull : 0ull; }

constexpr int BM = 32, BN = 32, BK = 32;

// 32 x 32 output tiles (BM = BN = 32): one output tile per work item; 16 x 16 threads, each 2 x 2 outputs at
// (ty + 16 i, tx + 16 j). Operand tiles are staged through shared memory (A transposed so
// a warp reads one broadcast row); outputs outside the block are predicated off so no FP64
// issue slot is spent on padding. Work items are taken longest-first from an atomic
// counter (the plan zeroes it before each launch), so the few very long tiles start first
// and the rest fill in behind them.
template <typename T>
__global__ void __launch_bounds__(NT) k_gemm_dfma32(const GemmCBlk* __restrict__ cblk, const GemmTask* __restrict__ task,
                                                  const GemmTile* __restrict__ tiles, int ntiles,
                                                  const T* __restrict__ A, const T* __restrict__ As,
                                                  const T* __restrict__ B, const T* __restrict__ Bs,
                                                  T* __restrict__ C, int* __restrict__ counter) {
  __shared__ T sA[BK][BM + 1];
  __shared__ T sB[BK][BN];
  __shared__ int s_ti;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  while (true) {
    if (threadIdx.x == 0) s_ti = atomicAdd(counter, 1);
    __syncthreads();
    const int ti = s_ti;
    __syncthreads();
    if (ti >= ntiles) break;
    const GemmTile tl = tiles[ti];
    const GemmCBlk cb = cblk[tl.cblk];
    const int r0 = tl.tm * BM, c0 = tl.tn * BN;
    const int m = cb.m, n = cb.n;
    T acc[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) acc[i][j] = zero_of(T());
    bool rv[2], cv[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) { rv[i] = r0 + ty + 16 * i < m; cv[i] = c0 + tx + 16 * i < n; }
    for (int t = cb.t0; t < cb.t1; ++t) {
      const GemmTask tk = task[t];
      const int k = tk.k;
      const T* a = operand_block(A, As, tk.a_off);
      const T* b = operand_block(B, Bs, tk.b_off);
      const unsigned long long sg = sign_mask(tk.sign);
      for (int k0 = 0; k0 < k; k0 += BK) {
        const int kc = min(BK, k - k0);
#pragma unroll
        for (int e = threadIdx.x; e < BM * BK; e += NT) {
          const int row = e / BK, kk = e % BK;
          T v = zero_of(T());
          if (kk < kc && r0 + row < m) v = flip(a[(int64_t)(r0 + row) * k + k0 + kk], sg);
          sA[kk][row] = v;
        }
#pragma unroll
        for (int e = threadIdx.x; e < BK * BN; e += NT) {
          const int kk = e / BN, col = e % BN;
          T v = zero_of(T());
          if (kk < kc && c0 + col < n) v = b[(int64_t)(k0 + kk) * n + c0 + col];
          sB[kk][col] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kc; ++kk) {
          const T a0 = sA[kk][ty], a1 = sA[kk][ty + 16];
          const T b0 = sB[kk][tx], b1 = sB[kk][tx + 16];
          if (rv[0]) {
            if (cv[0]) fma_acc(acc[0][0], a0, b0);
            if (cv[1]) fma_acc(acc[0][1], a0, b1);
          }
          if (rv[1]) {
            if (cv[0]) fma_acc(acc[1][0], a1, b0);
            if (cv[1]) fma_acc(acc[1][1], a1, b1);
          }
        }
        __syncthreads();
      }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
        if (rv[i] && cv[j]) C[cb.c_off + (int64_t)(r0 + ty + 16 * i) * n + c0 + tx + 16 * j] = acc[i][j];
  }
}

// k depth of one shared-memory stage: 32, or 16 where the two operand tiles would pass the
// 48 KB of static shared memory (complex 64-row tiles).
template <typename T, int BM, int BN>
constexpr int dfma_bk() { return (int)sizeof(T) * 32 * (BM + 1 + BN) <= 48 * 1024 ? 32 : 16; }

// One output tile of BM x BN per work item (BM = 16 TM, BN = 16 TN); 16 x 16 threads, each
// TM x TN outputs at (ty + 16 i, tx + 16 j). Operand tiles are staged through shared memory
// (A transposed so a warp reads one broadcast row); outputs outside the block are predicated
// off so no FP64 issue slot is spent on padding. Work items are taken longest-first from an
// atomic counter (the plan zeroes it before each launch), so the few very long tiles start
// first and the rest fill in behind them. Used for 64 x 32 tiles (TM = 4, TN = 2): the
// taller tile reads each staged operand value for twice the FMAs; the 32 x 32 tile above
// pads less on small blocks. The tuner picks between them per plan.
template <typename T, int TM, int TN>
__global__ void __launch_bounds__(NT, TM * TN <= 4 ? 4 : 2) k_gemm_dfma(const GemmCBlk* __restrict__ cblk, const GemmTask* __restrict__ task,
                                                  const GemmTile* __restrict__ tiles, int ntiles,
                                                  const T* __restrict__ A, const T* __restrict__ As,
                                                  const T* __restrict__ B, const T* __restrict__ Bs,
                                                  T* __restrict__ C, int* __restrict__ counter) {
  constexpr int BM = 16 * TM, BN = 16 * TN, BK = dfma_bk<T, BM, BN>();
  __shared__ T sA[BK][BM + 1];
  __shared__ T sB[BK][BN];
  __shared__ int s_ti;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  while (true) {
    if (threadIdx.x == 0) s_ti = atomicAdd(counter, 1);
    __syncthreads();
    const int ti = s_ti;
    __syncthreads();
    if (ti >= ntiles) break;
    const GemmTile tl = tiles[ti];
    const GemmCBlk cb = cblk[tl.cblk];
    const int r0 = tl.tm * BM, c0 = tl.tn * BN;
    const int m = cb.m, n = cb.n;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = zero_of(T());
    bool rv[TM], cv[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) rv[i] = r0 + ty + 16 * i < m;
#pragma unroll
    for (int j = 0; j < TN; ++j) cv[j] = c0 + tx + 16 * j < n;
    for (int t = cb.t0; t < cb.t1; ++t) {
      const GemmTask tk = task[t];
      const int k = tk.k;
      const T* a = operand_block(A, As, tk.a_off);
      const T* b = operand_block(B, Bs, tk.b_off);
      const unsigned long long sg = sign_mask(tk.sign);
      for (int k0 = 0; k0 < k; k0 += BK) {
        const int kc = min(BK, k - k0);
#pragma unroll
        for (int e = threadIdx.x; e < BM * BK; e += NT) {
          const int row = e / BK, kk = e % BK;
          T v = zero_of(T());
          if (kk < kc && r0 + row < m) v = flip(a[(int64_t)(r0 + row) * k + k0 + kk], sg);
          sA[kk][row] = v;
        }
#pragma unroll
        for (int e = threadIdx.x; e < BK * BN; e += NT) {
          const int kk = e / BN, col = e % BN;
          T v = zero_of(T());
          if (kk < kc && c0 + col < n) v = b[(int64_t)(k0 + kk) * n + c0 + col];
          sB[kk][col] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kc; ++kk) {
          T av[TM], bv[TN];
#pragma unroll
          for (int i = 0; i < TM; ++i) av[i] = sA[kk][ty + 16 * i];
#pragma unroll
          for (int j = 0; j < TN; ++j) bv[j] = sB[kk][tx + 16 * j];
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j)
              if (rv[i] && cv[j]) fma_acc(acc[i][j], av[i], bv[j]);
        }
        __syncthreads();
      }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j)
        if (rv[i] && cv[j]) C[cb.c_off + (int64_t)(r0 + ty + 16 * i) * n + c0 + tx + 16 * j] = acc[i][j];
  }
}

// Skinny output blocks (n <= 8, every task k <= 8): the rows' n outputs in registers,
// instantiated per n so no FP64 slot is spent on absent columns. A work item is 256 rows of
// one block; each of the 128 threads takes rows r and r + 128, both in one pass over the
// tasks when n <= 4 (real): the task records and B values are loaded once for two rows and
// two independent FMA chains hide each other's load latency.
constexpr int kSkinnyRows = 256;
constexpr int kSkinnyThreads = 128;
constexpr int kSkinnyMax = 8;

// Scale field of an output value as the split path defines it (0 for zero, else
// max(1, biased exponent)); complex outputs are never folded.
__device__ __forceinline__ int out_field(double v) {
  const uint32_t hi = (uint32_t)__double2hiint(v) & 0x7FFFFFFFu, lo = (uint32_t)__double2loint(v);
  return (hi | lo) ? max(1, (int)(hi >> 20)) : 0;
}
__device__ __forceinline__ int out_field(double2 v) { return max(out_field(v.x), out_field(v.y)); }

template <typename T, int NN>
__device__ __forceinline__ void skinny_row(const GemmCBlk& cb, const GemmTask* __restrict__ task, int row,
                                           const T* __restrict__ A, const T* __restrict__ As, const T* __restrict__ B,
                                           const T* __restrict__ Bs, T* __restrict__ C, bool want, int& f) {
  T acc[NN];
#pragma unroll
  for (int j = 0; j < NN; ++j) acc[j] = zero_of(T());
  for (int t = cb.t0; t < cb.t1; ++t) {
    const GemmTask tk = task[t];
    const int k = tk.k;
    const T* a = operand_block(A, As, tk.a_off) + (int64_t)row * tk.a_rs;
    const T* b = operand_block(B, Bs, tk.b_off);
    const unsigned long long sg = sign_mask(tk.sign);
    for (int kk = 0; kk < k; ++kk) {
      const T av = flip(__ldg(a + (int64_t)kk * tk.a_cs), sg);
#pragma unroll
      for (int j = 0; j < NN; ++j) fma_acc(acc[j], av, __ldg(b + kk * NN + j));
    }
  }
  T* out = C + cb.c_off + (int64_t)row * NN;
#pragma unroll
  for (int j = 0; j < NN; ++j) out[j] = acc[j];
  if (want) {
    f = 0;
#pragma unroll
    for (int j = 0; j < NN; ++j) f = max(f, out_field(acc[j]));
  }
}

// Rows row0 and row0 + kSkinnyThreads (both inside the block) in one pass.
template <typename T, int NN>
__device__ __forceinline__ void skinny_row_pair(const GemmCBlk& cb, const GemmTask* __restrict__ task, int row0,
                                                const T* __restrict__ A, const T* __restrict__ As,
                                                const T* __restrict__ B, const T* __restrict__ Bs,
                                                T* __restrict__ C, bool want, int& f0, int& f1) {
  T acc0[NN], acc1[NN];
#pragma unroll
  for (int j = 0; j < NN; ++j) acc0[j] = acc1[j] = zero_of(T());
  for (int t = cb.t0; t < cb.t1; ++t) {
    const GemmTask tk = task[t];
    const int k = tk.k;
    const T* a0 = operand_block(A, As, tk.a_off) + (int64_t)row0 * tk.a_rs;
    const T* a1 = a0 + (int64_t)kSkinnyThreads * tk.a_rs;
    const T* b = operand_block(B, Bs, tk.b_off);
    const unsigned long long sg = sign_mask(tk.sign);
    for (int kk = 0; kk < k; ++kk) {
      const T x0 = flip(__ldg(a0 + (int64_t)kk * tk.a_cs), sg);
      const T x1 = flip(__ldg(a1 + (int64_t)kk * tk.a_cs), sg);
#pragma unroll
      for (int j = 0; j < NN; ++j) {
        const T bj = __ldg(b + kk * NN + j);
        fma_acc(acc0[j], x0, bj);
        fma_acc(acc1[j], x1, bj);
      }
    }
  }
  T* out0 = C + cb.c_off + (int64_t)row0 * NN;
  T* out1 = out0 + (int64_t)kSkinnyThreads * NN;
#pragma unroll
  for (int j = 0; j < NN; ++j) {
    out0[j] = acc0[j];
    out1[j] = acc1[j];
  }
  if (want) {
    f0 = f1 = 0;
#pragma unroll
    for (int j = 0; j < NN; ++j) {
      f0 = max(f0, out_field(acc0[j]));
      f1 = max(f1, out_field(acc1[j]));
    }
  }
}

// Row row0 of an item and, if inside the block, row0 + kSkinnyThreads.
// f0, f1: the rows' output fields when `want` (f1 stays -1 when row1 is outside the block).
template <typename T, int NN>
__device__ __forceinline__ void skinny_rows(const GemmCBlk& cb, const GemmTask* __restrict__ task, int row0,
                                            const T* __restrict__ A, const T* __restrict__ As, const T* __restrict__ B,
                                            const T* __restrict__ Bs, T* __restrict__ C, bool want, int& f0,
                                            int& f1) {
  const int row1 = row0 + kSkinnyThreads;
  if constexpr (sizeof(T) == 8 && NN <= 4) {
    if (row1 < cb.m) {
      skinny_row_pair<T, NN>(cb, task, row0, A, As, B, Bs, C, want, f0, f1);
      return;
    }
  }
  skinny_row<T, NN>(cb, task, row0, A, As, B, Bs, C, want, f0);
  if (row1 < cb.m) skinny_row<T, NN>(cb, task, row1, A, As, B, Bs, C, want, f1);
}

// atomicMax of v into fields[key] once per group of lanes with the same key.
__device__ __forceinline__ void fold_field(unsigned mask, int key, int v, int32_t* __restrict__ fields) {
  const unsigned m = __match_any_sync(mask, key);
  const int x = (int)__reduce_max_sync(m, (unsigned)max(v, 0));
  if (key >= 0 && x > 0 && (int)(threadIdx.x & 31) == __ffs(m) - 1) atomicMax(fields + key, x);
}

// Resident CTAs per SM the kernel is compiled for: 8 for real operands (64 registers, no
// spills at two rows per thread); complex ones need their registers, the more the wider the
// blocks (the kernel is instantiated for the plan's largest n: MAXN = 2, 4 or 8).
template <typename T, int MAXN> struct SkinnyMinBlocks { static constexpr int value = MAXN <= 2 ? 6 : MAXN <= 4 ? 4 : 2; };
template <int MAXN> struct SkinnyMinBlocks<double, MAXN> { static constexpr int value = 8; };

template <typename T, int MAXN>
__global__ void __launch_bounds__(kSkinnyThreads, SkinnyMinBlocks<T, MAXN>::value) k_gemm_skinny(
    const GemmCBlk* __restrict__ cblk, const GemmTask* __restrict__ task, const GemmRowChunk* __restrict__ items,
    int nitems, const T* __restrict__ A, const T* __restrict__ As, const T* __restrict__ B, const T* __restrict__ Bs,
    T* __restrict__ C, const SkinnyFuse* __restrict__ fuse, int32_t* __restrict__ fields) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const GemmRowChunk item = items[it];
    const GemmCBlk cb = cblk[item.cblk];
    const int row = item.chunk * kSkinnyRows + threadIdx.x;
    if (row >= cb.m) continue;
    const SkinnyFuse fz = fuse ? fuse[item.cblk] : SkinnyFuse{-1, 1};
    const bool want = fz.exp_base >= 0;   // uniform over the item
    int f0 = 0, f1 = -1;
    if (MAXN <= 2) {
      if (cb.n == 1) skinny_rows<T, 1>(cb, task, row, A, As, B, Bs, C, want, f0, f1);
      else skinny_rows<T, 2>(cb, task, row, A, As, B, Bs, C, want, f0, f1);
    } else if (MAXN <= 4) {
      switch (cb.n) {
        case 1: skinny_rows<T, 1>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 2: skinny_rows<T, 2>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 3: skinny_rows<T, 3>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        default: skinny_rows<T, 4>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
      }
    } else {
      switch (cb.n) {
        case 1: skinny_rows<T, 1>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 2: skinny_rows<T, 2>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 3: skinny_rows<T, 3>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 4: skinny_rows<T, 4>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 5: skinny_rows<T, 5>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 6: skinny_rows<T, 6>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        case 7: skinny_rows<T, 7>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
        default: skinny_rows<T, 8>(cb, task, row, A, As, B, Bs, C, want, f0, f1); break;
      }
    }
    if (want) {
      // a row's n outputs lie in one row of the later operand (k3 is a multiple of n)
      const unsigned mask = __activemask();
      fold_field(mask, fz.exp_base + row * cb.n / fz.k3, f0, fields);
      fold_field(mask, f1 >= 0 ? fz.exp_base + (row + kSkinnyThreads) * cb.n / fz.k3 : -1, f1, fields);
    }
  }
}


}  // namespace

bool skinny_cblk(const GemmSchedule& g, int32_t q) {
  const GemmCBlk& cb = g.cblk[q];
  if (cb.n > kSkinnyMax) return false;
  for (int32_t t = cb.t0; t < cb.t1; ++t)
    if (g.task[t].k > kSkinnyMax) return false;
  return true;
}

int skinny_rows_per_item() { return kSkinnyRows; }

template <typename T, int MAXN>
void launch_skinny_t(const GemmSchedule& g, const Operands& op, void* c, int grid, cudaStream_t s,
                     const SkinnyFuse* fuse, int32_t* fields) {
  k_gemm_skinny<T, MAXN><<<grid, kSkinnyThreads, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(),
                                                   g.d_skinny.as<GemmRowChunk>(), (int)g.skinny.size(),
                                                   static_cast<const T*>(op.a), static_cast<const T*>(op.a_src),
                                                   static_cast<const T*>(op.b), static_cast<const T*>(op.b_src),
                                                   static_cast<T*>(c), fuse, fields);
}

template <typename T, int TM, int TN>
void launch_dfma_tile(const GemmSchedule& g, const Operands& op, void* c, int grid, cudaStream_t s) {
  k_gemm_dfma<T, TM, TN><<<grid, NT, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(), g.d_tile.as<GemmTile>(),
                                             (int)g.tile.size(), static_cast<const T*>(op.a),
                                             static_cast<const T*>(op.a_src), static_cast<const T*>(op.b),
                                             static_cast<const T*>(op.b_src), static_cast<T*>(c), g.d_counter.as<int>());
}

template <typename T>
void launch_dfma_t(const GemmSchedule& g, const Operands& op, void* c, int grid, cudaStream_t s) {
  if (g.bm == 64) {
    launch_dfma_tile<T, 4, 2>(g, op, c, grid, s);
  } else {
    k_gemm_dfma32<T><<<grid, NT, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(), g.d_tile.as<GemmTile>(),
                                         (int)g.tile.size(), static_cast<const T*>(op.a),
                                         static_cast<const T*>(op.a_src), static_cast<const T*>(op.b),
                                         static_cast<const T*>(op.b_src), static_cast<T*>(c), g.d_counter.as<int>());
  }
}

// CTAs of one full wave: the grid-stride loop then has no partial second wave.
template <typename T, int MAXN>
int skinny_wave(int num_sms) {
  static int per_sm = [] {
    int n = 0;
    QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_gemm_skinny<T, MAXN>, kSkinnyThreads, 0));
    return std::max(1, n);
  }();
  return std::max(1, num_sms) * per_sm;
}

// the kernel variant of a plan: real operands always use MAXN = 8 (64 registers either way);
// complex ones the narrowest that covers the plan's blocks
int skinny_variant(bool cplx, int maxn) { return !cplx ? 8 : maxn <= 2 ? 2 : maxn <= 4 ? 4 : 8; }

int skinny_grid(int items, bool cplx, int maxn, int num_sms) {
  int wave = 0;
  switch (skinny_variant(cplx, maxn)) {
    case 2: wave = skinny_wave<double2, 2>(num_sms); break;
    case 4: wave = skinny_wave<double2, 4>(num_sms); break;
    default: wave = cplx ? skinny_wave<double2, 8>(num_sms) : skinny_wave<double, 8>(num_sms); break;
  }
  return std::max(1, std::min(items, wave));
}

void launch_gemm_f64_skinny(const GemmSchedule& g, const Operands& op, void* c, bool cplx, int num_sms,
                            cudaStream_t s, const SkinnyFuse* fuse, int32_t* fields) {
  const int ns = (int)g.skinny.size();
  if (!ns) return;
  const int grid = skinny_grid(ns, cplx, g.skinny_maxn, num_sms);
  switch (skinny_variant(cplx, g.skinny_maxn)) {
    case 2: launch_skinny_t<double2, 2>(g, op, c, grid, s, fuse, fields); break;
    case 4: launch_skinny_t<double2, 4>(g, op, c, grid, s, fuse, fields); break;
    default:
      if (cplx) launch_skinny_t<double2, 8>(g, op, c, grid, s, fuse, fields);
      else launch_skinny_t<double, 8>(g, op, c, grid, s, fuse, fields);
  }
  QLTG_CUDA(cudaGetLastError());
}

void launch_gemm_f64(const GemmSchedule& g, const Operands& op, void* c, bool cplx, int num_sms, cudaStream_t s) {
  const int nt = (int)g.tile.size();
  launch_gemm_f64_skinny(g, op, c, cplx, num_sms, s);
  if (nt) {
    QLTG_CUDA(cudaMemsetAsync(g.d_counter.get(), 0, sizeof(int), s));
    const int grid = std::min(nt, std::max(1, num_sms) * 4);
    if (cplx)
      launch_dfma_t<double2>(g, op, c, grid, s);
    else
      launch_dfma_t<double>(g, op, c, grid, s);
    QLTG_CUDA(cudaGetLastError());
  }
}

// ------------------------------------------------------------------ FP64 rate self-test
// The two FP64 arithmetic paths of this GPU side by side, measured rather than assumed: a
// DFMA loop (8 independent chains per thread) and an mma.sync m8n8k4 f64 loop (4 independent
// accumulator fragments per warp; 8 x 8 x 4 multiply-adds = 512 flops per instruction). The
// FP64 GEMM kernels above use DFMA because the two run at the same rate here while the MMA
// path pads every block to 8 x 8 x 4 fragments.
constexpr int kRateIters = 4096;
__global__ void __launch_bounds__(256) k_rate_dfma(double* out, double seed) {
  double a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed + threadIdx.x + i;
  const double b = 1.0 + 1e-12 * seed, c = 1e-300;
  for (int it = 0; it < kRateIters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = fma(a[i], b, c);
  double t = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) t += a[i];
  if (t == 1.2345) out[0] = t;   // keeps the loop; never true for these inputs
}
__global__ void __launch_bounds__(256) k_rate_dmma(double* out, double seed) {
  const double av = seed + (threadIdx.x & 31), bv = 1.0 + 1e-12 * seed;
  double d[4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i][0] = d[i][1] = 0.0;
  for (int it = 0; it < kRateIters; ++it)
#pragma unroll
    for (int i = 0; i < 4; ++i)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(d[i][0]), "+d"(d[i][1])
                   : "d"(av), "d"(bv));
  double t = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) t += d[i][0] + d[i][1];
  if (t == 1.2345) out[0] = t;
}

void fp64_rates(int num_sms, cudaStream_t s, double* dfma_tflops, double* dmma_tflops) {
  DevBuf sink(sizeof(double));
  const int grid = std::max(1, num_sms) * 8;
  cudaEvent_t e[4];
  for (auto& x : e) QLTG_CUDA(cudaEventCreate(&x));
  k_rate_dfma<<<grid, 256, 0, s>>>(sink.as<double>(), 1.0);   // warm-up
  k_rate_dmma<<<grid, 256, 0, s>>>(sink.as<double>(), 1.0);
  QLTG_CUDA(cudaEventRecord(e[0], s));
  k_rate_dfma<<<grid, 256, 0, s>>>(sink.as<double>(), 2.0);
  QLTG_CUDA(cudaEventRecord(e[1], s));
  QLTG_CUDA(cudaEventRecord(e[2], s));
  k_rate_dmma<<<grid, 256, 0, s>>>(sink.as<double>(), 2.0);
  QLTG_CUDA(cudaEventRecord(e[3], s));
  QLTG_CUDA(cudaGetLastError());
  QLTG_CUDA(cudaEventSynchronize(e[3]));
  float ms_f = 0, ms_m = 0;
  QLTG_CUDA(cudaEventElapsedTime(&ms_f, e[0], e[1]));
  QLTG_CUDA(cudaEventElapsedTime(&ms_m, e[2], e[3]));
  for (auto x : e) cudaEventDestroy(x);
  const double threads = (double)grid * 256, warps = threads / 32;
  *dfma_tflops = threads * kRateIters * 8 * 2 / (ms_f * 1e-3) / 1e12;
  *dmma_tflops = warps * kRateIters * 4 * 512 / (ms_m * 1e-3) / 1e12;
}

}  // namespace qltg
