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

constexpr int BM = 32, BN = 32, BK = 32, NT = 256;

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

// One output tile of BM x BN per work item; 16 x 16 threads, each 2 x 2 outputs at
// (ty + 16 i, tx + 16 j). Operand tiles are staged through shared memory (A transposed so
// a warp reads one broadcast row); outputs outside the block are predicated off so no FP64
// issue slot is spent on padding. Work items are taken longest-first from an atomic
// counter (the plan zeroes it before each launch), so the few very long tiles start first
// and the rest fill in behind them.
template <typename T>
__global__ void __launch_bounds__(NT) k_gemm_dfma(const GemmCBlk* __restrict__ cblk, const GemmTask* __restrict__ task,
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

// Skinny output blocks (n <= 8, every task k <= 8): thread per output row, the row's n
// outputs in registers, instantiated per n so no FP64 slot is spent on absent columns.
constexpr int kSkinnyRows = 256;
constexpr int kSkinnyMax = 8;

template <typename T, int NN>
__device__ __forceinline__ void skinny_row(const GemmCBlk& cb, const GemmTask* __restrict__ task, int row,
                                           const T* __restrict__ A, const T* __restrict__ As, const T* __restrict__ B,
                                           const T* __restrict__ Bs, T* __restrict__ C) {
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
}

// Resident CTAs per SM the kernel is compiled for: 6 for real operands (40 registers, no
// spills); complex ones need their registers (1).
template <typename T> struct SkinnyMinBlocks { static constexpr int value = 1; };
template <> struct SkinnyMinBlocks<double> { static constexpr int value = 6; };

template <typename T>
__global__ void __launch_bounds__(kSkinnyRows, SkinnyMinBlocks<T>::value) k_gemm_skinny(const GemmCBlk* __restrict__ cblk,
                                                             const GemmTask* __restrict__ task,
                                                             const GemmRowChunk* __restrict__ items, int nitems,
                                                             const T* __restrict__ A, const T* __restrict__ As,
                                                             const T* __restrict__ B, const T* __restrict__ Bs,
                                                             T* __restrict__ C) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const GemmRowChunk item = items[it];
    const GemmCBlk cb = cblk[item.cblk];
    const int row = item.chunk * kSkinnyRows + threadIdx.x;
    if (row >= cb.m) continue;
    switch (cb.n) {
      case 1: skinny_row<T, 1>(cb, task, row, A, As, B, Bs, C); break;
      case 2: skinny_row<T, 2>(cb, task, row, A, As, B, Bs, C); break;
      case 3: skinny_row<T, 3>(cb, task, row, A, As, B, Bs, C); break;
      case 4: skinny_row<T, 4>(cb, task, row, A, As, B, Bs, C); break;
      case 5: skinny_row<T, 5>(cb, task, row, A, As, B, Bs, C); break;
      case 6: skinny_row<T, 6>(cb, task, row, A, As, B, Bs, C); break;
      case 7: skinny_row<T, 7>(cb, task, row, A, As, B, Bs, C); break;
      default: skinny_row<T, 8>(cb, task, row, A, As, B, Bs, C); break;
    }
  }
}


// ------------------------------------------------------------------ double-float skinny rows
// Split mode computes the skinny blocks in double-float arithmetic on the FP32 pipe: FP64
// issues at about 1/64 of the FP32 rate on this GPU and these blocks do about two flops per
// 8-byte element, so the FP64 skinny kernel is FP64-pipe bound. Each operand element becomes
// an unevaluated sum h + l of two floats (47 significant bits) after scaling by a power of
// two that brings the largest magnitude of its row (A) or stacked column (B) into [1, 2).
// Products are Dekker's exact product by FMA (TwoProd) plus the two cross terms h l, sums
// are Knuth's TwoSum, and the result goes back to FP64 by exponent arithmetic and one FP64
// add of its two parts. Terms below 2^-126 of the row or column scale are dropped; the error
// is about 2^-45 sum |a||b| per output (FP64's own bound is K 2^-53 sum |a||b|). Rows whose
// scale is tiny, subnormal or not finite, and blocks whose B has such a column, run the FP64
// rows instead, as do outputs that would leave the normal FP64 range.
constexpr int kDfFieldMin = 200;

// x (high, low words) scaled by 2^(1023 - F), F the largest exponent field of its row or
// column (kDfFieldMin <= F <= 2046), as h + l.
__device__ __forceinline__ float2 df_split(uint32_t hi, uint32_t lo, int F) {
  const uint32_t mag = hi & 0x7FFFFFFFu;
  const uint32_t thr = (uint32_t)(F - 126) << 20;   // mag >= thr: scaled value >= 2^-126
  // fraction bits 51..29 under the low 9 bits of the exponent field; adding (127 - F) << 23
  // makes the top bits the float exponent field - F + 127 (1..127 for kept values)
  const uint32_t hb = (__funnelshift_l(lo, hi, 3) + ((uint32_t)(127 - F) << 23)) | (hi & 0x80000000u);
  const float h = mag >= thr ? __uint_as_float(hb) : 0.0f;
  // fraction bits 28..6 as the integer part of 2^23 + r, times 2^-46 of h's power of two
  const float r = __fsub_rn(__uint_as_float(0x4B000000u | ((lo >> 6) & 0x7FFFFFu)), 8388608.0f);
  const float unit = __fmul_rn(__uint_as_float(__float_as_uint(h) & 0xFF800000u), 0x1p-46f);
  return make_float2(h, __fmul_rn(r, unit));
}

// The FP64 value with the sign and fraction of the normal float `bits` and exponent field
// (its float field + D): exact; the caller keeps that field in 1..2046.
__device__ __forceinline__ double df_to_double(uint32_t bits, int D) {
  const uint32_t mag = bits & 0x7FFFFFFFu;
  return __hiloint2double((int)(((mag >> 3) + ((uint32_t)D << 20)) | (bits & 0x80000000u)), (int)(bits << 29));
}

template <int K, int N>
__device__ __forceinline__ bool df_row(const DfADesc* __restrict__ ad, const float2* __restrict__ bp,
                                       const int* __restrict__ fb, int row, const double* __restrict__ A,
                                       const double* __restrict__ As, double* __restrict__ out) {
  uint32_t hi[K], lo[K];
  uint32_t mx = 0;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const DfADesc d = ad[i];
    const double v = __ldg(operand_block(A, As, d.a_off) + (int64_t)row * d.a_rs);
    hi[i] = (uint32_t)__double2hiint(v);
    lo[i] = (uint32_t)__double2loint(v);
    mx = max(mx, hi[i] & 0x7FFFFFFFu);
  }
  const int F = (int)(mx >> 20);
  if (F < kDfFieldMin || F > 2046) return false;
  float2 a[K];
#pragma unroll
  for (int i = 0; i < K; ++i) a[i] = df_split(hi[i], lo[i], F);
  double res[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    float sh = 0.0f, sl = 0.0f;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const float2 b = __ldg(bp + i * 8 + j);
      const float p = __fmul_rn(a[i].x, b.x);
      float e = __fmaf_rn(a[i].x, b.x, -p);   // TwoProd: a.h b.h = p + e exactly
      e = __fmaf_rn(a[i].x, b.y, e);
      e = __fmaf_rn(a[i].y, b.x, e);
      const float s = __fadd_rn(sh, p);       // TwoSum: sh + p = s + err exactly
      const float v = __fsub_rn(s, sh);
      const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(p, v));
      sh = s;
      sl = __fadd_rn(sl, __fadd_rn(err, e));
    }
    const float s = __fadd_rn(sh, sl);
    const float v = __fsub_rn(s, sh);
    const float l = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(sl, v));
    const uint32_t hs = __float_as_uint(s), ls = __float_as_uint(l);
    const uint32_t hm = hs & 0x7FFFFFFFu, lm = ls & 0x7FFFFFFFu;
    if (hm == 0) {
      res[j] = 0.0;
      continue;
    }
    // value = (s + l) 2^(F + FB - 2046): FP64 exponent field = float field + D
    const int D = F + __ldg(fb + j) - 1150;
    const int dh = (int)(hm >> 23) + D;
    if (hm < 0x00800000u || dh < 64 || dh > 2046) return false;
    const double H = df_to_double(hs, D);
    const double L = (lm >= 0x00800000u && (int)(lm >> 23) + D >= 1) ? df_to_double(ls, D) : 0.0;
    res[j] = __dadd_rn(H, L);
  }
#pragma unroll
  for (int j = 0; j < N; ++j) out[j] = res[j];
  return true;
}

template <int K>
__device__ __forceinline__ bool df_row_n(int n, const DfADesc* ad, const float2* bp, const int* fb, int row,
                                         const double* A, const double* As, double* out) {
  switch (n) {
    case 1: return df_row<K, 1>(ad, bp, fb, row, A, As, out);
    case 2: return df_row<K, 2>(ad, bp, fb, row, A, As, out);
    case 3: return df_row<K, 3>(ad, bp, fb, row, A, As, out);
    case 4: return df_row<K, 4>(ad, bp, fb, row, A, As, out);
    case 5: return df_row<K, 5>(ad, bp, fb, row, A, As, out);
    case 6: return df_row<K, 6>(ad, bp, fb, row, A, As, out);
    case 7: return df_row<K, 7>(ad, bp, fb, row, A, As, out);
    default: return df_row<K, 8>(ad, bp, fb, row, A, As, out);
  }
}

__device__ __forceinline__ bool df_row_kn(int k, int n, const DfADesc* ad, const float2* bp, const int* fb, int row,
                                          const double* A, const double* As, double* out) {
  switch (k) {
    case 1: return df_row_n<1>(n, ad, bp, fb, row, A, As, out);
    case 2: return df_row_n<2>(n, ad, bp, fb, row, A, As, out);
    case 3: return df_row_n<3>(n, ad, bp, fb, row, A, As, out);
    case 4: return df_row_n<4>(n, ad, bp, fb, row, A, As, out);
    case 5: return df_row_n<5>(n, ad, bp, fb, row, A, As, out);
    case 6: return df_row_n<6>(n, ad, bp, fb, row, A, As, out);
    case 7: return df_row_n<7>(n, ad, bp, fb, row, A, As, out);
    default: return df_row_n<8>(n, ad, bp, fb, row, A, As, out);
  }
}

// One thread per output row, as k_gemm_skinny; rows the double-float path declines run the
// FP64 row code.
__global__ void __launch_bounds__(kSkinnyRows, 4) k_gemm_skinny_df(
    const GemmCBlk* __restrict__ cblk, const GemmTask* __restrict__ task, const GemmRowChunk* __restrict__ items,
    int nitems, const DfCBlk* __restrict__ dcb, const DfADesc* __restrict__ ad, const float2* __restrict__ bp,
    const int* __restrict__ fb, const int* __restrict__ ok, const double* __restrict__ A,
    const double* __restrict__ As, const double* __restrict__ B, const double* __restrict__ Bs,
    double* __restrict__ C) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const GemmRowChunk item = items[it];
    const GemmCBlk cb = cblk[item.cblk];
    const int row = item.chunk * kSkinnyRows + threadIdx.x;
    if (row >= cb.m) continue;
    const DfCBlk d = dcb[item.cblk];
    if (d.k > 0 && __ldg(ok + item.cblk) &&
        df_row_kn(d.k, cb.n, ad + d.desc0, bp + (int64_t)d.desc0 * 8, fb + (int64_t)item.cblk * 8, row, A, As,
                  C + cb.c_off + (int64_t)row * cb.n))
      continue;
    switch (cb.n) {
      case 1: skinny_row<double, 1>(cb, task, row, A, As, B, Bs, C); break;
      case 2: skinny_row<double, 2>(cb, task, row, A, As, B, Bs, C); break;
      case 3: skinny_row<double, 3>(cb, task, row, A, As, B, Bs, C); break;
      case 4: skinny_row<double, 4>(cb, task, row, A, As, B, Bs, C); break;
      case 5: skinny_row<double, 5>(cb, task, row, A, As, B, Bs, C); break;
      case 6: skinny_row<double, 6>(cb, task, row, A, As, B, Bs, C); break;
      case 7: skinny_row<double, 7>(cb, task, row, A, As, B, Bs, C); break;
      default: skinny_row<double, 8>(cb, task, row, A, As, B, Bs, C); break;
    }
  }
}

// B side, one warp per output block: column scale fields of the stacked K x n operand, the
// block's eligibility (every column all zero or with a field in kDfFieldMin..2046), and the
// float pairs of every element with the task sign folded in.
__global__ void __launch_bounds__(256) k_df_prep_b(const GemmCBlk* __restrict__ cblk, const DfCBlk* __restrict__ dcb,
                                                   int ncb, const DfBDesc* __restrict__ bd,
                                                   const double* __restrict__ B, const double* __restrict__ Bs,
                                                   float2* __restrict__ bp, int* __restrict__ fb,
                                                   int* __restrict__ ok) {
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  for (int q = blockIdx.x * warps + (threadIdx.x >> 5); q < ncb; q += gridDim.x * warps) {
    const DfCBlk d = dcb[q];
    if (d.k == 0) continue;   // uniform over the warp
    const int n = cblk[q].n, K = d.k;
    int f = 0;
    bool nonzero = false;
    if (lane < n) {
      for (int i = 0; i < K; ++i) {
        const uint64_t ab =
            (uint64_t)__double_as_longlong(operand_block(B, Bs, bd[d.desc0 + i].b_off)[lane]) & 0x7FFFFFFFFFFFFFFFull;
        nonzero |= ab != 0;
        f = max(f, (int)(ab >> 52));
      }
      fb[(int64_t)q * 8 + lane] = f;
    }
    const bool good = __all_sync(0xffffffffu, lane >= n || !nonzero || (f >= kDfFieldMin && f <= 2046));
    if (lane == 0) ok[q] = good ? 1 : 0;
    for (int base = 0; base < K * n; base += 32) {
      const int idx = base + lane;
      const int i = idx / n, j = idx - i * n;
      const int fj = __shfl_sync(0xffffffffu, f, j & 31);
      if (idx < K * n) {
        const DfBDesc e = bd[d.desc0 + i];
        uint64_t bits = (uint64_t)__double_as_longlong(operand_block(B, Bs, e.b_off)[j]);
        if (e.sign < 0) bits ^= 0x8000000000000000ull;
        float2 pr = make_float2(0.0f, 0.0f);
        if (good && fj >= kDfFieldMin) pr = df_split((uint32_t)(bits >> 32), (uint32_t)bits, fj);
        bp[(int64_t)(d.desc0 + i) * 8 + j] = pr;
      }
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

template <typename T>
void launch_skinny_t(const GemmSchedule& g, const Operands& op, void* c, int grid, cudaStream_t s) {
  k_gemm_skinny<T><<<grid, kSkinnyRows, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(),
                                                g.d_skinny.as<GemmRowChunk>(), (int)g.skinny.size(),
                                                static_cast<const T*>(op.a), static_cast<const T*>(op.a_src),
                                                static_cast<const T*>(op.b), static_cast<const T*>(op.b_src),
                                                static_cast<T*>(c));
}

template <typename T>
void launch_dfma_t(const GemmSchedule& g, const Operands& op, void* c, int grid, cudaStream_t s) {
  k_gemm_dfma<T><<<grid, NT, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(), g.d_tile.as<GemmTile>(),
                                     (int)g.tile.size(), static_cast<const T*>(op.a), static_cast<const T*>(op.a_src),
                                     static_cast<const T*>(op.b), static_cast<const T*>(op.b_src), static_cast<T*>(c),
                                     g.d_counter.as<int>());
}

// CTAs of one full wave: the grid-stride loop then has no partial second wave.
template <typename T>
int skinny_wave(int num_sms) {
  static int per_sm = [] {
    int n = 0;
    QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_gemm_skinny<T>, kSkinnyRows, 0));
    return std::max(1, n);
  }();
  return std::max(1, num_sms) * per_sm;
}

int skinny_grid(int items, bool cplx, int num_sms) {
  return std::max(1, std::min(items, cplx ? skinny_wave<double2>(num_sms) : skinny_wave<double>(num_sms)));
}

void launch_gemm_f64_skinny(const GemmSchedule& g, const Operands& op, void* c, bool cplx, int num_sms,
                            cudaStream_t s) {
  const int ns = (int)g.skinny.size();
  if (!ns) return;
  const int grid = skinny_grid(ns, cplx, num_sms);
  if (cplx)
    launch_skinny_t<double2>(g, op, c, grid, s);
  else
    launch_skinny_t<double>(g, op, c, grid, s);
  QLTG_CUDA(cudaGetLastError());
}

void df_build(DfSkinny& df, const GemmSchedule& g, int num_sms, cudaStream_t s) {
  const int ncb = (int)g.cblk.size();
  std::vector<DfCBlk> cbs(std::max(ncb, 1), DfCBlk{0, 0});
  std::vector<DfADesc> ad;
  std::vector<DfBDesc> bd;
  for (int32_t q = 0; q < ncb; ++q) {
    if (!skinny_cblk(g, q)) continue;
    const GemmCBlk& cb = g.cblk[q];
    int k = 0;
    for (int32_t t = cb.t0; t < cb.t1; ++t) k += g.task[t].k;
    if (k < 1 || k > kDfMaxK) continue;
    cbs[q] = DfCBlk{(int32_t)ad.size(), k};
    for (int32_t t = cb.t0; t < cb.t1; ++t) {
      const GemmTask& tk = g.task[t];
      for (int kk = 0; kk < tk.k; ++kk) {
        ad.push_back(DfADesc{tk.a_off + (int64_t)kk * tk.a_cs, tk.a_rs, 0});
        bd.push_back(DfBDesc{tk.b_off + (int64_t)kk * cb.n, tk.sign, 0});
      }
    }
  }
  QLTG_CHECK(ad.size() < ((size_t)1 << 28), QLTG_ERR_UNSUPPORTED, "too many skinny rows");
  df.nrows = (int64_t)ad.size();
  df.ready = false;
  if (ad.empty()) ad.push_back(DfADesc{0, 0, 0});
  if (bd.empty()) bd.push_back(DfBDesc{0, 1, 0});
  df.d_cb = upload(cbs, s);
  df.d_adesc = upload(ad, s);
  df.d_bdesc = upload(bd, s);
  df.d_bpair.alloc(std::max<int64_t>(df.nrows, 1) * 8 * sizeof(float2));
  df.d_fb.alloc((int64_t)std::max(ncb, 1) * 8 * sizeof(int));
  df.d_ok.alloc((int64_t)std::max(ncb, 1) * sizeof(int));
  QLTG_CUDA(cudaMemsetAsync(df.d_ok.get(), 0, (int64_t)std::max(ncb, 1) * sizeof(int), s));
  df.prep_grid = std::max(1, std::min((ncb + 7) / 8, std::max(1, num_sms) * 8));
  int per_sm = 0;
  QLTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_skinny_df, kSkinnyRows, 0));
  df.grid = std::max(1, std::min((int)g.skinny.size(), std::max(1, num_sms) * std::max(1, per_sm)));
}

void df_prep_b(DfSkinny& df, const GemmSchedule& g, const Operands& op, cudaStream_t s) {
  if (df.nrows > 0) {
    k_df_prep_b<<<df.prep_grid, 256, 0, s>>>(g.d_cblk.as<GemmCBlk>(), df.d_cb.as<DfCBlk>(), (int)g.cblk.size(),
                                             df.d_bdesc.as<DfBDesc>(), static_cast<const double*>(op.b),
                                             static_cast<const double*>(op.b_src), df.d_bpair.as<float2>(),
                                             df.d_fb.as<int>(), df.d_ok.as<int>());
    QLTG_CUDA(cudaGetLastError());
  }
  df.ready = true;
}

void launch_skinny_df(const GemmSchedule& g, const DfSkinny& df, const Operands& op, void* c, int num_sms,
                      cudaStream_t s) {
  const int ns = (int)g.skinny.size();
  if (!ns) return;
  if (df.nrows == 0) {   // no block on the double-float path
    launch_gemm_f64_skinny(g, op, c, false, num_sms, s);
    return;
  }
  k_gemm_skinny_df<<<df.grid, kSkinnyRows, 0, s>>>(
      g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(), g.d_skinny.as<GemmRowChunk>(), ns, df.d_cb.as<DfCBlk>(),
      df.d_adesc.as<DfADesc>(), df.d_bpair.as<float2>(), df.d_fb.as<int>(), df.d_ok.as<int>(),
      static_cast<const double*>(op.a), static_cast<const double*>(op.a_src), static_cast<const double*>(op.b),
      static_cast<const double*>(op.b_src), static_cast<double*>(c));
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

}  // namespace qltg
