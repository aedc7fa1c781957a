// Grouped FP64 / complex128 GEMM over all tasks of one contraction, one launch.
//
// Replaces the reference's serial loop of one cblas_dgemm / cublasDgemm per task with
// beta = 0 for the first task of an output block and beta = 1 after it
// (global_operations.h:895-992 -> raw_data_operations.h:530-548 -> blas_level3.h:35-56,
// :797-856). Here every 64 x 64 output tile is owned by one CTA that loops over all
// tasks of its output block, accumulating C_tile += sign_t * A_t[tile rows, :] B_t[:, tile
// cols] in registers, and stores the tile once: no read-modify-write of C, no atomics,
// deterministic. Tiles are issued longest-first over a persistent grid.
#include <algorithm>

#include "ctrct.h"

namespace qltg {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

struct Cd { double x, y; };

__device__ __forceinline__ void fma_acc(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void fma_acc(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ double zero_of(double) { return 0.0; }
__device__ __forceinline__ double2 zero_of(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double scale(double x, double s) { return x * s; }
__device__ __forceinline__ double2 scale(double2 x, double s) { return make_double2(x.x * s, x.y * s); }

template <typename T>
__global__ void __launch_bounds__(NT) k_gemm_grouped(const GemmCBlk* __restrict__ cblk,
                                                     const GemmTask* __restrict__ task,
                                                     const GemmTile* __restrict__ tiles, int ntiles,
                                                     const T* __restrict__ A, const T* __restrict__ B,
                                                     T* __restrict__ C) {
  __shared__ T As[BK][BM];
  __shared__ T Bs[BK][BN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    const GemmTile tl = tiles[ti];
    const GemmCBlk cb = cblk[tl.cblk];
    const int r0 = tl.tm * BM, c0 = tl.tn * BN;
    const int m = cb.m, n = cb.n;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = zero_of(T());
    bool rv[4], cv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) { rv[i] = r0 + ty + 16 * i < m; cv[i] = c0 + tx + 16 * i < n; }
    for (int t = cb.t0; t < cb.t1; ++t) {
      const GemmTask tk = task[t];
      const T* a = A + tk.a_off;
      const T* b = B + tk.b_off;
      const int k = tk.k;
      const double sg = (double)tk.sign;
      for (int k0 = 0; k0 < k; k0 += BK) {
        const int kc = min(BK, k - k0);
        // A tile: rows r0.., cols k0.. of the m x k row-major operand
#pragma unroll
        for (int e = threadIdx.x; e < BM * BK; e += NT) {
          const int row = e / BK, kk = e % BK;
          T v = zero_of(T());
          if (kk < kc && r0 + row < m) v = scale(a[(int64_t)(r0 + row) * k + k0 + kk], sg);
          As[kk][row] = v;
        }
        // B tile: rows k0.., cols c0.. of the k x n row-major operand
#pragma unroll
        for (int e = threadIdx.x; e < BK * BN; e += NT) {
          const int kk = e / BN, col = e % BN;
          T v = zero_of(T());
          if (kk < kc && c0 + col < n) v = b[(int64_t)(k0 + kk) * n + c0 + col];
          Bs[kk][col] = v;
        }
        __syncthreads();
        for (int kk = 0; kk < kc; ++kk) {
          T av[4], bv[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
          for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (rv[i])
#pragma unroll
              for (int j = 0; j < 4; ++j)
                if (cv[j]) fma_acc(acc[i][j], av[i], bv[j]);
        }
        __syncthreads();
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (rv[i] && cv[j]) C[cb.c_off + (int64_t)(r0 + ty + 16 * i) * n + c0 + tx + 16 * j] = acc[i][j];
  }
}

}  // namespace

void launch_gemm_f64(const GemmSchedule& g, const void* a, const void* b, void* c, bool cplx, int num_sms,
                     cudaStream_t s) {
  const int nt = (int)g.tile.size();
  if (nt == 0) return;
  const int grid = std::min(nt, std::max(1, num_sms) * (cplx ? 2 : 3));
  if (cplx)
    k_gemm_grouped<double2><<<grid, NT, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(),
                                                g.d_tile.as<GemmTile>(), nt, static_cast<const double2*>(a),
                                                static_cast<const double2*>(b), static_cast<double2*>(c));
  else
    k_gemm_grouped<double><<<grid, NT, 0, s>>>(g.d_cblk.as<GemmCBlk>(), g.d_task.as<GemmTask>(),
                                               g.d_tile.as<GemmTile>(), nt, static_cast<const double*>(a),
                                               static_cast<const double*>(b), static_cast<double*>(c));
  QLTG_CUDA(cudaGetLastError());
}

}  // namespace qltg
