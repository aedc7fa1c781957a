// Block-diagonal SVD (truncated) and QR of a block-sparse tensor.
//
// Reference path (per block-matrix, serial): group blocks by (left flux, right flux)
// (tensor_manipulation/ten_decomp/ten_decomp_basic.h:68-106), densify each group
// (raw_data_operations.h:550-575), one LAPACK/cuSOLVER gesvd or geqrf+orgqr call each
// (framework/hp_numeric/lapack.h:41-82, :332-366, :811-909, :1483-1631), host truncation
// (tensor_manipulation/ten_decomp/ten_svd.h:281-372) and per-row copies into U/S/Vt or
// Q/R blocks (data_blk_operations.h:969-1078).
//
// Here: grouping is host metadata; one gather launch densifies every group; one batched
// launch decomposes all groups - one-sided (Hestenes) Jacobi in FP64 with round-robin pair
// ordering for the SVD, Householder with LAPACK's reflector convention for the QR - where a
// group is spread over a thread-block cluster of up to 16 CTAs (one SM each, in proportion
// to its share of the work) that step through the rotation rounds together on the cluster
// barrier, and the QR runs in panels whose updates spread over every group's column tiles;
// one scatter launch builds the result blocks. The truncation (the reference's global sort
// of the singular values, kept dimension and error) runs on the device too; the host reads
// back only the kept dimension, the error and the kept count per group, which size the
// result tensors.
#include <cooperative_groups.h>
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>

#include "ctrct.h"

namespace cg = cooperative_groups;

namespace qltg {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSweeps = 60;
constexpr int kMaxCluster = 16;   // CTAs of the largest Jacobi cluster (non-portable size)
constexpr int kJacobiSmem = 200 * 1024;   // dynamic shared memory of k_jacobi (two column blocks)

// ------------------------------------------------------------------ complex helpers
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double abs2(double a) { return a * a; }
__device__ __forceinline__ double abs2(double2 a) { return a.x * a.x + a.y * a.y; }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ------------------------------------------------------------------ gather / scatter
struct CopyDesc {
  int64_t src_off;     // element offset of the source block (row-major rd x cd)
  int64_t dst_off;     // element offset of the dense group matrix
  int64_t elem_begin;  // prefix over descriptors (elements)
  int32_t rd, cd;      // block rows / cols
  int32_t ro, co;      // row / col offset inside the group matrix
  int32_t ld;          // leading dimension of the dense storage
  int32_t col_major;   // 1: dense[c * ld + r]; 0: dense[r * ld + c]
};

template <typename T>
__global__ void k_gather(const CopyDesc* __restrict__ d, int nd, int64_t total, const T* __restrict__ src,
                         T* __restrict__ dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (d[mid].elem_begin <= e) lo = mid; else hi = mid - 1;
    }
    const CopyDesc c = d[lo];
    const int64_t l = e - c.elem_begin;
    const int64_t i = l / c.cd, j = l % c.cd;
    const int64_t r = c.ro + i, col = c.co + j;
    dst[c.dst_off + (c.col_major ? col * c.ld + r : r * c.ld + col)] = src[c.src_off + l];
  }
}

// Result scatter: out_blk[i, j] = dense[row(i), col(j)] where one of the two index maps is a
// contiguous range and the other goes through a column list (kept singular vectors).
struct ScatterDesc {
  int64_t dst_off, src_off, elem_begin;
  int32_t rows, cols;      // output block shape
  int32_t r0, c0;          // start of the contiguous part
  int32_t ld;              // leading dimension of the dense factor
  int32_t col_major;       // dense factor storage
  int32_t list_on_cols;    // 1: cols map through list; 0: rows map through list
  int32_t list_off;        // offset into the index list
  int32_t conj;            // complex conjugate on the way (complex element types only)
};

template <typename T>
__global__ void k_scatter(const ScatterDesc* __restrict__ d, int nd, int64_t total, const int32_t* __restrict__ list,
                          const T* __restrict__ src, T* __restrict__ dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (d[mid].elem_begin <= e) lo = mid; else hi = mid - 1;
    }
    const ScatterDesc c = d[lo];
    const int64_t l = e - c.elem_begin;
    const int64_t i = l / c.cols, j = l % c.cols;
    const int64_t r = c.list_on_cols ? c.r0 + i : list[c.list_off + i];
    const int64_t q = c.list_on_cols ? list[c.list_off + j] : c.c0 + j;
    T v = src[c.src_off + (c.col_major ? q * c.ld + r : r * c.ld + q)];
    if (c.conj == 2 && r > q) v = T{};   // R: upper triangle only
    if constexpr (sizeof(T) == 16) {
      if (c.conj == 1) v.y = -v.y;
    }
    dst[c.dst_off + l] = v;
  }
}

// ------------------------------------------------------------------ one-sided Jacobi
struct JacobiJob {
  int64_t w_off;     // q vectors of length p, vector-major: W[v * p + e]
  int64_t v_off;     // q x q accumulated rotations, column-major: V[c * q + r]
  int32_t p, q;
};

// Round-robin ("circle") schedule: in round r of qq - 1 rounds, slot k pairs players
// pos(k) and pos(qq - 1 - k), with player 0 fixed.
__device__ __forceinline__ int rr_player(int slot, int r, int qq) {
  return slot == 0 ? 0 : ((slot - 1 + r) % (qq - 1)) + 1;
}

// ---- one-sided Jacobi: a round of disjoint column pairs in shared memory ----------------
// Columns are held scaled: the true column i is sc[i] * x_i (x_i in shared memory), its
// squared 2-norm (of the first p entries) tracked in dn[i]. A rotation that makes columns i
// and j orthogonal (the Jacobi angle of their 2 x 2 Gram matrix [[a, g], [conj g, b]],
// zeta = (b - a) / 2|g|, t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), c = 1 / sqrt(1 + t^2),
// tau = t conj(g) / |g|) becomes two multiply-adds per entry,
//   x_i <- x_i - (tau sc_j / sc_i) x_j,   x_j <- x_j + (conj(tau) sc_i / sc_j) x_i,
// with sc_i, sc_j <- c sc_i, c sc_j, and the norms follow a <- a - t|g|, b <- b + t|g|.
// A norm that fell below half its value is recomputed from the data the next time its
// column is in a pair; every column is recomputed when it is loaded. The reciprocal of every
// scale is kept beside it, so the rotation needs no division. A round runs in three phases
// between barriers: (1) one warp per pair forms <x_i, x_j>; (2) warps 0-3 (one per
// scheduler) decide and compute the rotations, one lane per pair, and list the rotated ones;
// (3) all warps apply them over (pair, 32-entry chunk) items.
constexpr int kJacThreads = 512;
constexpr int kJacWarps = kJacThreads / 32;
constexpr int kJacAuxPerCol = 64;    // shared-memory bytes per column for the bookkeeping below
constexpr int kJacAuxFixed = 256;

template <typename T>
struct JacRot {
  int32_t i, j;
  T alpha, beta;
};

template <typename T>
__device__ __forceinline__ T jac_conj(T x) {
  if constexpr (sizeof(T) == 8) return x; else return make_double2(x.x, -x.y);
}
template <typename T>
__device__ __forceinline__ T jac_scale(T x, double s) {
  if constexpr (sizeof(T) == 8) return x * s; else return make_double2(x.x * s, x.y * s);
}
// x - a y and y + b x, fused
template <typename T>
__device__ __forceinline__ void jac_apply(T& x, T& y, T a, T b) {
  if constexpr (sizeof(T) == 8) {
    const double x0 = x;
    x = fma(-a, y, x0);
    y = fma(b, x0, y);
  } else {
    const double2 x0 = x;
    x = make_double2(fma(-a.x, y.x, fma(a.y, y.y, x0.x)), fma(-a.x, y.y, fma(-a.y, y.x, x0.y)));
    y = make_double2(fma(b.x, x0.x, fma(-b.y, x0.y, y.x)), fma(b.x, x0.y, fma(b.y, x0.x, y.y)));
  }
}
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src));
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Blocked one-sided Jacobi. The q columns of the stacked matrix [W; V] (W: p x q, V: q x q
// accumulated rotations, both vector-major in global memory) are cut into 2M blocks of nb
// columns, nb chosen so that two blocks (and their bookkeeping) fit in shared memory. A sweep
// is the 2M - 1 steps of a round-robin tournament over the blocks; in each step a CTA takes
// block pairs (a, b), loads their columns into shared memory, runs all pairs between them
// there (the first step of a sweep also all pairs inside the two blocks) and writes them
// back. With M = 1 all columns stay in shared memory for every sweep. One cluster of cl
// CTAs per job; the cluster barrier separates steps, so a sweep costs 2M - 1 barriers.
// Sweeps stop after one without a rotation (bounded by kMaxSweeps; status[job] = sweeps
// used, or -1 if not converged).
struct JacobiShape {
  int nb;   // columns per block
  int M;    // block pairs per step (2M blocks)
};

template <typename T>
__host__ __device__ inline JacobiShape jacobi_shape(int p, int q, int smem_bytes, int cl) {
  const int L = p + q;
  int nb = (smem_bytes - kJacAuxFixed) / (2 * (L * (int)sizeof(T) + kJacAuxPerCol));
  if (nb < 1) nb = 1;
  if (cl == 1 && 2 * nb >= q) return JacobiShape{(q + 1) / 2, 1};
  // block pairs per step: a multiple of the cluster size, so no CTA of the cluster idles
  int M = (q + 2 * nb - 1) / (2 * nb);
  M = (M + cl - 1) / cl * cl;
  return JacobiShape{(q + 2 * M - 1) / (2 * M), M};
}

template <typename T>
__global__ void __launch_bounds__(kJacThreads) k_jacobi(const JacobiJob* __restrict__ jobs, int cl, T* __restrict__ ws,
                                                        T* __restrict__ vs, int* __restrict__ sweep_rot,
                                                        int* __restrict__ status, double tol, int smem_bytes) {
  extern __shared__ __align__(16) uint8_t jac_smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int job = blockIdx.x / cl;
  const int rank = blockIdx.x % cl;
  const JacobiJob jb = jobs[job];
  T* W = ws + jb.w_off;
  T* V = vs + jb.v_off;
  const int p = jb.p, q = jb.q, L = p + q;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ int rotated, nrot_s;
  T one, zero;
  if constexpr (sizeof(T) == 8) { one = 1.0; zero = 0.0; } else { one = make_double2(1, 0); zero = make_double2(0, 0); }
  auto barrier = [&]() {
    __threadfence();
    if (cl > 1) cluster.sync(); else __syncthreads();
  };
  // V = identity
  for (int64_t e = (int64_t)rank * kJacThreads + threadIdx.x; e < (int64_t)q * q; e += (int64_t)cl * kJacThreads)
    V[e] = (e / q == e % q) ? one : zero;
  // ||A||_F (every CTA of the cluster computes it, in the same order)
  __shared__ double red[kJacWarps];
  double f2 = 0.0;
  for (int64_t e = threadIdx.x; e < (int64_t)p * q; e += kJacThreads) f2 += abs2(W[e]);
  f2 = warp_sum(f2);
  if (lane == 0) red[warp] = f2;
  __syncthreads();
  double normA = 0.0;
  for (int w = 0; w < kJacWarps; ++w) normA += red[w];
  normA = sqrt(normA);
  // rotate while |<wi, wj>| > tol ||wi|| ||wj|| (relative orthogonality) and
  // |<wi, wj>| > tol ||A||_F max(||wi||, ||wj||) (absolute floor: pairs whose inner product
  // is at the rounding level of the whole matrix are left alone, which bounds the
  // singular-value change to about tol ||A|| absolute - the accuracy LAPACK's ?gesvd gives)
  const double tol2 = tol * tol, tola2 = (tol * normA) * (tol * normA);
  barrier();
  if (q < 2) {
    if (rank == 0 && threadIdx.x == 0) status[job] = 0;
    return;
  }
  const JacobiShape sh = jacobi_shape<T>(p, q, smem_bytes, cl);
  const int nb = sh.nb, M = sh.M, nblk = 2 * sh.M;
  const int cols_cap = M == 1 ? q : 2 * nb;
  // shared memory: columns, then scales and their reciprocals, norms, flags, pair inner
  // products, rotations
  T* X = reinterpret_cast<T*>(jac_smem);
  size_t off = (size_t)cols_cap * L * sizeof(T);
  double* sc = reinterpret_cast<double*>(jac_smem + off);
  off += (size_t)cols_cap * sizeof(double);
  double* isc = reinterpret_cast<double*>(jac_smem + off);
  off += (size_t)cols_cap * sizeof(double);
  double* dn = reinterpret_cast<double*>(jac_smem + off);
  off += (size_t)cols_cap * sizeof(double);
  int* fl = reinterpret_cast<int*>(jac_smem + off);
  off += (size_t)cols_cap * sizeof(int);
  off = (off + 15) & ~size_t(15);
  T* G = reinterpret_cast<T*>(jac_smem + off);
  off += (size_t)(cols_cap / 2 + 1) * sizeof(T);
  off = (off + 15) & ~size_t(15);
  JacRot<T>* R = reinterpret_cast<JacRot<T>*>(jac_smem + off);

  // global column c of block `blk` and its count
  auto block_cols = [&](int blk, int& c0) {
    c0 = blk * nb;
    return max(0, min(q, c0 + nb) - c0);
  };
  // columns c0 .. c0+n-1 into shared slots x0 .. (asynchronous; cp_async_wait_all + barrier after)
  auto load = [&](int c0, int n, int x0) {
    for (int c = warp; c < n; c += kJacWarps) {
      T* dst = X + (int64_t)(x0 + c) * L;
      const T* sw = W + (int64_t)(c0 + c) * p;
      const T* sv = V + (int64_t)(c0 + c) * q;
      for (int r = lane; r < p; r += 32) cp_async_elem(dst + r, sw + r);
      for (int r = lane; r < q; r += 32) cp_async_elem(dst + p + r, sv + r);
      if (lane == 0) {
        sc[x0 + c] = 1.0;
        isc[x0 + c] = 1.0;
        fl[x0 + c] = 1;
      }
    }
  };
  // true columns (scale applied) back to global memory
  auto store = [&](int c0, int n, int x0) {
    for (int c = warp; c < n; c += kJacWarps) {
      const T* src = X + (int64_t)(x0 + c) * L;
      const double s = sc[x0 + c];
      for (int r = lane; r < p; r += 32) W[(int64_t)(c0 + c) * p + r] = jac_scale(src[r], s);
      for (int r = lane; r < q; r += 32) V[(int64_t)(c0 + c) * q + r] = jac_scale(src[p + r], s);
    }
  };
  // The pairs of one round. kind 0: round r of a round-robin over lc columns (slots lcc / 2,
  // slot k pairs players k and lcc - 1 - k; a pair with the bye column lc is skipped);
  // kind 1: round r of all pairs between columns 0..na-1 and na..na+nbb-1 (slot k pairs k with
  // na + (k + r) mod max(na, nbb)).
  auto run_round = [&](int kind, int r, int n0, int n1) {
    int nslots;
    if (kind == 0) nslots = (n0 + (n0 & 1)) / 2; else nslots = max(n0, n1);
    auto slot_pair = [&](int k, int& i, int& j) -> bool {
      if (kind == 0) {
        const int lcc = n0 + (n0 & 1);
        i = rr_player(k, r, lcc);
        j = rr_player(lcc - 1 - k, r, lcc);
        if (i > j) { const int t = i; i = j; j = t; }
        return j < n0;
      }
      const int nm = max(n0, n1);
      const int jj = (k + r) % nm;
      i = k;
      j = n0 + jj;
      return k < n0 && jj < n1;
    };
    // (1) inner products (and the norms of flagged columns)
    if (threadIdx.x == 0) nrot_s = 0;
    for (int k = warp; k < nslots; k += kJacWarps) {
      int i, j;
      if (!slot_pair(k, i, j)) continue;
      const T* xi = X + (int64_t)i * L;
      const T* xj = X + (int64_t)j * L;
      const bool fi = fl[i] != 0, fj = fl[j] != 0;
      double a = 0, b = 0;
      T g;
      if constexpr (sizeof(T) == 8) {
        double gg = 0;
        if (fi || fj) {
          for (int e = lane; e < p; e += 32) {
            const double x = xi[e], y = xj[e];
            a = fma(x, x, a); b = fma(y, y, b); gg = fma(x, y, gg);
          }
        } else {
          for (int e = lane; e < p; e += 32) gg = fma(xi[e], xj[e], gg);
        }
        g = warp_sum(gg);
      } else {
        double gr = 0, gi = 0;
        if (fi || fj) {
          for (int e = lane; e < p; e += 32) {
            const double2 x = xi[e], y = xj[e];
            a += abs2(x); b += abs2(y);
            gr = fma(x.x, y.x, fma(x.y, y.y, gr));
            gi = fma(x.x, y.y, fma(-x.y, y.x, gi));
          }
        } else {
          for (int e = lane; e < p; e += 32) {
            const double2 x = xi[e], y = xj[e];
            gr = fma(x.x, y.x, fma(x.y, y.y, gr));
            gi = fma(x.x, y.y, fma(-x.y, y.x, gi));
          }
        }
        g = make_double2(warp_sum(gr), warp_sum(gi));
      }
      if (fi || fj) {
        a = warp_sum(a);
        b = warp_sum(b);
      }
      if (lane == 0) {
        const double si = sc[i], sj = sc[j];
        G[k] = jac_scale(g, si * sj);
        if (fi) { dn[i] = a * si * si; fl[i] = 0; }
        if (fj) { dn[j] = b * sj * sj; fl[j] = 0; }
      }
    }
    __syncthreads();
    // (2) rotations: warp w < 4 takes slots w, w + 4, ... one lane per slot
    if (warp < 4) {
      for (int k0 = 0; k0 < nslots; k0 += 128) {
        const int k = k0 + 4 * lane + warp;
        int i = 0, j = 0;
        bool rot = false;
        T alpha = zero, beta = zero;
        if (k < nslots && slot_pair(k, i, j)) {
          const T g = G[k];
          const double a = dn[i], b = dn[j];
          const double g2 = abs2(g);
          rot = g2 > tol2 * a * b && g2 > tola2 * fmax(a, b) && g2 > 0.0;
          if (rot) {
            const double rg = rsqrt(g2);                  // 1 / |g|
            const double gabs = g2 * rg;
            const double zeta = (b - a) * (0.5 * rg);
            const double z1 = fma(zeta, zeta, 1.0);
            const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + z1 * rsqrt(z1));
            const double t1 = fma(t, t, 1.0);
            const double c = rsqrt(t1), ic = t1 * c;       // cos, 1 / cos
            const double si = sc[i], sj = sc[j], isi = isc[i], isj = isc[j];
            T tau;
            if constexpr (sizeof(T) == 8) tau = g >= 0 ? t : -t;
            else tau = make_double2(t * g.x * rg, -t * g.y * rg);
            alpha = jac_scale(tau, sj * isi);
            beta = jac_scale(jac_conj(tau), si * isj);
            sc[i] = c * si;
            sc[j] = c * sj;
            isc[i] = ic * isi;
            isc[j] = ic * isj;
            const double an = a - t * gabs, bn = b + t * gabs;
            dn[i] = an;
            dn[j] = bn;
            if (!(an >= 0.5 * a)) fl[i] = 1;
            if (!(bn >= 0.5 * b)) fl[j] = 1;
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, rot);
        int base = 0;
        if (lane == 0 && m) base = atomicAdd(&nrot_s, __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (rot) {
          JacRot<T> e;
          e.i = i;
          e.j = j;
          e.alpha = alpha;
          e.beta = beta;
          R[base + __popc(m & ((1u << lane) - 1u))] = e;
        }
        if (lane == 0 && m) rotated = 1;
      }
    }
    __syncthreads();
    // (3) updates over (rotation, 32-entry chunk) items
    const int nrot = nrot_s;
    const int nch = (L + 31) >> 5;
    for (int it = warp; it < nrot * nch; it += kJacWarps) {
      const int k = it / nch, e = (it - k * nch) * 32 + lane;
      if (e < L) {
        const JacRot<T> rr = R[k];
        T* xi = X + (int64_t)rr.i * L + e;
        T* xj = X + (int64_t)rr.j * L + e;
        T x = *xi, y = *xj;
        jac_apply(x, y, rr.alpha, rr.beta);
        *xi = x;
        *xj = y;
      }
    }
    __syncthreads();
  };

  int sweep = 0;
  if (M == 1) {
    // every column in shared memory for all sweeps (one CTA: cl == 1 for these jobs)
    load(0, q, 0);
    cp_async_wait_all();
    __syncthreads();
    const int lcc = q + (q & 1);
    for (; sweep < kMaxSweeps; ++sweep) {
      if (threadIdx.x == 0) rotated = 0;
      __syncthreads();
      for (int r = 0; r < lcc - 1; ++r) run_round(0, r, q, 0);
      const int any = rotated;
      // fold the scales into the columns; norms are recomputed in the next sweep
      for (int idx = threadIdx.x; idx < q * L; idx += kJacThreads) X[idx] = jac_scale(X[idx], sc[idx / L]);
      __syncthreads();
      for (int c = threadIdx.x; c < q; c += kJacThreads) {
        sc[c] = 1.0;
        isc[c] = 1.0;
        fl[c] = 1;
      }
      __syncthreads();
      if (!any) break;
    }
    store(0, q, 0);
    barrier();
  } else {
    for (; sweep < kMaxSweeps; ++sweep) {
      if (threadIdx.x == 0) rotated = 0;
      __syncthreads();
      for (int st = 0; st < nblk - 1; ++st) {
        for (int k = rank; k < M; k += cl) {
          const int ba = rr_player(k, st, nblk), bb = rr_player(nblk - 1 - k, st, nblk);
          int ca, cb;
          const int na = block_cols(ba, ca), nbb = block_cols(bb, cb);
          if (na + nbb < 2) continue;
          load(ca, na, 0);
          load(cb, nbb, na);
          cp_async_wait_all();
          __syncthreads();
          if (st == 0) {
            // the first step of a sweep also orthogonalises the columns inside each block
            const int lc = na + nbb, lcc = lc + (lc & 1);
            for (int r = 0; r < lcc - 1; ++r) run_round(0, r, lc, 0);
          } else {
            const int nm = max(na, nbb);
            for (int r = 0; r < nm; ++r) run_round(1, r, na, nbb);
          }
          store(ca, na, 0);
          store(cb, nbb, na);
          __syncthreads();
        }
        barrier();
      }
      if (threadIdx.x == 0 && rotated) atomicAdd(&sweep_rot[job * kMaxSweeps + sweep], 1);
      barrier();
      const int any = *((volatile int*)&sweep_rot[job * kMaxSweeps + sweep]);
      if (any == 0) break;
    }
  }
  if (rank == 0 && threadIdx.x == 0) status[job] = sweep < kMaxSweeps ? sweep + 1 : -1;
}

// Singular values = vector norms, sorted descending; left vectors normalised in place.
// order[job][k] = vector index of the k-th largest singular value, svs[job][k] its value.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_svd_finish(const JacobiJob* __restrict__ jobs, T* __restrict__ ws,
                                                         double* __restrict__ sv, const int64_t* __restrict__ sv_off,
                                                         int32_t* __restrict__ order, double* __restrict__ svs) {
  const JacobiJob jb = jobs[blockIdx.x];
  T* W = ws + jb.w_off;
  const int p = jb.p, q = jb.q;
  double* s = sv + sv_off[blockIdx.x];
  int32_t* ord = order + sv_off[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int v = warp; v < q; v += kWarps) {
    double a = 0;
    for (int e = lane; e < p; e += 32) a += abs2(W[(int64_t)v * p + e]);
    a = sqrt(warp_sum(a));
    if (lane == 0) s[v] = a;
    const double inv = a > 0 ? 1.0 / a : 0.0;
    for (int e = lane; e < p; e += 32) {
      T x = W[(int64_t)v * p + e];
      if constexpr (sizeof(T) == 8) x *= inv; else { x.x *= inv; x.y *= inv; }
      W[(int64_t)v * p + e] = x;
    }
  }
  __syncthreads();
  // rank sort (descending, ties by index) - q <= a few thousand
  for (int v = threadIdx.x; v < q; v += kThreads) {
    const double x = s[v];
    int rk = 0;
    for (int u = 0; u < q; ++u) {
      const double y = s[u];
      rk += (y > x) || (y == x && u < v);
    }
    ord[rk] = v;
    svs[sv_off[blockIdx.x] + rk] = x;
  }
}

// ---- truncation on the device, the reference's rule (tensor_manipulation/ten_decomp/
// ten_svd.h:281-372): all groups' nonzero singular values in descending order (ties by group,
// then rank), keep Dmin of them, then one more while the kept weight sum s^2 is <= (1 - eps)
// of the total and the count stays <= Dmax. The order comes from a stable radix sort of the
// entries - held group by group in rank order - keyed by the complement of the value's bits
// (for values >= 0 the bit patterns order like the values, so ascending keys are descending
// values, equal values keep their group-then-rank order, zeros sort last).
struct SvCut {
  int64_t kept;    // kept dimension D
  double err;      // truncation error 1 - kept weight / total weight (0 when nothing is cut)
  int32_t nnz;     // nonzero singular values over all groups
  int32_t pad;
};

__global__ void __launch_bounds__(256) k_sv_keys(const double* __restrict__ svs, int64_t n, uint64_t* __restrict__ key,
                                                 int32_t* __restrict__ idx, SvCut* __restrict__ cut) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const double v = svs[e];
    key[e] = v == 0.0 ? ~0ull : ~(uint64_t)__double_as_longlong(v);
    idx[e] = (int32_t)e;
    if (v != 0.0) atomicAdd(&cut->nnz, 1);
  }
}

// sorted entries -> their values and groups (the group: the last one starting at or before e)
__global__ void __launch_bounds__(256) k_sv_sorted(const double* __restrict__ svs, const int64_t* __restrict__ sv_off,
                                                   int ng, const int32_t* __restrict__ idx, int64_t n,
                                                   double* __restrict__ sorted_v, int32_t* __restrict__ sorted_g) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = idx[j];
    int lo = 0, hi = ng - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sv_off[mid] <= e) lo = mid; else hi = mid - 1;
    }
    sorted_v[j] = svs[e];
    sorted_g[j] = lo;
  }
}

// One CTA. The weights s^2 are summed in one thread in the sorted order (the order the
// reference sums in; each square is rounded before its addition), chunk by chunk through
// shared memory, keeping every prefix W(k) = weight of the first k values. The reference's
// loop (keep Dmin, add one while W(kept) <= (1 - eps) W(total) and kept < min(total, Dmax))
// ends at the smallest k in [Dmin, min(total, Dmax)) with W(k) > (1 - eps) W(total), else at
// min(total, Dmax): the threads search for it. Then the kept entries are counted per group.
constexpr int kCutChunk = 2048;

__global__ void __launch_bounds__(256) k_sv_cut(const double* __restrict__ sorted_v, const int32_t* __restrict__ sorted_g,
                                                double* __restrict__ prefix, double trunc, int64_t dmin, int64_t dmax,
                                                int ng, SvCut* __restrict__ cut, int* __restrict__ kcnt) {
  __shared__ double buf[kCutChunk];
  __shared__ unsigned long long kept_s;
  __shared__ double target_s;
  const int64_t total = cut->nnz;
  const bool cuts = total > dmin;
  const int64_t lim = cuts ? (total < dmax ? total : dmax) : total;
  if (threadIdx.x == 0) kept_s = (unsigned long long)lim;
  if (cuts) {
    double run = 0;   // thread 0's running sum
    for (int64_t base = 0; base < total; base += kCutChunk) {
      const int n = (int)(total - base < kCutChunk ? total - base : kCutChunk);
      for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = __dmul_rn(sorted_v[base + i], sorted_v[base + i]);
      __syncthreads();
      if (threadIdx.x == 0) {
#pragma unroll 16
        for (int i = 0; i < n; ++i) {
          run = __dadd_rn(run, buf[i]);
          buf[i] = run;
        }
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) prefix[base + i] = buf[i];
      __syncthreads();
    }
    if (threadIdx.x == 0) target_s = __dmul_rn(run, __dsub_rn(1.0, trunc));
    __syncthreads();   // also orders the prefix stores before the reads below
    for (int64_t k = dmin + threadIdx.x; k < lim; k += blockDim.x) {
      const double w = k == 0 ? 0.0 : prefix[k - 1];
      if (w > target_s) atomicMin(&kept_s, (unsigned long long)k);
    }
  }
  __syncthreads();
  const int64_t kept = (int64_t)kept_s;
  if (threadIdx.x == 0) {
    double err = 0;
    if (cuts) {
      const double w = kept == 0 ? 0.0 : prefix[kept - 1];
      const double x = __dsub_rn(1.0, __ddiv_rn(w, prefix[total - 1]));
      err = x > 0 ? x : 0;
    }
    cut->kept = kept;
    cut->err = err;
  }
  for (int64_t j = threadIdx.x; j < kept; j += blockDim.x) {
    const int g = sorted_g[j];
    if (g >= 0 && g < ng) atomicAdd(kcnt + g, 1);
  }
}

// S blocks: the kept values of a group on the diagonal of its (zero-filled) kd x kd block
struct SvDiag {
  int64_t dst_off, src_off;
  int32_t kd, pad;
};

__global__ void k_sv_diag(const SvDiag* __restrict__ d, int nd, const double* __restrict__ svs, double* __restrict__ S) {
  for (int b = blockIdx.x; b < nd; b += gridDim.x) {
    const SvDiag x = d[b];
    for (int i = threadIdx.x; i < x.kd; i += blockDim.x) S[x.dst_off + (int64_t)i * x.kd + i] = svs[x.src_off + i];
  }
}

// ------------------------------------------------------------------ Householder QR
struct QrJob {
  int64_t a_off;     // m x n column-major, reflectors below the diagonal after the factorisation
  int64_t tau_off;
  int64_t q_off;     // m x k column-major Q
  int32_t m, n;
  int64_t t_off;     // triangular factors of the panels' block reflectors, 32 x 32 each
};

template <typename T>
__device__ __forceinline__ T mk(double re, double im);
template <>
__device__ __forceinline__ double mk<double>(double re, double) { return re; }
template <>
__device__ __forceinline__ double2 mk<double2>(double re, double im) { return make_double2(re, im); }

__device__ __forceinline__ double re_of(double x) { return x; }
__device__ __forceinline__ double re_of(double2 x) { return x.x; }
__device__ __forceinline__ double im_of(double) { return 0.0; }
__device__ __forceinline__ double im_of(double2 x) { return x.y; }


template <typename T>
__device__ __forceinline__ T conjT(T x) {
  if constexpr (sizeof(T) == 8) return x; else return make_double2(x.x, -x.y);
}
template <typename T>
__device__ __forceinline__ T mulT(T a, T b) {
  if constexpr (sizeof(T) == 8) return a * b; else return cmul(a, b);
}
template <typename T>
__device__ __forceinline__ T subT(T a, T b) {
  if constexpr (sizeof(T) == 8) return a - b; else return make_double2(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ T scaleT(T a, double s) {
  if constexpr (sizeof(T) == 8) return a * s; else return make_double2(a.x * s, a.y * s);
}

// ------------------------------------------------------------------ blocked Householder QR
// LAPACK's Householder QR (?geqrf / ?ungqr) restated in panels of kQrNb columns. Reflector
// j: beta = -sign(Re alpha) ||(alpha, x)||, tau = (beta - alpha) / beta, v = x / (alpha -
// beta), R(j, j) = beta (LAPACK's ?larfg convention, so Q and R compare directly with
// ?geqrf + ?orgqr). A panel is factorised by one CTA column by column (reflectors applied
// inside the panel only), which then forms the triangular factor T of the panel's block
// reflector H = H_j0 ... H_j0+nb-1 = I - V T V^H (?larft, forward, columnwise). The rest of
// the matrix is updated by many CTAs at once, one per 32-column tile of every group:
// A_tile -= V T^H (V^H A_tile). Q is formed backwards over the panels the same way, with
// Q_tile -= V T (V^H Q_tile) on the columns j0 .. k-1 of Q = I(:, 0:k). A large group thus
// spreads its O(m n^2) work over as many SMs as it has column tiles, instead of one.
constexpr int kQrNb = 32;   // panel width
// the panel kernel's CTA: 32 warps, so each of a panel's columns has a warp for the in-panel
// updates and the column norms reduce over 1024 threads
constexpr int kPanelThreads = 1024;
constexpr int kPanelWarps = kPanelThreads / 32;
// dynamic shared memory for a panel held on chip (beside the kernel's static 17 / 34 KB)
template <typename T>
constexpr int qr_panel_smem() { return sizeof(T) == 8 ? 200 * 1024 : 184 * 1024; }
// rows per shared-memory chunk of the update kernel (its three 32-column buffers stay within
// the 48 KB of static shared memory)
template <typename T>
constexpr int qr_rows_per_chunk() { return sizeof(T) == 8 ? 64 : 16; }

// One work item of the block-reflector updates: rows [r0, r1) of the 32-column tile that
// starts at column c0. The row chunks of one tile are consecutive items, the first at index
// `first`, `nchunks` of them; they share the tile's W = V^H X through partial sums.
constexpr int kQrRowChunk = 128;
struct QrTile {
  int32_t job, c0;
  int32_t r0, r1;
  int32_t first, nchunks;
};

template <typename T>
__device__ __forceinline__ T addT(T a, T b) {
  if constexpr (sizeof(T) == 8) return a + b; else return make_double2(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ T fmaT(T a, T b, T c) {   // a b + c
  if constexpr (sizeof(T) == 8) return fma(a, b, c);
  else return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
template <typename T>
__device__ __forceinline__ T fma_conj(T a, T b, T c) {   // conj(a) b + c
  if constexpr (sizeof(T) == 8) return fma(a, b, c);
  else return make_double2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
template <typename T>
__device__ __forceinline__ T zeroT() {
  if constexpr (sizeof(T) == 8) return 0.0; else return make_double2(0.0, 0.0);
}

// Element (r, l) of panel j0's reflector block V: 1 on its diagonal, the stored reflector
// below it, 0 above.
template <typename T>
__device__ __forceinline__ T v_elem(const T* __restrict__ A, int m, int j0, int nbe, int r, int l) {
  if (l >= nbe || r >= m) return zeroT<T>();
  const int d = j0 + l;
  if (r == d) return mk<T>(1.0, 0.0);
  return r > d ? A[(int64_t)d * m + r] : zeroT<T>();
}

// The panel (rows j0 .. m-1 of its 32 columns) is worked on in shared memory when it fits
// (panel_rows_cap rows; the launch provides the space), else in place in global memory.
template <typename T>
__global__ void __launch_bounds__(kPanelThreads) k_qr_panel(const QrJob* __restrict__ jobs, int j0, T* __restrict__ as,
                                                       T* __restrict__ taus, T* __restrict__ tfac,
                                                       int panel_rows_cap) {
  extern __shared__ __align__(16) uint8_t panel_smem[];
  const QrJob jb = jobs[blockIdx.x];
  const int m = jb.m, n = jb.n, k = min(m, n);
  if (j0 >= k) return;
  const int nbe = min(kQrNb, k - j0);
  T* A = as + jb.a_off;
  T* tau = taus + jb.tau_off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pr = m - j0;                       // panel rows
  const bool in_smem = pr <= panel_rows_cap;
  T* sp = reinterpret_cast<T*>(panel_smem);
  // column c of the panel, indexed by (row - j0)
  auto pcol = [&](int c) -> T* { return in_smem ? sp + (int64_t)c * pr : A + (int64_t)(j0 + c) * m + j0; };
  if (in_smem) {
    for (int64_t e = threadIdx.x; e < (int64_t)nbe * pr; e += kPanelThreads) {
      const int c = (int)(e / pr), r = (int)(e - (int64_t)c * pr);
      sp[e] = A[(int64_t)(j0 + c) * m + j0 + r];
    }
    __syncthreads();
  }
  __shared__ double red[kPanelWarps];
  __shared__ T s_tau, s_scale;
  __shared__ T sY[kQrNb][kQrNb + 1], sT[kQrNb][kQrNb + 1];
  for (int jc = 0; jc < nbe; ++jc) {
    const int j = j0 + jc;
    T* col = pcol(jc);
    double part = 0;
    for (int r = jc + 1 + threadIdx.x; r < pr; r += kPanelThreads) part += abs2(col[r]);
    part = warp_sum(part);
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      double xn2 = 0;
      for (int w = 0; w < kPanelWarps; ++w) xn2 += red[w];
      const T alpha = col[jc];
      const double ar = re_of(alpha), ai = im_of(alpha);
      if (xn2 == 0.0 && ai == 0.0) {
        s_tau = mk<T>(0.0, 0.0);
        s_scale = mk<T>(0.0, 0.0);
      } else {
        const double nrm = sqrt(ar * ar + ai * ai + xn2);
        const double beta = ar >= 0 ? -nrm : nrm;
        s_tau = mk<T>((beta - ar) / beta, -ai / beta);
        const double dr = ar - beta, di = ai;
        const double den = dr * dr + di * di;
        s_scale = mk<T>(dr / den, -di / den);
        col[jc] = mk<T>(beta, 0.0);
      }
      tau[j] = s_tau;
    }
    __syncthreads();
    const T sc = s_scale;
    for (int r = jc + 1 + threadIdx.x; r < pr; r += kPanelThreads) col[r] = mulT(col[r], sc);
    __syncthreads();
    // H_j^H on the panel's later columns only (the rest waits for the block update)
    const T tconj = conjT(s_tau);
    if (re_of(s_tau) != 0.0 || im_of(s_tau) != 0.0) {
      for (int c = jc + 1 + warp; c < nbe; c += kPanelWarps) {
        T* ac = pcol(c);
        double wr = 0, wi = 0;
#pragma unroll 4
        for (int r = jc + lane; r < pr; r += 32) {
          const T v = (r == jc) ? mk<T>(1.0, 0.0) : col[r];
          const T prod = mulT(conjT(v), ac[r]);
          wr += re_of(prod);
          wi += im_of(prod);
        }
        wr = warp_sum(wr);
        wi = warp_sum(wi);
        const T w = mulT(tconj, mk<T>(wr, wi));
#pragma unroll 4
        for (int r = jc + lane; r < pr; r += 32) {
          const T v = (r == jc) ? mk<T>(1.0, 0.0) : col[r];
          ac[r] = subT(ac[r], mulT(v, w));
        }
      }
    }
    __syncthreads();
  }
  // T: y(l, i) = v_l^H v_i for l < i (v_i starts at panel row i with a 1)
  for (int i = 1; i < nbe; ++i) {
    const T* vi = pcol(i);
    for (int l = warp; l < i; l += kPanelWarps) {
      const T* vl = pcol(l);
      T acc = zeroT<T>();
      for (int r = i + 1 + lane; r < pr; r += 32) acc = fma_conj(vl[r], vi[r], acc);
      double ar = warp_sum(re_of(acc)), ai = warp_sum(im_of(acc));
      if (lane == 0) sY[l][i] = addT(mk<T>(ar, ai), conjT(vl[i]));
    }
  }
  __syncthreads();
  // column by column: T(i, i) = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) y(0:i, i)
  for (int i = 0; i < nbe; ++i) {
    const T ti = tau[j0 + i];
    if (threadIdx.x < i) {
      const int l = threadIdx.x;
      T z = zeroT<T>();
      for (int lp = l; lp < i; ++lp) z = fmaT(sT[l][lp], sY[lp][i], z);
      sT[l][i] = mulT(mk<T>(-re_of(ti), -im_of(ti)), z);
    } else if ((int)threadIdx.x == i) {
      sT[i][i] = ti;
    }
    __syncthreads();
  }
  T* Tp = tfac + jb.t_off + (int64_t)(j0 / kQrNb) * kQrNb * kQrNb;
  for (int e = threadIdx.x; e < kQrNb * kQrNb; e += kPanelThreads) {
    const int c = e / kQrNb, r = e % kQrNb;
    Tp[e] = (r < nbe && c < nbe && r <= c) ? sT[r][c] : zeroT<T>();
  }
  if (in_smem) {
    for (int64_t e = threadIdx.x; e < (int64_t)nbe * pr; e += kPanelThreads) {
      const int c = (int)(e / pr), r = (int)(e - (int64_t)c * pr);
      A[(int64_t)(j0 + c) * m + j0 + r] = sp[e];
    }
  }
}

// The block-reflector update X_tile -= V op(T) (V^H X_tile), op(T) = T^H for the trailing
// columns of A (FORM_Q false, X = A) and T for the backward formation of Q (FORM_Q true,
// X = Q), in two launches over (tile, row chunk) items so a tall group spreads over many
// CTAs: k_qr_wpart writes each item's partial W = V^H X over its rows, k_qr_apply sums the
// partials of its tile in chunk order (deterministic), forms op(T) W and updates its rows.
// Rows are streamed through shared memory kQrRc at a time.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_qr_wpart(const QrJob* __restrict__ jobs,
                                                       const QrTile* __restrict__ tiles, int j0, bool form_q,
                                                       const T* __restrict__ as, const T* __restrict__ xs,
                                                       T* __restrict__ part) {
  const QrTile tl = tiles[blockIdx.x];
  const QrJob jb = jobs[tl.job];
  const int m = jb.m, n = jb.n, k = min(m, n);
  const int nbe = min(kQrNb, k - j0);
  const T* A = as + jb.a_off;
  const T* X = form_q ? xs + jb.q_off : xs + jb.a_off;
  const int ncols = form_q ? k : n;
  const int c0 = tl.c0, nc = min(32, ncols - c0);
  constexpr int kQrRc = qr_rows_per_chunk<T>();
  __shared__ T sV[kQrRc][kQrNb + 1], sX[kQrRc][33];
  const int l = threadIdx.x & 31, cg = threadIdx.x >> 5;   // W entries (l, cg + 8 u)
  T acc[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) acc[u] = zeroT<T>();
  for (int r0 = tl.r0; r0 < tl.r1; r0 += kQrRc) {
    for (int e = threadIdx.x; e < kQrRc * kQrNb; e += kThreads) {
      const int rr = e % kQrRc, ll = e / kQrRc;
      sV[rr][ll] = r0 + rr < tl.r1 ? v_elem(A, m, j0, nbe, r0 + rr, ll) : zeroT<T>();
    }
    for (int e = threadIdx.x; e < kQrRc * 32; e += kThreads) {
      const int rr = e % kQrRc, c = e / kQrRc;
      sX[rr][c] = (r0 + rr < tl.r1 && c < nc) ? X[(int64_t)(c0 + c) * m + r0 + rr] : zeroT<T>();
    }
    __syncthreads();
    const int rn = min(kQrRc, tl.r1 - r0);
    for (int rr = 0; rr < rn; ++rr) {
      const T v = sV[rr][l];
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[u] = fma_conj(v, sX[rr][cg + 8 * u], acc[u]);
    }
    __syncthreads();
  }
  T* pw = part + (int64_t)blockIdx.x * kQrNb * 32;
#pragma unroll
  for (int u = 0; u < 4; ++u) pw[l * 32 + cg + 8 * u] = acc[u];
}

template <typename T, bool FORM_Q>
__global__ void __launch_bounds__(kThreads) k_qr_apply(const QrJob* __restrict__ jobs,
                                                       const QrTile* __restrict__ tiles, int j0,
                                                       const T* __restrict__ as, const T* __restrict__ tfac,
                                                       const T* __restrict__ part, T* __restrict__ xs) {
  const QrTile tl = tiles[blockIdx.x];
  const QrJob jb = jobs[tl.job];
  const int m = jb.m, n = jb.n, k = min(m, n);
  const int nbe = min(kQrNb, k - j0);
  const T* A = as + jb.a_off;
  T* X = FORM_Q ? xs + jb.q_off : xs + jb.a_off;
  const int ncols = FORM_Q ? k : n;
  const int c0 = tl.c0, nc = min(32, ncols - c0);
  constexpr int kQrRc = qr_rows_per_chunk<T>();
  __shared__ T sV[kQrRc][kQrNb + 1], sW[kQrNb][33];
  // T(r, c) of this panel, column-major 32 x 32 (read through the cache)
  const T* Tp = tfac + jb.t_off + (int64_t)(j0 / kQrNb) * kQrNb * kQrNb;
  const int l = threadIdx.x & 31, cg = threadIdx.x >> 5;
  // W of the tile: its chunks' partials summed in chunk order
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    T w = zeroT<T>();
    for (int ch = 0; ch < tl.nchunks; ++ch) w = addT(w, part[((int64_t)(tl.first + ch) * kQrNb + l) * 32 + cg + 8 * u]);
    sW[l][cg + 8 * u] = w;
  }
  __syncthreads();
  // W2 = T^H W (trailing update) or T W (Q), T upper triangular
  T acc[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int c = cg + 8 * u;
    T z = zeroT<T>();
    if (FORM_Q) {
      for (int lp = l; lp < kQrNb; ++lp) z = fmaT(__ldg(Tp + lp * kQrNb + l), sW[lp][c], z);
    } else {
      for (int lp = 0; lp <= l; ++lp) z = fma_conj(__ldg(Tp + l * kQrNb + lp), sW[lp][c], z);
    }
    acc[u] = z;
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u) sW[l][cg + 8 * u] = acc[u];
  __syncthreads();
  // X -= V W2 over this item's rows
  const int c = threadIdx.x & 31, rg = threadIdx.x >> 5;
  for (int r0 = tl.r0; r0 < tl.r1; r0 += kQrRc) {
    for (int e = threadIdx.x; e < kQrRc * kQrNb; e += kThreads) {
      const int rr = e % kQrRc, ll = e / kQrRc;
      sV[rr][ll] = r0 + rr < tl.r1 ? v_elem(A, m, j0, nbe, r0 + rr, ll) : zeroT<T>();
    }
    __syncthreads();
    if (c < nc) {
      for (int rr = rg; rr < kQrRc; rr += kThreads / 32) {
        const int r = r0 + rr;
        if (r >= tl.r1) break;
        T z = zeroT<T>();
#pragma unroll 8
        for (int ll = 0; ll < kQrNb; ++ll) z = fmaT(sV[rr][ll], sW[ll][c], z);
        T* x = X + (int64_t)(c0 + c) * m + r;
        *x = subT(*x, z);
      }
    }
    __syncthreads();
  }
}

// Q = I(:, 0:k) for every job (the start of the backward formation).
template <typename T>
__global__ void k_qr_qinit(const QrJob* __restrict__ jobs, int njobs, T* __restrict__ qs) {
  for (int g = blockIdx.y; g < njobs; g += gridDim.y) {
    const QrJob jb = jobs[g];
    const int k = min(jb.m, jb.n);
    const int64_t tot = (int64_t)jb.m * k;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
      const int64_t c = e / jb.m, r = e % jb.m;
      qs[jb.q_off + e] = mk<T>(r == c ? 1.0 : 0.0, 0.0);
    }
  }
}

// ------------------------------------------------------------------ host side
struct Group {
  std::vector<int32_t> lflux, rflux, mid;
  int64_t rows = 0, cols = 0;
  std::vector<std::vector<int64_t>> rkeys, ckeys;
  std::vector<int64_t> roff, rdim, coff, cdim;
  std::vector<int64_t> eblk, erow, ecol;
};

std::vector<int32_t> divergence(const Meta& t) {
  std::vector<int32_t> d(t.ncomp, 0);
  if (t.nblk == 0) return d;
  for (int l = 0; l < t.rank; ++l)
    for (int k = 0; k < t.ncomp; ++k) {
      const int32_t q = t.qns[l][t.coords[l] * t.ncomp + k];
      d[k] += t.dirs[l] == QLTG_OUT ? q : -q;
    }
  return d;
}

std::vector<Group> group_blocks(const Meta& t, int ldims, const std::vector<int32_t>& lqndiv) {
  std::vector<Group> gs;
  const auto div = divergence(t);
  const int r = t.rank, nc = t.ncomp;
  for (int64_t b = 0; b < t.nblk; ++b) {
    std::vector<int32_t> lf(nc, 0), rf(nc), mid(nc);
    for (int l = 0; l < ldims; ++l)
      for (int k = 0; k < nc; ++k) {
        const int32_t q = t.qns[l][t.coords[b * r + l] * nc + k];
        lf[k] += t.dirs[l] == QLTG_OUT ? q : -q;
      }
    for (int k = 0; k < nc; ++k) { rf[k] = div[k] - lf[k]; mid[k] = lqndiv[k] - lf[k]; }
    int64_t m = 1, n = 1;
    for (int l = 0; l < ldims; ++l) m *= t.dim(b, l);
    for (int l = ldims; l < r; ++l) n *= t.dim(b, l);
    size_t g = 0;
    while (g < gs.size() && !(gs[g].lflux == lf && gs[g].rflux == rf)) ++g;
    if (g == gs.size()) { gs.emplace_back(); gs[g].lflux = lf; gs[g].rflux = rf; gs[g].mid = mid; }
    Group& G = gs[g];
    std::vector<int64_t> lk(t.coords.begin() + b * r, t.coords.begin() + b * r + ldims);
    std::vector<int64_t> rk(t.coords.begin() + b * r + ldims, t.coords.begin() + b * r + r);
    size_t i = 0;
    while (i < G.rkeys.size() && G.rkeys[i] != lk) ++i;
    if (i == G.rkeys.size()) { G.rkeys.push_back(lk); G.roff.push_back(G.rows); G.rdim.push_back(m); G.rows += m; }
    size_t j = 0;
    while (j < G.ckeys.size() && G.ckeys[j] != rk) ++j;
    if (j == G.ckeys.size()) { G.ckeys.push_back(rk); G.coff.push_back(G.cols); G.cdim.push_back(n); G.cols += n; }
    G.eblk.push_back(b); G.erow.push_back((int64_t)i); G.ecol.push_back((int64_t)j);
  }
  return gs;
}

Meta leg_subset(const Meta& t, int from, int to) {
  Meta m;
  m.dtype = t.dtype;
  m.ncomp = t.ncomp;
  m.parity_comp = t.parity_comp;
  for (int l = from; l < to; ++l) { m.dirs.push_back(t.dirs[l]); m.qns.push_back(t.qns[l]); m.dims.push_back(t.dims[l]); }
  m.rank = to - from;
  return m;
}

void sort_blocks(Meta& t, std::vector<std::vector<int64_t>>& coords) {
  std::sort(coords.begin(), coords.end(), [&](const std::vector<int64_t>& x, const std::vector<int64_t>& y) {
    return t.blk_idx(x.data()) < t.blk_idx(y.data());
  });
  t.coords.clear();
  for (auto& c : coords) t.coords.insert(t.coords.end(), c.begin(), c.end());
  t.nblk = (int64_t)coords.size();
  t.refresh_offsets();
}

int64_t block_of(const Meta& t, const std::vector<int64_t>& c) {
  int64_t lo = 0, hi = t.nblk;
  const uint64_t key = t.blk_idx(c.data());
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (t.blk_idx(&t.coords[mid * t.rank]) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)current_sm_count() * 16)); }

// Blocked Householder QR of every job (A in place, tau, Q): per panel one factorisation
// launch (one CTA per job) and one trailing-update launch over all jobs' column tiles; then
// Q = I and one update launch per panel, last panel first. The jobs' t_off are assigned here.
struct QrBuffers {
  DevBuf jobs, tiles, tfac, part;
};
template <typename T>
void launch_blocked_qr(std::vector<QrJob>& jobs, T* A, T* tau, T* Q, cudaStream_t s, QrBuffers& keep) {
  const int ng = (int)jobs.size();
  if (!ng) return;
  int kmax = 0;
  int64_t toff = 0;
  for (auto& j : jobs) {
    const int k = std::min(j.m, j.n);
    kmax = std::max(kmax, k);
    j.t_off = toff;
    toff += (int64_t)((k + kQrNb - 1) / kQrNb) * kQrNb * kQrNb;
  }
  const int np = (kmax + kQrNb - 1) / kQrNb;
  // tiles of panel p: trailing columns of A (p in [0, np)), then columns j0 .. k-1 of Q
  std::vector<QrTile> tiles;
  std::vector<int64_t> trail_begin(np + 1), q_begin(np + 1);
  // one item per (tile, chunk of kQrRowChunk rows from j0); item indices are relative to the
  // launch that runs them (the partial sums of a launch start at 0)
  int64_t max_items = 1;
  auto add_tile = [&](int g, int c0, int j0, int64_t begin) {
    const int m = jobs[g].m;
    const int nch = (m - j0 + kQrRowChunk - 1) / kQrRowChunk;
    const int first = (int)((int64_t)tiles.size() - begin);
    for (int ch = 0; ch < nch; ++ch)
      tiles.push_back(QrTile{g, c0, j0 + ch * kQrRowChunk, std::min(m, j0 + (ch + 1) * kQrRowChunk), first, nch});
  };
  for (int p = 0; p < np; ++p) {
    trail_begin[p] = (int64_t)tiles.size();
    const int j0 = p * kQrNb;
    for (int g = 0; g < ng; ++g) {
      const int k = std::min(jobs[g].m, jobs[g].n);
      if (j0 >= k) continue;
      for (int c0 = j0 + std::min(kQrNb, k - j0); c0 < jobs[g].n; c0 += 32) add_tile(g, c0, j0, trail_begin[p]);
    }
    max_items = std::max<int64_t>(max_items, (int64_t)tiles.size() - trail_begin[p]);
  }
  trail_begin[np] = (int64_t)tiles.size();
  for (int p = 0; p < np; ++p) {
    q_begin[p] = (int64_t)tiles.size();
    const int j0 = p * kQrNb;
    for (int g = 0; g < ng; ++g) {
      const int k = std::min(jobs[g].m, jobs[g].n);
      if (j0 >= k) continue;
      for (int c0 = j0; c0 < k; c0 += 32) add_tile(g, c0, j0, q_begin[p]);
    }
    max_items = std::max<int64_t>(max_items, (int64_t)tiles.size() - q_begin[p]);
  }
  q_begin[np] = (int64_t)tiles.size();
  QLTG_CHECK(tiles.size() < ((size_t)1 << 31), QLTG_ERR_UNSUPPORTED, "too many QR work items");
  keep.jobs = upload(jobs, s);
  keep.tiles = upload(tiles.empty() ? std::vector<QrTile>{QrTile{0, 0}} : tiles, s);
  keep.tfac.alloc(std::max<int64_t>(1, toff) * sizeof(T));
  keep.part.alloc(max_items * kQrNb * 32 * sizeof(T));
  T* pw = keep.part.as<T>();
  {
    static std::mutex mu;
    static bool done[2][64] = {};
    int dev = 0;
    QLTG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !done[sizeof(T) == 16][dev]) {
      QLTG_CUDA(cudaFuncSetAttribute(k_qr_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, qr_panel_smem<T>()));
      if (dev >= 0 && dev < 64) done[sizeof(T) == 16][dev] = true;
    }
  }
  const QrJob* dj = keep.jobs.as<QrJob>();
  const QrTile* dt = keep.tiles.as<QrTile>();
  T* tf = keep.tfac.as<T>();
  for (int p = 0; p < np; ++p) {
    const int j0 = p * kQrNb;
    // the panel in shared memory when the tallest active one fits
    int rows_max = 0;
    for (auto& j : jobs)
      if (j0 < std::min(j.m, j.n)) rows_max = std::max(rows_max, j.m - j0);
    const int cap = qr_panel_smem<T>() / (kQrNb * (int)sizeof(T));
    const size_t smem = rows_max <= cap ? (size_t)rows_max * kQrNb * sizeof(T) : 0;
    k_qr_panel<T><<<ng, kPanelThreads, smem, s>>>(dj, j0, A, tau, tf, smem ? rows_max : 0);
    const int64_t nt = trail_begin[p + 1] - trail_begin[p];
    if (nt) {
      k_qr_wpart<T><<<(unsigned)nt, kThreads, 0, s>>>(dj, dt + trail_begin[p], j0, false, A, A, pw);
      k_qr_apply<T, false><<<(unsigned)nt, kThreads, 0, s>>>(dj, dt + trail_begin[p], j0, A, tf, pw, A);
    }
  }
  const int64_t total_q = std::accumulate(jobs.begin(), jobs.end(), (int64_t)0, [](int64_t a, const QrJob& j) {
    return std::max<int64_t>(a, (int64_t)j.m * std::min(j.m, j.n));
  });
  k_qr_qinit<T><<<dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>((total_q + 255) / 256, 64)),
                       (unsigned)std::min(ng, 1024)), 256, 0, s>>>(dj, ng, Q);
  for (int p = np - 1; p >= 0; --p) {
    const int64_t nt = q_begin[p + 1] - q_begin[p];
    if (nt) {
      k_qr_wpart<T><<<(unsigned)nt, kThreads, 0, s>>>(dj, dt + q_begin[p], p * kQrNb, true, A, Q, pw);
      k_qr_apply<T, true><<<(unsigned)nt, kThreads, 0, s>>>(dj, dt + q_begin[p], p * kQrNb, A, tf, pw, Q);
    }
  }
  QLTG_CUDA(cudaGetLastError());
}

template <typename T>
void launch_gather(const std::vector<CopyDesc>& d, int64_t total, const void* src, void* dst, cudaStream_t s,
                   DevBuf& keep) {
  if (total == 0) return;
  keep = upload(d, s);
  k_gather<T><<<grid_for(total), 256, 0, s>>>(keep.as<CopyDesc>(), (int)d.size(), total, static_cast<const T*>(src),
                                               static_cast<T*>(dst));
  QLTG_CUDA(cudaGetLastError());
}

template <typename T>
void launch_scatter(const std::vector<ScatterDesc>& d, int64_t total, const int32_t* list_dev, const void* src,
                    void* dst, cudaStream_t s, DevBuf& keep_d) {
  if (total == 0) return;
  keep_d = upload(d, s);
  k_scatter<T><<<grid_for(total), 256, 0, s>>>(keep_d.as<ScatterDesc>(), (int)d.size(), total, list_dev,
                                                static_cast<const T*>(src), static_cast<T*>(dst));
  QLTG_CUDA(cudaGetLastError());
}

template <typename T>
void launch_scatter(const std::vector<ScatterDesc>& d, int64_t total, const std::vector<int32_t>& list,
                    const void* src, void* dst, cudaStream_t s, DevBuf& keep_d, DevBuf& keep_l) {
  if (total == 0) return;
  keep_l = upload(list.empty() ? std::vector<int32_t>{0} : list, s);
  launch_scatter<T>(d, total, keep_l.as<int32_t>(), src, dst, s, keep_d);
}

}  // namespace
}  // namespace qltg

using namespace qltg;

struct qltg_decomp {
  Meta t[3];
  DevBuf buf[3];
  int ntensors = 0;
  double err = 0;
  int64_t D = 0;
};

namespace qltg {
namespace {


// ---- QR preconditioning of the one-sided Jacobi (the Drmac-Veselic scheme, restated):
// M = Q R (blocked Householder), Jacobi on X = R^H, then M = (Q J) S Xn^H with
// Xn the normalised columns of X and J the accumulated rotations. On graded spectra (the
// decaying singular values of a DMRG bond) this cuts the sweeps from ~30 to ~8.
struct PrecondJob {
  int64_t a_off;   // R in the upper triangle of the factorised p x q matrix (column-major, ld p)
  int64_t q_off;   // Q, p x q column-major
  int64_t x_off;   // X = R^H, q vectors of length q (vector i = conj of row i of R)
  int64_t j_off;   // J, q x q vector-major
  int64_t w_off;   // output Q J, q vectors of length p
  int32_t p, q;
};

template <typename T>
__global__ void k_r_to_x(const PrecondJob* __restrict__ jobs, int njobs, const T* __restrict__ as,
                         T* __restrict__ xs) {
  const PrecondJob jb = jobs[blockIdx.x];
  const int p = jb.p, q = jb.q;
  for (int64_t e = threadIdx.x; e < (int64_t)q * q; e += blockDim.x) {
    const int i = (int)(e / q), c = (int)(e - (int64_t)i * q);   // vector i, element c = conj(R[i, c])
    T v{};
    if (c >= i) {
      v = as[jb.a_off + (int64_t)c * p + i];
      if constexpr (sizeof(T) == 16) v.y = -v.y;
    }
    xs[jb.x_off + e] = v;
  }
}

// W = Q J per job: 32 x 32 output tiles (tile list flattened over jobs), FP64 FMA.
struct QjTile {
  int32_t job, tm, tn;
};

template <typename T>
__global__ void __launch_bounds__(256) k_qj(const PrecondJob* __restrict__ jobs, const QjTile* __restrict__ tiles,
                                            int ntiles, const T* __restrict__ qs, const T* __restrict__ js,
                                            T* __restrict__ ws) {
  __shared__ T sq[32][33];
  __shared__ T sj[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
    const QjTile tl = tiles[ti];
    const PrecondJob jb = jobs[tl.job];
    const int p = jb.p, q = jb.q;
    const int r0 = tl.tm * 32, c0 = tl.tn * 32;
    T acc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = T{};
    for (int k0 = 0; k0 < q; k0 += 32) {
      // Q[r0 + tx, k0 + kk] (column-major) and J[k0 + kk, c0 + col] (vector-major: J[col * q + kk])
      for (int kk = ty; kk < 32; kk += 8) {
        sq[kk][tx] = (r0 + tx < p && k0 + kk < q) ? qs[jb.q_off + (int64_t)(k0 + kk) * p + r0 + tx] : T{};
        sj[tx][kk] = (c0 + tx < q && k0 + kk < q) ? js[jb.j_off + (int64_t)(c0 + tx) * q + k0 + kk] : T{};
      }
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < 32; ++kk) {
        const T a = sq[kk][tx];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const T b = sj[ty + 8 * u][kk];
          if constexpr (sizeof(T) == 8) acc[u] = fma(a, b, acc[u]);
          else acc[u] = make_double2(acc[u].x + a.x * b.x - a.y * b.y, acc[u].y + a.x * b.y + a.y * b.x);
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int c = c0 + ty + 8 * u, r = r0 + tx;
      if (r < p && c < q) ws[jb.w_off + (int64_t)c * p + r] = acc[u];
    }
  }
}

template <typename T>
void svd_impl(const Meta& t, const void* t_dev, int ldims, const std::vector<int32_t>& lqndiv, double trunc,
              int64_t dmin, int64_t dmax, cudaStream_t s, qltg_decomp& out) {
  auto groups = group_blocks(t, ldims, lqndiv);
  const int ng = (int)groups.size();
  // Work layout (one workspace): for every group its q vectors of length p (the columns of
  // the group matrix when rows >= cols, else its rows), then every group's q x q rotations.
  std::vector<JacobiJob> jobs(ng);
  std::vector<CopyDesc> cd;
  int64_t woff = 0, eoff = 0;
  std::vector<int64_t> sv_off(ng + 1, 0);
  std::vector<char> cols_vec(ng);
  for (int g = 0; g < ng; ++g) {
    const Group& G = groups[g];
    cols_vec[g] = G.rows >= G.cols;
    JacobiJob& j = jobs[g];
    j.p = (int32_t)(cols_vec[g] ? G.rows : G.cols);
    j.q = (int32_t)(cols_vec[g] ? G.cols : G.rows);
    j.w_off = woff;
    woff += (int64_t)j.p * j.q;
    sv_off[g + 1] = sv_off[g] + j.q;
    for (size_t e = 0; e < G.eblk.size(); ++e) {
      CopyDesc c{};
      c.src_off = t.offsets[G.eblk[e]];
      c.dst_off = j.w_off;
      c.elem_begin = eoff;
      c.rd = (int32_t)G.rdim[G.erow[e]];
      c.cd = (int32_t)G.cdim[G.ecol[e]];
      c.ro = (int32_t)G.roff[G.erow[e]];
      c.co = (int32_t)G.coff[G.ecol[e]];
      c.ld = (int32_t)(cols_vec[g] ? G.rows : G.cols);
      c.col_major = cols_vec[g] ? 1 : 0;
      eoff += (int64_t)c.rd * c.cd;
      cd.push_back(c);
    }
  }
  int64_t voff = woff;
  for (int g = 0; g < ng; ++g) { jobs[g].v_off = voff; voff += (int64_t)jobs[g].q * jobs[g].q; }
  const size_t eb = sizeof(T);
  DevBuf ws(std::max<int64_t>(1, voff) * eb), keep_g;
  const int64_t nsv = sv_off[ng];
  QLTG_CHECK(nsv < ((int64_t)1 << 31), QLTG_ERR_INVALID, "more than 2^31 singular values");
  DevBuf sv(std::max<int64_t>(1, nsv) * 8), order(std::max<int64_t>(1, nsv) * 4);
  DevBuf svs(std::max<int64_t>(1, nsv) * 8), sorted_v(std::max<int64_t>(1, nsv) * 8),
      sorted_g(std::max<int64_t>(1, nsv) * 4), sv_key(std::max<int64_t>(1, nsv) * 8),
      sv_key_s(std::max<int64_t>(1, nsv) * 8), sv_idx(std::max<int64_t>(1, nsv) * 4),
      sv_idx_s(std::max<int64_t>(1, nsv) * 4);
  DevBuf d_svoff = upload(sv_off, s);
  if (woff) QLTG_CUDA(cudaMemsetAsync(ws.get(), 0, woff * eb, s));
  launch_gather<T>(cd, eoff, t_dev, ws.get(), s, keep_g);
  // QR preconditioning: M = Q R (Householder, in place in the W region), X = R^H into the
  // V region; the Jacobi below works on X with its rotations J in their own buffer
  std::vector<QrJob> qjobs(ng);
  std::vector<PrecondJob> pre(ng);
  std::vector<JacobiJob> xjobs(ng);
  std::vector<QjTile> qtiles;
  int64_t qoff = 0, toff = 0, joff = 0;
  for (int g = 0; g < ng; ++g) {
    const JacobiJob& j = jobs[g];
    qjobs[g] = QrJob{j.w_off, toff, qoff, j.p, j.q};
    pre[g] = PrecondJob{j.w_off, qoff, j.v_off, joff, j.w_off, j.p, j.q};
    xjobs[g] = JacobiJob{j.v_off, joff, j.q, j.q};
    qoff += (int64_t)j.p * j.q;
    toff += j.q;
    joff += (int64_t)j.q * j.q;
    for (int tm = 0; tm * 32 < j.p; ++tm)
      for (int tn = 0; tn * 32 < j.q; ++tn) qtiles.push_back(QjTile{g, tm, tn});
  }
  DevBuf qbuf(std::max<int64_t>(1, qoff) * eb), taubuf(std::max<int64_t>(1, toff) * eb),
      jbuf(std::max<int64_t>(1, joff) * eb);
  DevBuf d_pre = upload(pre, s), d_qtiles = upload(qtiles, s);
  QrBuffers qr_keep;
  if (ng) {
    launch_blocked_qr<T>(qjobs, ws.as<T>(), taubuf.as<T>(), qbuf.as<T>(), s, qr_keep);
    k_r_to_x<T><<<ng, kThreads, 0, s>>>(d_pre.as<PrecondJob>(), ng, ws.as<T>(), ws.as<T>());
    QLTG_CUDA(cudaGetLastError());
  }
  // Jacobi jobs by cluster size: starting from one CTA each, the job with the most work per
  // CTA (q^2 (p + q) multiply-adds per sweep / CTAs) gets one CTA more, until the SMs are
  // used up (clusters of at most 16 CTAs, at least two columns per CTA), so the largest
  // groups finish about together. Each cluster size is one launch on its own stream, forked
  // from s and joined back, largest clusters first. A one-CTA job whose columns fit in shared
  // memory keeps them there for all sweeps; the others step through block pairs on the
  // cluster barrier.
  const int nsm = current_sm_count();
  std::vector<double> jwork(ng);
  std::vector<int> jcl(ng, 1);
  for (int g = 0; g < ng; ++g) jwork[g] = (double)xjobs[g].q * xjobs[g].q * (xjobs[g].p + xjobs[g].q);
  for (int used = ng; used < nsm;) {
    int best = -1;
    for (int g = 0; g < ng; ++g)
      if (jcl[g] < kMaxCluster && 2 * (jcl[g] + 1) <= xjobs[g].q &&
          (best < 0 || jwork[g] / jcl[g] > jwork[best] / jcl[best]))
        best = g;
    if (best < 0) break;
    ++jcl[best];
    ++used;
  }
  constexpr int kClasses = kMaxCluster;   // class ci holds the jobs on clusters of ci + 1 CTAs
  std::vector<JacobiJob> cls_jobs[kClasses];
  for (int g = 0; g < ng; ++g) cls_jobs[jcl[g] - 1].push_back(xjobs[g]);
  {
    static std::mutex mu;
    static bool done[2][64] = {};
    int dev = 0;
    QLTG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !done[sizeof(T) == 16][dev]) {
      QLTG_CUDA(cudaFuncSetAttribute(k_jacobi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kJacobiSmem));
      QLTG_CUDA(cudaFuncSetAttribute(k_jacobi<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      if (dev >= 0 && dev < 64) done[sizeof(T) == 16][dev] = true;
    }
  }
  DevBuf d_cls[kClasses], st_cls[kClasses], sr_cls[kClasses];
  for (int ci = 0; ci < kClasses; ++ci) {
    if (cls_jobs[ci].empty()) continue;
    d_cls[ci] = upload(cls_jobs[ci], s);
    st_cls[ci].alloc(cls_jobs[ci].size() * 4);
    sr_cls[ci].alloc(cls_jobs[ci].size() * kMaxSweeps * 4);
    QLTG_CUDA(cudaMemsetAsync(sr_cls[ci].get(), 0, sr_cls[ci].bytes(), s));
  }
  // rotate while |<wi, wj>| > tol ||wi|| ||wj||: columns orthogonal to a few ulps
  const double tol = 64.0 * 2.220446049250313e-16;
  cudaEvent_t fork = nullptr;
  QLTG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  QLTG_CUDA(cudaEventRecord(fork, s));
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> joins;
  cudaError_t le = cudaSuccess;
  for (int ci = kClasses - 1; ci >= 0 && le == cudaSuccess; --ci) {
    if (cls_jobs[ci].empty()) continue;
    const int cl = ci + 1;
    cudaStream_t sx = nullptr;
    le = cudaStreamCreateWithFlags(&sx, cudaStreamNonBlocking);
    if (le != cudaSuccess) break;
    side.push_back(sx);
    le = cudaStreamWaitEvent(sx, fork, 0);
    if (le != cudaSuccess) break;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(cls_jobs[ci].size() * cl));
    cfg.blockDim = dim3(kJacThreads);
    cfg.dynamicSmemBytes = kJacobiSmem;
    cfg.stream = sx;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = cl > 1 ? 1 : 0;
    le = cudaLaunchKernelEx(&cfg, k_jacobi<T>, d_cls[ci].as<const JacobiJob>(), cl, ws.as<T>(), jbuf.as<T>(),
                            sr_cls[ci].as<int>(), st_cls[ci].as<int>(), tol, (int)kJacobiSmem);
    if (le != cudaSuccess) break;
    cudaEvent_t j = nullptr;
    le = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    if (le != cudaSuccess) break;
    joins.push_back(j);
    le = cudaEventRecord(j, sx);
  }
  for (auto j : joins) {
    cudaStreamWaitEvent(s, j, 0);
    cudaEventDestroy(j);
  }
  cudaEventDestroy(fork);
  for (auto sx : side) cudaStreamDestroy(sx);   // freed by CUDA once its queued work is done
  QLTG_CUDA(le);
  // singular values and the right vectors from X; the left vectors W = Q J
  DevBuf d_jobs = upload(xjobs, s);
  if (ng) {
    k_qj<T><<<(unsigned)std::min<size_t>(std::max<size_t>(1, qtiles.size()), (size_t)current_sm_count() * 8), 256, 0, s>>>(
        d_pre.as<PrecondJob>(), d_qtiles.as<QjTile>(), (int)qtiles.size(), qbuf.as<T>(), jbuf.as<T>(), ws.as<T>());
    QLTG_CUDA(cudaGetLastError());
    k_svd_finish<T><<<ng, kThreads, 0, s>>>(d_jobs.as<JacobiJob>(), ws.as<T>(), sv.as<double>(),
                                             d_svoff.as<int64_t>(), order.as<int32_t>(), svs.as<double>());
    QLTG_CUDA(cudaGetLastError());
  }
  // truncation on the device; only the kept dimension, the error and the kept count of each
  // group come back (they size the result tensors)
  const size_t cut_bytes = sizeof(SvCut) + (size_t)ng * 4;
  DevBuf cutbuf(cut_bytes);
  QLTG_CUDA(cudaMemsetAsync(cutbuf.get(), 0, cut_bytes, s));
  SvCut* d_cut = cutbuf.as<SvCut>();
  int* d_kcnt = reinterpret_cast<int*>(static_cast<char*>(cutbuf.get()) + sizeof(SvCut));
  DevBuf sort_tmp;
  if (nsv) {
    k_sv_keys<<<grid_for(nsv), 256, 0, s>>>(svs.as<double>(), nsv, sv_key.as<uint64_t>(), sv_idx.as<int32_t>(), d_cut);
    QLTG_CUDA(cudaGetLastError());
    size_t tmp_bytes = 0;
    QLTG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, sv_key.as<uint64_t>(), sv_key_s.as<uint64_t>(),
                                              sv_idx.as<int32_t>(), sv_idx_s.as<int32_t>(), (int)nsv, 0, 64, s));
    sort_tmp.alloc(std::max<size_t>(tmp_bytes, 16));
    QLTG_CUDA(cub::DeviceRadixSort::SortPairs(sort_tmp.get(), tmp_bytes, sv_key.as<uint64_t>(), sv_key_s.as<uint64_t>(),
                                              sv_idx.as<int32_t>(), sv_idx_s.as<int32_t>(), (int)nsv, 0, 64, s));
    k_sv_sorted<<<grid_for(nsv), 256, 0, s>>>(svs.as<double>(), d_svoff.as<int64_t>(), ng, sv_idx_s.as<int32_t>(), nsv,
                                              sorted_v.as<double>(), sorted_g.as<int32_t>());
    QLTG_CUDA(cudaGetLastError());
  }
  k_sv_cut<<<1, 256, 0, s>>>(sorted_v.as<double>(), sorted_g.as<int32_t>(), sv.as<double>(), trunc, dmin, dmax, ng,
                             d_cut, d_kcnt);   // sv (by vector index) is free again: the prefix sums
  QLTG_CUDA(cudaGetLastError());
  std::vector<char> h_cut(cut_bytes);
  QLTG_CUDA(cudaMemcpyAsync(h_cut.data(), cutbuf.get(), cut_bytes, cudaMemcpyDeviceToHost, s));
  std::vector<int> h_st;
  {
    size_t total_jobs = 0;
    for (int ci = 0; ci < kClasses; ++ci) total_jobs += cls_jobs[ci].size();
    h_st.resize(total_jobs);
    size_t at = 0;
    for (int ci = 0; ci < kClasses; ++ci) {
      if (cls_jobs[ci].empty()) continue;
      QLTG_CUDA(cudaMemcpyAsync(h_st.data() + at, st_cls[ci].get(), cls_jobs[ci].size() * 4, cudaMemcpyDeviceToHost, s));
      at += cls_jobs[ci].size();
    }
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
  for (int x : h_st) QLTG_CHECK(x >= 0, QLTG_ERR_NOCONV, "one-sided Jacobi did not converge within 60 sweeps");

  SvCut hc;
  std::memcpy(&hc, h_cut.data(), sizeof(SvCut));
  std::vector<int> kcnt(ng);
  if (ng) std::memcpy(kcnt.data(), h_cut.data() + sizeof(SvCut), (size_t)ng * 4);
  out.err = hc.err;
  out.D = hc.kept;
  QLTG_CHECK(hc.kept > 0, QLTG_ERR_EMPTY_SVD,
             "SVD failed: empty result. The input tensor has no data blocks compatible with the specified "
             "quantum number divergence (lqndiv).");
  std::map<int, int> kept_n;   // group -> kept count (its leading ranks)
  for (int g = 0; g < ng; ++g)
    if (kcnt[g] > 0) kept_n[g] = kcnt[g];

  // ---- result metadata (reference ten_svd.h:467-582) --------------------------------
  std::vector<int32_t> mid_q;
  std::vector<int64_t> mid_d;
  for (auto& kv : kept_n) {
    for (auto q : groups[kv.first].mid) mid_q.push_back(q);
    mid_d.push_back((int64_t)kv.second);
  }
  Meta U = leg_subset(t, 0, ldims), Vt = leg_subset(t, ldims, t.rank), S = leg_subset(t, 0, 0);
  U.rank += 1;
  U.dirs.push_back(QLTG_OUT); U.qns.push_back(mid_q); U.dims.push_back(mid_d);
  Vt.rank += 1;
  Vt.dirs.insert(Vt.dirs.begin(), QLTG_IN); Vt.qns.insert(Vt.qns.begin(), mid_q); Vt.dims.insert(Vt.dims.begin(), mid_d);
  S.rank = 2;
  S.dtype = QLTG_F64;
  S.dirs = {QLTG_IN, QLTG_OUT};
  S.qns = {mid_q, mid_q};
  S.dims = {mid_d, mid_d};
  std::vector<std::vector<int64_t>> uc, vc, sc;
  int64_t mc = 0;
  for (auto& kv : kept_n) {
    const Group& G = groups[kv.first];
    sc.push_back({mc, mc});
    for (auto& rk : G.rkeys) { auto c = rk; c.push_back(mc); uc.push_back(c); }
    for (auto& ck : G.ckeys) { std::vector<int64_t> c{mc}; c.insert(c.end(), ck.begin(), ck.end()); vc.push_back(c); }
    ++mc;
  }
  sort_blocks(U, uc);
  sort_blocks(Vt, vc);
  sort_blocks(S, sc);
  out.ntensors = 3;
  out.buf[0].alloc(std::max<int64_t>(1, U.size) * eb);
  out.buf[1].alloc(std::max<int64_t>(1, S.size) * 8);
  out.buf[2].alloc(std::max<int64_t>(1, Vt.size) * eb);

  // ---- scatter U / Vt from the dense factors (one launch each), S's diagonals ---------
  // With M = A (rows >= cols) or A^T (rows < cols) factorised as M = W S G^H (W = Q J in the
  // W region, G = the normalised X in the V region):
  // rows >= cols: U = W and Vt = G^H.
  // rows <  cols: A = conj(G) S W^T: U = conj(G) and Vt = W^T.
  // The kept vectors of a group are its leading ranks: the column list is the group's
  // part of the rank order on the device.
  std::vector<ScatterDesc> su, sd;
  std::vector<SvDiag> sdg;
  int64_t eu = 0, ev = 0;
  mc = 0;
  for (auto& kv : kept_n) {
    const int g = kv.first;
    const Group& G = groups[g];
    const JacobiJob& j = jobs[g];
    const int kd = kv.second;
    const int32_t lbase = (int32_t)sv_off[g];
    for (size_t ri = 0; ri < G.rkeys.size(); ++ri) {
      auto c = G.rkeys[ri];
      c.push_back(mc);
      ScatterDesc d{};
      d.dst_off = U.offsets[block_of(U, c)];
      d.elem_begin = eu;
      d.rows = (int32_t)G.rdim[ri];
      d.cols = kd;
      d.r0 = (int32_t)G.roff[ri];
      d.col_major = 1;
      d.list_on_cols = 1;
      d.list_off = lbase;
      if (cols_vec[g]) { d.src_off = j.w_off; d.ld = j.p; d.conj = 0; }
      else { d.src_off = j.v_off; d.ld = j.q; d.conj = 1; }
      eu += (int64_t)d.rows * d.cols;
      su.push_back(d);
    }
    for (size_t ci = 0; ci < G.ckeys.size(); ++ci) {
      std::vector<int64_t> c{mc};
      c.insert(c.end(), G.ckeys[ci].begin(), G.ckeys[ci].end());
      ScatterDesc d{};
      d.dst_off = Vt.offsets[block_of(Vt, c)];
      d.elem_begin = ev;
      d.rows = kd;
      d.cols = (int32_t)G.cdim[ci];
      d.c0 = (int32_t)G.coff[ci];
      d.col_major = 0;
      d.list_on_cols = 0;
      d.list_off = lbase;
      if (cols_vec[g]) { d.src_off = j.v_off; d.ld = j.q; d.conj = 1; }
      else { d.src_off = j.w_off; d.ld = j.p; d.conj = 0; }
      ev += (int64_t)d.rows * d.cols;
      sd.push_back(d);
    }
    sdg.push_back({S.offsets[block_of(S, {mc, mc})], sv_off[g], kd, 0});
    ++mc;
  }
  DevBuf k1, k3, k5;
  launch_scatter<T>(su, eu, order.as<int32_t>(), ws.get(), out.buf[0].get(), s, k1);
  launch_scatter<T>(sd, ev, order.as<int32_t>(), ws.get(), out.buf[2].get(), s, k3);
  if (S.size) {
    QLTG_CUDA(cudaMemsetAsync(out.buf[1].get(), 0, S.size * 8, s));
    k5 = upload(sdg, s);
    k_sv_diag<<<(unsigned)std::min<size_t>(sdg.size(), 1024), 128, 0, s>>>(k5.as<SvDiag>(), (int)sdg.size(),
                                                                         svs.as<double>(), out.buf[1].as<double>());
    QLTG_CUDA(cudaGetLastError());
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
  out.t[0] = U;
  out.t[1] = S;
  out.t[2] = Vt;
}

template <typename T>
void qr_impl(const Meta& t, const void* t_dev, int ldims, const std::vector<int32_t>& lqndiv, cudaStream_t s,
             qltg_decomp& out) {
  auto groups = group_blocks(t, ldims, lqndiv);
  const int ng = (int)groups.size();
  std::vector<QrJob> jobs(ng);
  std::vector<CopyDesc> cd;
  int64_t aoff = 0, toff = 0, qoff = 0, eoff = 0;
  for (int g = 0; g < ng; ++g) {
    const Group& G = groups[g];
    QrJob& j = jobs[g];
    j.m = (int32_t)G.rows;
    j.n = (int32_t)G.cols;
    j.a_off = aoff;
    j.tau_off = toff;
    aoff += G.rows * G.cols;
    toff += std::min(G.rows, G.cols);
    for (size_t e = 0; e < G.eblk.size(); ++e) {
      CopyDesc c{};
      c.src_off = t.offsets[G.eblk[e]];
      c.dst_off = j.a_off;
      c.elem_begin = eoff;
      c.rd = (int32_t)G.rdim[G.erow[e]];
      c.cd = (int32_t)G.cdim[G.ecol[e]];
      c.ro = (int32_t)G.roff[G.erow[e]];
      c.co = (int32_t)G.coff[G.ecol[e]];
      c.ld = (int32_t)G.rows;
      c.col_major = 1;
      eoff += (int64_t)c.rd * c.cd;
      cd.push_back(c);
    }
  }
  for (int g = 0; g < ng; ++g) { jobs[g].q_off = qoff; qoff += (int64_t)jobs[g].m * std::min(jobs[g].m, jobs[g].n); }
  const size_t eb = sizeof(T);
  DevBuf A(std::max<int64_t>(1, aoff) * eb), tau(std::max<int64_t>(1, toff) * eb), Qd(std::max<int64_t>(1, qoff) * eb);
  DevBuf keep_g;
  if (aoff) QLTG_CUDA(cudaMemsetAsync(A.get(), 0, aoff * eb, s));
  launch_gather<T>(cd, eoff, t_dev, A.get(), s, keep_g);
  QrBuffers qr_keep;
  if (ng) launch_blocked_qr<T>(jobs, A.as<T>(), tau.as<T>(), Qd.as<T>(), s, qr_keep);
  // result metadata (reference ten_qr.h:199-291): mid dim min(rows, cols) per group
  std::vector<int32_t> mid_q;
  std::vector<int64_t> mid_d;
  for (auto& G : groups) {
    for (auto q : G.mid) mid_q.push_back(q);
    mid_d.push_back(std::min(G.rows, G.cols));
  }
  Meta Q = leg_subset(t, 0, ldims), R = leg_subset(t, ldims, t.rank);
  Q.rank += 1;
  Q.dirs.push_back(QLTG_OUT); Q.qns.push_back(mid_q); Q.dims.push_back(mid_d);
  R.rank += 1;
  R.dirs.insert(R.dirs.begin(), QLTG_IN); R.qns.insert(R.qns.begin(), mid_q); R.dims.insert(R.dims.begin(), mid_d);
  std::vector<std::vector<int64_t>> qc, rc;
  for (int g = 0; g < ng; ++g) {
    for (auto& rk : groups[g].rkeys) { auto c = rk; c.push_back(g); qc.push_back(c); }
    for (auto& ck : groups[g].ckeys) { std::vector<int64_t> c{(int64_t)g}; c.insert(c.end(), ck.begin(), ck.end()); rc.push_back(c); }
  }
  if (ng) {
    sort_blocks(Q, qc);
    sort_blocks(R, rc);
  } else {
    Q.nblk = R.nblk = 0;
    Q.refresh_offsets();
    R.refresh_offsets();
  }
  out.ntensors = 2;
  out.buf[0].alloc(std::max<int64_t>(1, Q.size) * eb);
  out.buf[1].alloc(std::max<int64_t>(1, R.size) * eb);
  // Q blocks: rows of the row sector, all k columns (column-major dense Q, ld m)
  // R blocks: the k x n upper triangle (zero below the diagonal) restricted to a col sector
  std::vector<ScatterDesc> sq, sr;
  std::vector<int32_t> list;
  int64_t eq = 0, er = 0;
  for (int g = 0; g < ng; ++g) {
    const Group& G = groups[g];
    const QrJob& j = jobs[g];
    const int k = std::min(j.m, j.n);
    const int32_t lbase = (int32_t)list.size();
    for (int i = 0; i < k; ++i) list.push_back(i);
    for (size_t ri = 0; ri < G.rkeys.size(); ++ri) {
      auto c = G.rkeys[ri];
      c.push_back(g);
      ScatterDesc d{};
      d.dst_off = Q.offsets[block_of(Q, c)];
      d.src_off = j.q_off;
      d.elem_begin = eq;
      d.rows = (int32_t)G.rdim[ri];
      d.cols = k;
      d.r0 = (int32_t)G.roff[ri];
      d.ld = j.m;
      d.col_major = 1;
      d.list_on_cols = 1;
      d.list_off = lbase;
      eq += (int64_t)d.rows * d.cols;
      sq.push_back(d);
    }
    for (size_t ci = 0; ci < G.ckeys.size(); ++ci) {
      std::vector<int64_t> c{(int64_t)g};
      c.insert(c.end(), G.ckeys[ci].begin(), G.ckeys[ci].end());
      ScatterDesc d{};
      d.dst_off = R.offsets[block_of(R, c)];
      d.src_off = j.a_off;
      d.elem_begin = er;
      d.rows = k;
      d.cols = (int32_t)G.cdim[ci];
      d.c0 = (int32_t)G.coff[ci];
      d.ld = j.m;
      d.col_major = 1;
      d.list_on_cols = 0;
      d.list_off = lbase;
      d.conj = 2;   // marker: keep only the upper triangle (row <= col)
      er += (int64_t)d.rows * d.cols;
      sr.push_back(d);
    }
  }
  DevBuf k1, k2, k3, k4;
  launch_scatter<T>(sq, eq, list, Qd.get(), out.buf[0].get(), s, k1, k2);
  launch_scatter<T>(sr, er, list, A.get(), out.buf[1].get(), s, k3, k4);
  QLTG_CUDA(cudaStreamSynchronize(s));
  out.t[0] = Q;
  out.t[1] = R;
  out.err = 0;
  int64_t dsum = 0;
  for (auto d : mid_d) dsum += d;
  out.D = dsum;
}

}  // namespace
}  // namespace qltg

extern "C" {

int qltg_svd(qltg_ctx* ctx, const qltg_tensor_desc* t, const void* t_dev, int32_t ldims, const int32_t* lqndiv,
             double trunc_err, int64_t dmin, int64_t dmax, void* stream, qltg_decomp** out) {
  return guarded([&] {
    QLTG_CHECK(ctx && out && lqndiv, QLTG_ERR_INVALID, "null ctx, lqndiv or output pointer");
    Meta m = meta_from_desc(t);
    QLTG_CHECK(m.rank >= 2 && ldims >= 1 && ldims < m.rank, QLTG_ERR_INVALID, "SVD needs rank >= 2 and 0 < ldims < rank");
    QLTG_CHECK(trunc_err >= 0 && dmin >= 0 && dmin <= dmax, QLTG_ERR_INVALID, "bad truncation parameters");
    QLTG_CHECK(m.nblk == 0 || t_dev, QLTG_ERR_INVALID, "null tensor buffer");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    std::vector<int32_t> div(lqndiv, lqndiv + m.ncomp);
    auto h = std::make_unique<qltg_decomp>();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (m.dtype == QLTG_C128) svd_impl<double2>(m, t_dev, ldims, div, trunc_err, dmin, dmax, s, *h);
    else svd_impl<double>(m, t_dev, ldims, div, trunc_err, dmin, dmax, s, *h);
    *out = h.release();
  });
}

int qltg_qr(qltg_ctx* ctx, const qltg_tensor_desc* t, const void* t_dev, int32_t ldims, const int32_t* lqndiv,
            void* stream, qltg_decomp** out) {
  return guarded([&] {
    QLTG_CHECK(ctx && out && lqndiv, QLTG_ERR_INVALID, "null ctx, lqndiv or output pointer");
    Meta m = meta_from_desc(t);
    QLTG_CHECK(m.rank >= 2 && ldims >= 1 && ldims < m.rank, QLTG_ERR_INVALID, "QR needs rank >= 2 and 0 < ldims < rank");
    QLTG_CHECK(m.nblk == 0 || t_dev, QLTG_ERR_INVALID, "null tensor buffer");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    std::vector<int32_t> div(lqndiv, lqndiv + m.ncomp);
    auto h = std::make_unique<qltg_decomp>();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (m.dtype == QLTG_C128) qr_impl<double2>(m, t_dev, ldims, div, s, *h);
    else qr_impl<double>(m, t_dev, ldims, div, s, *h);
    *out = h.release();
  });
}

int qltg_decomp_info(const qltg_decomp* d, double* trunc_err, int64_t* kept_dim) {
  return guarded([&] {
    QLTG_CHECK(d, QLTG_ERR_INVALID, "null decomposition");
    if (trunc_err) *trunc_err = d->err;
    if (kept_dim) *kept_dim = d->D;
  });
}

int qltg_decomp_tensor_info(const qltg_decomp* d, int32_t which, int64_t* info) {
  return guarded([&] {
    QLTG_CHECK(d && info, QLTG_ERR_INVALID, "null decomposition or info");
    QLTG_CHECK(which >= 0 && which < d->ntensors, QLTG_ERR_INVALID, "no such result tensor");
    const Meta& m = d->t[which];
    int64_t ts = 0;
    for (auto& x : m.dims) ts += (int64_t)x.size();
    info[0] = m.rank; info[1] = m.ncomp; info[2] = m.dtype; info[3] = m.nblk; info[4] = m.size; info[5] = ts;
  });
}

int qltg_decomp_tensor_export(const qltg_decomp* d, int32_t which, int32_t* dirs, int32_t* nsct, int32_t* qns,
                              int64_t* dims, int64_t* coords, int64_t* offsets, const void** dev) {
  return guarded([&] {
    QLTG_CHECK(d, QLTG_ERR_INVALID, "null decomposition");
    QLTG_CHECK(which >= 0 && which < d->ntensors, QLTG_ERR_INVALID, "no such result tensor");
    d->t[which].export_arrays(dirs, nsct, qns, dims, coords, offsets);
    if (dev) *dev = d->buf[which].get();
  });
}

int qltg_decomp_destroy(qltg_decomp* d) {
  delete d;
  return QLTG_OK;
}

}  // extern "C"
