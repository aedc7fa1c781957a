// Lanczos on the two-site effective Hamiltonian, every vector operation on the device.
//
// The reference leaves the eigensolver to its callers and gives them the BSDT vector
// primitives: Dot / Norm / Normalize / ScaleByFactor / LinearCombine on the raw buffer
// (framework/hp_numeric/blas_level1.h, complex forms :381-1080;
// tensor_manipulation/ten_linear_combine.h:186-459;
// qltensor/blk_spar_data_ten/raw_data_operations.h:225-272). Lanczos vectors all share ψ's
// block topology, so here they are plain raw buffers (FP64, or complex128 interleaved) and the
// primitives act on them directly.
//
// Step j (v_0 = ψ0 / ||ψ0||, V = [v_0 .. v_j] kept on the device):
//   w = H v_j                                   (the matvec's four contractions)
//   two passes of classical Gram-Schmidt:       c = Vᴴ w;  w -= V c;  α_j += Re c_j
//   β_{j+1} = ||w||;  v_{j+1} = w / β_{j+1}
// Full reorthogonalisation replaces the three-term recurrence (the projection on v_{j-1} is
// β_j). For a Hermitian H, α and β are real; complex dots are <x, y> = Σ conj(x) y, the
// reference's complex Dot. All of it is FP64 with deterministic reductions (fixed per-CTA
// partials summed in a fixed order), and α, β never leave the device until the caller asks
// for them. Each step is one CUDA graph (the matvec's kernels plus the vector kernels), built
// on first use.
#include <cmath>
#include <memory>

#include "matvec.h"

using namespace qltg;

namespace {

constexpr int kVecThreads = 256;
// fixed grid, deliberately independent of the device's SM count: the partial-sum order, and
// so every α and β, is the same on every run and every GPU (608 CTAs = four per SM on a
// 152-SM GB300)
constexpr int kVecBlocks = 608;

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;   // valid in thread 0
}

// Scalar algebra of the two vector kinds: real FP64 (double) and complex128 (double2).
struct RealOps {
  using T = double;
  static constexpr int kParts = 1;   // doubles per dot result
  __device__ static void dot_acc(double v, double w, double* acc) { acc[0] = fma(v, w, acc[0]); }
  __device__ static double axpy_neg(const double* c, double v, double x) { return fma(-c[0], v, x); }
};
struct ComplexOps {
  using T = double2;
  static constexpr int kParts = 2;
  // acc += conj(v) w
  __device__ static void dot_acc(double2 v, double2 w, double* acc) {
    acc[0] = fma(v.x, w.x, fma(v.y, w.y, acc[0]));
    acc[1] = fma(v.x, w.y, fma(-v.y, w.x, acc[1]));
  }
  // x - c v
  __device__ static double2 axpy_neg(const double* c, double2 v, double2 x) {
    return make_double2(fma(-c[0], v.x, fma(c[1], v.y, x.x)), fma(-c[0], v.y, fma(-c[1], v.x, x.y)));
  }
};

// N sums at once: one warp shuffle tree each, one shared-memory round for all (valid in
// thread 0). The per-value order is fixed, as in block_sum.
template <int N>
__device__ __forceinline__ void block_sum_n(double (&v)[N], double* red) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    if (lane == 0) red[i * (kVecThreads / 32) + warp] = v[i];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double t = lane < nw ? red[i * (kVecThreads / 32) + lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      v[i] = t;
    }
  }
  __syncthreads();
}

// part[(i * gridDim.x + b) * kParts + r] = part r of the sum over CTA b's chunk of conj(V_i[e]) w[e].
// Four vectors per pass over the chunk: w is loaded once for them, and the four load streams
// keep more reads in flight than one vector at a time.
template <class Ops>
__global__ void __launch_bounds__(kVecThreads) k_multi_dot(const typename Ops::T* __restrict__ V, int nv, int64_t ld,
                                                           const typename Ops::T* __restrict__ w, int64_t n,
                                                           double* __restrict__ part) {
  constexpr int kG = 4, kN = kG * Ops::kParts;
  __shared__ double red[kN * (kVecThreads / 32)];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t e0 = (int64_t)blockIdx.x * per, e1 = min(n, e0 + per);
  for (int i0 = 0; i0 < nv; i0 += kG) {
    const int g = min(kG, nv - i0);
    double acc[kG][Ops::kParts] = {};
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const typename Ops::T x = __ldg(w + e);
#pragma unroll
      for (int u = 0; u < kG; ++u)
        if (u < g) Ops::dot_acc(__ldg(V + (int64_t)(i0 + u) * ld + e), x, acc[u]);
    }
    double flat[kN];
#pragma unroll
    for (int u = 0; u < kG; ++u)
#pragma unroll
      for (int r = 0; r < Ops::kParts; ++r) flat[u * Ops::kParts + r] = acc[u][r];
    block_sum_n<kN>(flat, red);
    if (threadIdx.x == 0)
      for (int u = 0; u < g; ++u)
        for (int r = 0; r < Ops::kParts; ++r)
          part[((int64_t)(i0 + u) * gridDim.x + blockIdx.x) * Ops::kParts + r] = flat[u * Ops::kParts + r];
  }
}

// c[i] = sum_b part[i][b] in a fixed order (kParts doubles each); if alpha != null,
// alpha[0] += Re c[j].
template <int kParts>
__global__ void k_finish_dots(const double* __restrict__ part, int nv, int nb, double* __restrict__ c,
                              double* __restrict__ alpha, int j) {
  __shared__ double red[kVecThreads / 32];
  for (int i = 0; i < nv; ++i) {
    for (int r = 0; r < kParts; ++r) {
      double acc = 0.0;
      for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[((int64_t)i * nb + b) * kParts + r];
      const double t = block_sum(acc, red);
      if (threadIdx.x == 0) {
        c[i * kParts + r] = t;
        if (alpha && i == j && r == 0) alpha[0] += t;
      }
    }
  }
}

// w -= sum_i c[i] V_i
template <class Ops>
__global__ void __launch_bounds__(kVecThreads) k_subtract(const typename Ops::T* __restrict__ V, int nv, int64_t ld,
                                                          const double* __restrict__ c, typename Ops::T* __restrict__ w,
                                                          int64_t n) {
  __shared__ double cs[64 * Ops::kParts];
  for (int i = threadIdx.x; i < nv * Ops::kParts; i += blockDim.x) cs[i] = c[i];
  __syncthreads();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    typename Ops::T x = w[e];
    for (int i = 0; i < nv; ++i) x = Ops::axpy_neg(cs + i * Ops::kParts, __ldg(V + (int64_t)i * ld + e), x);
    w[e] = x;
  }
}

// beta = ||w|| (from the partial sums of squares); v = w / beta (zero vector if beta == 0).
__global__ void k_finish_norm(const double* __restrict__ part, int nb, double* __restrict__ beta) {
  __shared__ double red[kVecThreads / 32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[b];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) beta[0] = sqrt(t);
}

__global__ void __launch_bounds__(kVecThreads) k_scale_into(const double* __restrict__ w,
                                                            const double* __restrict__ beta, double* __restrict__ v,
                                                            int64_t n) {
  const double b = beta[0];
  const double inv = b > 0.0 ? 1.0 / b : 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    v[e] = w[e] * inv;
}

__global__ void k_zero(double* p, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0.0;
}

}  // namespace

struct qltg_lanczos {
  qltg_matvec* mv = nullptr;
  int max_iter = 0;
  bool cplx = false;
  int64_t n = 0;          // elements of ψ
  int64_t ld = 0;         // stride between Krylov vectors in elements (n rounded up to 32)
  int steps = 0;          // steps taken since the last start
  // coef: alpha[max_iter] | beta[max_iter + 1] | c[2 (max_iter + 1)]
  DevBuf V, w, part, coef;
  std::vector<cudaGraphExec_t> graphs;
  std::vector<cudaGraph_t> graph_defs;
  cudaStream_t capture = nullptr;

  int parts() const { return cplx ? 2 : 1; }
  int64_t n_doubles() const { return n * parts(); }
  double* alpha() const { return coef.as<double>(); }
  double* beta() const { return coef.as<double>() + max_iter; }
  double* cbuf() const { return coef.as<double>() + 2 * max_iter + 1; }
  double* vec(int i) const { return V.as<double>() + (int64_t)i * ld * parts(); }

  ~qltg_lanczos() {
    for (size_t i = 0; i < graphs.size(); ++i) {
      if (graphs[i]) cudaGraphExecDestroy(graphs[i]);
      if (graph_defs[i]) cudaGraphDestroy(graph_defs[i]);
    }
    if (capture) cudaStreamDestroy(capture);
  }

  template <class Ops>
  void gram_schmidt(int j, cudaStream_t s) {
    using T = typename Ops::T;
    const T* Vt = V.as<T>();
    T* wt = w.as<T>();
    for (int pass = 0; pass < 2; ++pass) {
      k_multi_dot<Ops><<<kVecBlocks, kVecThreads, 0, s>>>(Vt, j + 1, ld, wt, n, part.as<double>());
      k_finish_dots<Ops::kParts><<<1, kVecThreads, 0, s>>>(part.as<double>(), j + 1, kVecBlocks, cbuf(),
                                                           alpha() + j, j);
      k_subtract<Ops><<<kVecBlocks, kVecThreads, 0, s>>>(Vt, j + 1, ld, cbuf(), wt, n);
    }
  }

  // ||x||: the real multi-dot of x with itself over its doubles (|z|^2 = re^2 + im^2)
  void norm_into(const double* x, double* out, cudaStream_t s) {
    k_multi_dot<RealOps><<<kVecBlocks, kVecThreads, 0, s>>>(x, 1, 0, x, n_doubles(), part.as<double>());
    k_finish_norm<<<1, kVecThreads, 0, s>>>(part.as<double>(), kVecBlocks, out);
  }

  // the kernels of step j, enqueued on s
  void enqueue_step(int j, cudaStream_t s) {
    mv->enqueue(vec(j), w.get(), s);
    if (cplx) gram_schmidt<ComplexOps>(j, s);
    else gram_schmidt<RealOps>(j, s);
    norm_into(w.as<double>(), beta() + j + 1, s);
    k_scale_into<<<kVecBlocks, kVecThreads, 0, s>>>(w.as<double>(), beta() + j + 1, vec(j + 1), n_doubles());
  }
};

extern "C" {

int qltg_lanczos_create(qltg_matvec* mv, int32_t max_iter, qltg_lanczos** lz) {
  return guarded([&] {
    QLTG_CHECK(mv && lz, QLTG_ERR_INVALID, "null matvec or out-pointer");
    QLTG_CHECK(max_iter >= 1 && max_iter <= 63, QLTG_ERR_INVALID, "max_iter must be 1 .. 63");
    QLTG_CUDA(cudaSetDevice(mv->ctx->device));
    auto h = std::make_unique<qltg_lanczos>();
    h->mv = mv;
    mv->frozen = true;   // the step graphs capture the matvec's current form
    h->max_iter = max_iter;
    h->cplx = mv->step[3].c.dtype == QLTG_C128;
    h->n = mv->psi_size;
    QLTG_CHECK(mv->step[3].c.size == h->n, QLTG_ERR_INVALID, "matvec result and psi differ in size");
    h->ld = (h->n + 31) / 32 * 32;
    const int64_t eb = h->cplx ? 16 : 8;
    h->V.alloc(std::max<int64_t>(1, (int64_t)(max_iter + 1) * h->ld) * eb);
    h->w.alloc(std::max<int64_t>(1, h->ld) * eb);
    h->part.alloc((int64_t)kVecBlocks * (max_iter + 1) * 2 * 8);
    h->coef.alloc((int64_t)(4 * max_iter + 3) * 8);
    h->graphs.assign(max_iter, nullptr);
    h->graph_defs.assign(max_iter, nullptr);
    QLTG_CUDA(cudaStreamCreateWithFlags(&h->capture, cudaStreamNonBlocking));
    *lz = h.release();
  });
}

int qltg_lanczos_start(qltg_lanczos* lz, const void* psi0_dev, void* stream) {
  return guarded([&] {
    QLTG_CHECK(lz && psi0_dev, QLTG_ERR_INVALID, "null Lanczos or psi0");
    QLTG_CUDA(cudaSetDevice(lz->mv->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_zero<<<1, kVecThreads, 0, s>>>(lz->coef.as<double>(), 4 * lz->max_iter + 3);
    const double* x = static_cast<const double*>(psi0_dev);
    lz->norm_into(x, lz->beta(), s);   // beta_0 = ||psi0||
    k_scale_into<<<kVecBlocks, kVecThreads, 0, s>>>(x, lz->beta(), lz->vec(0), lz->n_doubles());
    QLTG_CUDA(cudaGetLastError());
    lz->steps = 0;
  });
}

int qltg_lanczos_step(qltg_lanczos* lz, void* stream) {
  return guarded([&] {
    QLTG_CHECK(lz, QLTG_ERR_INVALID, "null Lanczos");
    QLTG_CHECK(lz->steps < lz->max_iter, QLTG_ERR_INVALID, "Lanczos: max_iter steps already taken");
    QLTG_CUDA(cudaSetDevice(lz->mv->ctx->device));
    const int j = lz->steps;
    if (!lz->graphs[j]) {
      // the matvec's split-precision schedule must exist before capture (its first use builds it)
      QLTG_CUDA(cudaStreamBeginCapture(lz->capture, cudaStreamCaptureModeThreadLocal));
      try {
        lz->enqueue_step(j, lz->capture);
      } catch (...) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(lz->capture, &junk);
        if (junk) cudaGraphDestroy(junk);
        throw;
      }
      QLTG_CUDA(cudaStreamEndCapture(lz->capture, &lz->graph_defs[j]));
      QLTG_CUDA(cudaGraphInstantiate(&lz->graphs[j], lz->graph_defs[j], 0));
    }
    QLTG_CUDA(cudaGraphLaunch(lz->graphs[j], static_cast<cudaStream_t>(stream)));
    lz->steps = j + 1;
  });
}

int qltg_lanczos_coeffs(qltg_lanczos* lz, int32_t* nsteps, double* alpha, double* beta, void* stream) {
  return guarded([&] {
    QLTG_CHECK(lz, QLTG_ERR_INVALID, "null Lanczos");
    QLTG_CUDA(cudaSetDevice(lz->mv->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int k = lz->steps;
    if (nsteps) *nsteps = k;
    if (alpha && k) QLTG_CUDA(cudaMemcpyAsync(alpha, lz->alpha(), k * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (beta) QLTG_CUDA(cudaMemcpyAsync(beta, lz->beta(), (k + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
    QLTG_CUDA(cudaStreamSynchronize(s));
  });
}

int qltg_lanczos_vector(const qltg_lanczos* lz, int32_t i, const void** v_dev) {
  return guarded([&] {
    QLTG_CHECK(lz && v_dev, QLTG_ERR_INVALID, "null Lanczos or out-pointer");
    QLTG_CHECK(i >= 0 && i <= lz->steps, QLTG_ERR_INVALID, "Krylov vector index out of range");
    *v_dev = lz->vec(i);
  });
}

int qltg_lanczos_destroy(qltg_lanczos* lz) {
  delete lz;
  return QLTG_OK;
}

}  // extern "C"
