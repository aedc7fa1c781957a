// Lanczos on the two-site effective Hamiltonian, every vector operation on the device.
//
// The reference leaves the eigensolver to its callers and gives them the BSDT vector
// primitives: Dot / Norm / Normalize / ScaleByFactor / LinearCombine on the raw buffer
// (framework/hp_numeric/blas_level1.h; tensor_manipulation/ten_linear_combine.h:186-459;
// qltensor/blk_spar_data_ten/raw_data_operations.h:225-272). Lanczos vectors all share ψ's
// block topology, so here they are plain FP64 raw buffers and the primitives act on them
// directly.
//
// Step j (v_0 = ψ0 / ||ψ0||, V = [v_0 .. v_j] kept on the device):
//   w = H v_j                                   (the matvec's four contractions)
//   two passes of classical Gram-Schmidt:       c = Vᵀ w;  w -= V c;  α_j += c_j
//   β_{j+1} = ||w||;  v_{j+1} = w / β_{j+1}
// Full reorthogonalisation replaces the three-term recurrence (the projection on v_{j-1} is
// β_j). All of it is FP64 with deterministic reductions (fixed per-CTA partials summed in a
// fixed order), and α, β never leave the device until the caller asks for them. Each step
// is one CUDA graph (the matvec's kernels plus the vector kernels), built on first use.
#include <cmath>
#include <memory>

#include "matvec.h"

using namespace qltg;

namespace {

constexpr int kVecThreads = 256;
constexpr int kVecBlocks = 152 * 4;   // fixed grid: the partial-sum order is fixed too

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

// part[i * gridDim.x + b] = sum over CTA b's chunk of V_i[e] w[e], i = 0 .. nv-1.
__global__ void __launch_bounds__(kVecThreads) k_multi_dot(const double* __restrict__ V, int nv, int64_t ld,
                                                           const double* __restrict__ w, int64_t n,
                                                           double* __restrict__ part) {
  __shared__ double red[kVecThreads / 32];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t e0 = (int64_t)blockIdx.x * per, e1 = min(n, e0 + per);
  for (int i = 0; i < nv; ++i) {
    const double* v = V + (int64_t)i * ld;
    double acc = 0.0;
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) acc = fma(__ldg(v + e), __ldg(w + e), acc);
    const double t = block_sum(acc, red);
    if (threadIdx.x == 0) part[(int64_t)i * gridDim.x + blockIdx.x] = t;
  }
}

// c[i] = sum_b part[i * nb + b] in a fixed order; if alpha != null, alpha[0] += c[j].
__global__ void k_finish_dots(const double* __restrict__ part, int nv, int nb, double* __restrict__ c,
                              double* __restrict__ alpha, int j) {
  __shared__ double red[kVecThreads / 32];
  for (int i = 0; i < nv; ++i) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[(int64_t)i * nb + b];
    const double t = block_sum(acc, red);
    if (threadIdx.x == 0) {
      c[i] = t;
      if (alpha && i == j) alpha[0] += t;
    }
  }
}

// w -= sum_i c[i] V_i
__global__ void __launch_bounds__(kVecThreads) k_subtract(const double* __restrict__ V, int nv, int64_t ld,
                                                          const double* __restrict__ c, double* __restrict__ w,
                                                          int64_t n) {
  __shared__ double cs[64];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) cs[i] = c[i];
  __syncthreads();
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double x = w[e];
    for (int i = 0; i < nv; ++i) x = fma(-cs[i], __ldg(V + (int64_t)i * ld + e), x);
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
  int64_t n = 0;          // elements of ψ
  int64_t ld = 0;         // stride between Krylov vectors (n rounded up to 32 elements)
  int steps = 0;          // steps taken since the last start
  DevBuf V, w, part, coef;   // coef: alpha[max_iter] | beta[max_iter + 1] | c[max_iter + 1]
  std::vector<cudaGraphExec_t> graphs;
  std::vector<cudaGraph_t> graph_defs;
  cudaStream_t capture = nullptr;

  double* alpha() const { return coef.as<double>(); }
  double* beta() const { return coef.as<double>() + max_iter; }
  double* cbuf() const { return coef.as<double>() + 2 * max_iter + 1; }
  double* vec(int i) const { return V.as<double>() + (int64_t)i * ld; }

  ~qltg_lanczos() {
    for (size_t i = 0; i < graphs.size(); ++i) {
      if (graphs[i]) cudaGraphExecDestroy(graphs[i]);
      if (graph_defs[i]) cudaGraphDestroy(graph_defs[i]);
    }
    if (capture) cudaStreamDestroy(capture);
  }

  void dots(int nv, const double* x, cudaStream_t s, double* alpha_acc, int j) {
    k_multi_dot<<<kVecBlocks, kVecThreads, 0, s>>>(V.as<double>(), nv, ld, x, n, part.as<double>());
    k_finish_dots<<<1, kVecThreads, 0, s>>>(part.as<double>(), nv, kVecBlocks, cbuf(), alpha_acc, j);
  }

  // the kernels of step j, enqueued on s
  void enqueue_step(int j, cudaStream_t s) {
    mv->enqueue(vec(j), w.get(), s);
    for (int pass = 0; pass < 2; ++pass) {
      dots(j + 1, w.as<double>(), s, alpha() + j, j);
      k_subtract<<<kVecBlocks, kVecThreads, 0, s>>>(V.as<double>(), j + 1, ld, cbuf(), w.as<double>(), n);
    }
    // ||w||: the multi-dot of w with itself (one vector)
    k_multi_dot<<<kVecBlocks, kVecThreads, 0, s>>>(w.as<double>(), 1, ld, w.as<double>(), n, part.as<double>());
    k_finish_norm<<<1, kVecThreads, 0, s>>>(part.as<double>(), kVecBlocks, beta() + j + 1);
    k_scale_into<<<kVecBlocks, kVecThreads, 0, s>>>(w.as<double>(), beta() + j + 1, vec(j + 1), n);
  }
};

extern "C" {

int qltg_lanczos_create(qltg_matvec* mv, int32_t max_iter, qltg_lanczos** lz) {
  return guarded([&] {
    QLTG_CHECK(mv && lz, QLTG_ERR_INVALID, "null matvec or out-pointer");
    QLTG_CHECK(max_iter >= 1 && max_iter <= 63, QLTG_ERR_INVALID, "max_iter must be 1 .. 63");
    QLTG_CHECK(mv->step[3].c.dtype == QLTG_F64, QLTG_ERR_UNSUPPORTED, "Lanczos supports real FP64 matvecs");
    QLTG_CUDA(cudaSetDevice(mv->ctx->device));
    auto h = std::make_unique<qltg_lanczos>();
    h->mv = mv;
    h->max_iter = max_iter;
    h->n = mv->psi_size;
    QLTG_CHECK(mv->step[3].c.size == h->n, QLTG_ERR_INVALID, "matvec result and psi differ in size");
    h->ld = (h->n + 31) / 32 * 32;
    h->V.alloc(std::max<int64_t>(1, (int64_t)(max_iter + 1) * h->ld) * 8);
    h->w.alloc(std::max<int64_t>(1, h->ld) * 8);
    h->part.alloc((int64_t)kVecBlocks * (max_iter + 1) * 8);
    h->coef.alloc((int64_t)(3 * max_iter + 2) * 8);
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
    k_zero<<<1, kVecThreads, 0, s>>>(lz->coef.as<double>(), 3 * lz->max_iter + 2);
    const double* x = static_cast<const double*>(psi0_dev);
    k_multi_dot<<<kVecBlocks, kVecThreads, 0, s>>>(x, 1, lz->ld, x, lz->n, lz->part.as<double>());
    k_finish_norm<<<1, kVecThreads, 0, s>>>(lz->part.as<double>(), kVecBlocks, lz->beta());   // beta_0 = ||psi0||
    k_scale_into<<<kVecBlocks, kVecThreads, 0, s>>>(x, lz->beta(), lz->vec(0), lz->n);
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
