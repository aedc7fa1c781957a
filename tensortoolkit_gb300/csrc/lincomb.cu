// Linear combination of block-sparse tensors with the same indexes:
//   out = sum_i coef_i T_i + beta res
// over the union of the blocks of every tensor that contributes (coef_i != 0; res when
// beta != 0, or always when the caller keeps res's topology), in ascending block index.
// Reference: LinearCombine / TensorLinearCombinationExecutor
// (tensor_manipulation/ten_linear_combine.h:33-163, :186-197): the result is rebuilt from
// the contributing tensors' blocks, the first contribution to a block copies (scaled) and
// later ones add, res last. AddScaledAssign (:211-221) is the case (coefs {alpha}, T {x},
// beta 1, res y).
//
// GB300 form: the union topology and, per output chunk of up to 4096 elements, the list of
// (tensor, element offset) contributions are built on the host once; one streaming kernel
// writes every output element once, reading each contribution in the reference's order.
#include <algorithm>
#include <map>
#include <memory>

#include "qltg_internal.h"

namespace qltg {
namespace {

constexpr int kLincombMax = 64;          // tensors per plan (res is one more)
constexpr int kLincombChunk = 4096;

struct LincombItem {
  int64_t out_off;
  int32_t n;        // elements
  int32_t c0, c1;   // contributions [c0, c1)
  int32_t pad;
};
struct LincombSrc {
  int64_t off;      // element offset of the block chunk in its tensor
  int32_t t;        // tensor ordinal; kLincombMax: res
  int32_t pad;
};
// Source pointers and coefficients of one execution, read from the parameter space by index
// (__grid_constant__: no per-thread copy).
template <typename T>
struct LincombArgs {
  const T* src[kLincombMax + 1];
  T coef[kLincombMax + 1];
};

__device__ __forceinline__ double lc_mul(double a, double x) { return a * x; }
__device__ __forceinline__ double2 lc_mul(double2 a, double2 x) {
  return make_double2(fma(a.x, x.x, -a.y * x.y), fma(a.x, x.y, a.y * x.x));
}
__device__ __forceinline__ double lc_add(double a, double b) { return a + b; }
__device__ __forceinline__ double2 lc_add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double lc_zero(double) { return 0.0; }
__device__ __forceinline__ double2 lc_zero(double2) { return make_double2(0.0, 0.0); }

// `out` may be one of the source buffers (in-place LinearCombine / AddScaledAssign: the same
// layout, so each element is read and written by one thread at the same position); it is
// therefore not declared __restrict__.
template <typename T>
__global__ void __launch_bounds__(256) k_lincomb(const LincombItem* __restrict__ items, int nitems,
                                                 const LincombSrc* __restrict__ srcs,
                                                 const __grid_constant__ LincombArgs<T> args,
                                                 T* out) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const LincombItem w = items[it];
    for (int e = threadIdx.x; e < w.n; e += blockDim.x) {
      T v = lc_zero(T());
      for (int c = w.c0; c < w.c1; ++c) {
        const LincombSrc s = srcs[c];
        const T x = lc_mul(args.coef[s.t], args.src[s.t][s.off + e]);
        v = c == w.c0 ? x : lc_add(v, x);
      }
      out[w.out_off + e] = v;
    }
  }
}

}  // namespace
}  // namespace qltg

using namespace qltg;

struct qltg_lincomb_plan {
  qltg_ctx* ctx = nullptr;
  Meta out;
  int32_t n = 0;
  bool has_res = false;
  std::vector<double> coefs;     // n + 1 entries (res last), 2 doubles each for complex
  std::vector<uint8_t> used;     // per tensor (res last): contributes to some block
  std::vector<uint8_t> same;     // per tensor (res last): its topology is the output's
  std::vector<LincombItem> items;
  std::vector<LincombSrc> srcs;
  DevBuf d_items, d_srcs;
};

int qltg_lincomb_plan_create(qltg_ctx* ctx, int32_t n, const qltg_tensor_desc* const* tens, const double* coefs,
                             const qltg_tensor_desc* res, const double* beta, int32_t keep_res,
                             qltg_lincomb_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan && tens && coefs && beta, QLTG_ERR_INVALID, "null argument");
    QLTG_CHECK(n >= 1 && n <= kLincombMax, QLTG_ERR_UNSUPPORTED, "between 1 and 64 tensors per linear combination");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    std::vector<Meta> m(n);
    for (int i = 0; i < n; ++i) m[i] = meta_from_desc(tens[i]);
    QLTG_CHECK(m[0].rank >= 1, QLTG_ERR_UNSUPPORTED, "linear combination of rank-0 tensors");
    for (int i = 1; i < n; ++i)
      QLTG_CHECK(same_indexes(m[i], m[0]), QLTG_ERR_LAYOUT, "tensors of a linear combination have different indexes");
    const int per = m[0].dtype == QLTG_C128 ? 2 : 1;
    auto h = std::make_unique<qltg_lincomb_plan>();
    h->ctx = ctx;
    h->n = n;
    h->coefs.assign((size_t)(n + 1) * 2, 0.0);
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < per; ++c) h->coefs[2 * i + c] = coefs[per * i + c];
    for (int c = 0; c < per; ++c) h->coefs[2 * n + c] = beta[c];
    const bool beta_nz = beta[0] != 0.0 || (per == 2 && beta[1] != 0.0);
    Meta rm;
    if (res) {
      rm = meta_from_desc(res);
      QLTG_CHECK(same_indexes(rm, m[0]), QLTG_ERR_LAYOUT, "result tensor has other indexes than the combined tensors");
      h->has_res = true;
    }
    QLTG_CHECK(!beta_nz || res, QLTG_ERR_INVALID, "beta != 0 needs an existing result tensor");
    // contributors in order, res last; res joins the topology when it contributes or is kept
    std::vector<const Meta*> src;
    std::vector<int32_t> ord;
    for (int i = 0; i < n; ++i) {
      const bool nz = coefs[per * i] != 0.0 || (per == 2 && coefs[per * i + 1] != 0.0);
      if (nz) {
        src.push_back(&m[i]);
        ord.push_back(i);
      }
    }
    const bool res_in = res && (beta_nz || keep_res);
    // blk_idx -> per contributor ordinal of the block (-1: absent); with beta == 0 a kept res
    // only adds its blocks (as zeros)
    std::map<uint64_t, std::vector<int64_t>> blocks;
    const size_t nsrc = src.size() + (res_in ? 1 : 0);
    auto visit = [&](const Meta& t, size_t j) {
      for (int64_t q = 0; q < t.nblk; ++q) {
        auto& v = blocks[t.blk_idx(&t.coords[q * t.rank])];
        if (v.empty()) v.assign(nsrc, -1);
        v[j] = q;
      }
    };
    for (size_t j = 0; j < src.size(); ++j) visit(*src[j], j);
    if (res_in) visit(rm, src.size());
    Meta& O = h->out;
    O = m[0];
    O.coords.clear();
    for (auto& kv : blocks) {
      const size_t j = std::find_if(kv.second.begin(), kv.second.end(), [](int64_t x) { return x >= 0; }) -
                       kv.second.begin();
      const Meta& t = j < src.size() ? *src[j] : rm;
      O.coords.insert(O.coords.end(), t.coords.begin() + kv.second[j] * t.rank,
                      t.coords.begin() + (kv.second[j] + 1) * t.rank);
    }
    O.nblk = (int64_t)blocks.size();
    O.refresh_offsets();
    h->used.assign(n + 1, 0);
    h->same.assign(n + 1, 0);
    auto same_topology = [&](const Meta& t) { return t.nblk == O.nblk && t.coords == O.coords; };
    for (int i = 0; i < n; ++i) h->same[i] = same_topology(m[i]) ? 1 : 0;
    if (res) h->same[n] = same_topology(rm) ? 1 : 0;
    int64_t q = 0;
    for (auto& kv : blocks) {
      const int64_t size = O.blk_size(q);
      for (int64_t e = 0; e < size; e += kLincombChunk) {
        LincombItem it{O.offsets[q] + e, (int32_t)std::min<int64_t>(kLincombChunk, size - e),
                       (int32_t)h->srcs.size(), 0, 0};
        for (size_t j = 0; j < src.size(); ++j)
          if (kv.second[j] >= 0) {
            h->srcs.push_back(LincombSrc{src[j]->offsets[kv.second[j]] + e, ord[j], 0});
            h->used[ord[j]] = 1;
          }
        if (res_in && beta_nz && kv.second[src.size()] >= 0) {
          h->srcs.push_back(LincombSrc{rm.offsets[kv.second[src.size()]] + e, kLincombMax, 0});
          h->used[n] = 1;
        }
        it.c1 = (int32_t)h->srcs.size();
        h->items.push_back(it);
      }
      ++q;
    }
    QLTG_CHECK(h->items.size() < ((size_t)1 << 31) && h->srcs.size() < ((size_t)1 << 31), QLTG_ERR_UNSUPPORTED,
               "linear combination too large");
    cudaStream_t s;
    QLTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    h->d_items = upload(h->items, s);
    h->d_srcs = upload(h->srcs, s);
    QLTG_CUDA(cudaStreamSynchronize(s));
    QLTG_CUDA(cudaStreamDestroy(s));
    *plan = h.release();
  });
}

int qltg_lincomb_plan_result(const qltg_lincomb_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    if (rank) *rank = plan->out.rank;
    if (nblk) *nblk = plan->out.nblk;
    if (size) *size = plan->out.size;
  });
}

int qltg_lincomb_plan_result_blocks(const qltg_lincomb_plan* plan, int64_t* coords, int64_t* offsets) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    plan->out.export_arrays(nullptr, nullptr, nullptr, nullptr, coords, offsets);
  });
}

int qltg_lincomb_exec(qltg_lincomb_plan* plan, const void* const* tens_dev, const void* res_dev, void* out_dev,
                      void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan && tens_dev && out_dev, QLTG_ERR_INVALID, "null argument");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    const int n = plan->n;
    for (int i = 0; i < n; ++i) {
      QLTG_CHECK(!plan->used[i] || tens_dev[i], QLTG_ERR_INVALID, "null device buffer of a combined tensor");
      // an output written over an input must have that input's layout (each element reads
      // only its own position)
      QLTG_CHECK(!(plan->used[i] && tens_dev[i] == out_dev && !plan->same[i]), QLTG_ERR_INVALID,
                 "output aliases a combined tensor of another block layout");
    }
    QLTG_CHECK(!plan->used[n] || res_dev, QLTG_ERR_INVALID, "null result buffer with beta != 0");
    QLTG_CHECK(!(plan->used[n] && res_dev == out_dev && !plan->same[n]), QLTG_ERR_INVALID,
               "result expanded to new blocks cannot be written in place");
    const int ni = (int)plan->items.size();
    if (!ni) return;
    const int grid = std::min(ni, std::max(1, plan->ctx->num_sms) * 8);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (plan->out.dtype == QLTG_C128) {
      LincombArgs<double2> a{};
      for (int i = 0; i < n; ++i) {
        a.src[i] = static_cast<const double2*>(tens_dev[i]);
        a.coef[i] = make_double2(plan->coefs[2 * i], plan->coefs[2 * i + 1]);
      }
      a.src[kLincombMax] = static_cast<const double2*>(res_dev);
      a.coef[kLincombMax] = make_double2(plan->coefs[2 * n], plan->coefs[2 * n + 1]);
      k_lincomb<double2><<<grid, 256, 0, s>>>(plan->d_items.as<LincombItem>(), ni, plan->d_srcs.as<LincombSrc>(), a,
                                              static_cast<double2*>(out_dev));
    } else {
      LincombArgs<double> a{};
      for (int i = 0; i < n; ++i) {
        a.src[i] = static_cast<const double*>(tens_dev[i]);
        a.coef[i] = plan->coefs[2 * i];
      }
      a.src[kLincombMax] = static_cast<const double*>(res_dev);
      a.coef[kLincombMax] = plan->coefs[2 * n];
      k_lincomb<double><<<grid, 256, 0, s>>>(plan->d_items.as<LincombItem>(), ni, plan->d_srcs.as<LincombSrc>(), a,
                                             static_cast<double*>(out_dev));
    }
    QLTG_CUDA(cudaGetLastError());
  });
}

int qltg_lincomb_plan_destroy(qltg_lincomb_plan* plan) {
  return guarded([&] { delete plan; });
}
