// Contiguous-axes contraction and its accumulating form.
//
// ContractContiguousAxes<ASide, BSide>(A, B, a_start, b_start, n, C)
// (tensor_manipulation/contract_contiguous_axes.h:849-868) contracts A's axes
// (a_start + i) mod rank_A with B's (b_start + i) mod rank_B; C's legs are A's saved legs
// then B's, each in cyclic order from the end of its contracted range. The sides only tell
// the reference which matrix view needs no transpose; the result does not depend on them.
// Here it is the generic plan with that saved-leg order (plan.cu applies the fermionic sign
// of the reordering).
//
// ContractTailHeadContiguousAccumulate / TryContractTailHeadContiguousAccumulate
// (contract_contiguous_axes.h:953-1040, executor :333-472, :557-783):
//   C = beta C + alpha A.B
// An existing C must have the contraction's indexes; its blocks may be a superset (extra
// blocks are only scaled by beta). Blocks the contraction needs and C lacks expand C to the
// union topology (new blocks get alpha A.B: an effective beta of 0), unless the caller asks
// for the no-expansion form, which then reports QLTG_ERR_LAYOUT. A default C needs beta = 0.
// beta = 0 never reads C.
//
// GB300 form: the contraction runs into a scratch buffer through the grouped kernels (FP64 or
// split precision), then one streaming kernel writes every output element once from
// (old C, scratch) over the union topology. The reference's point of accumulating without a
// temporary is host memory; on this GPU the scratch is one more pass over the contraction's
// result at HBM bandwidth.
#include <algorithm>
#include <map>
#include <memory>

#include "ctrct.h"
#include "split.h"

namespace qltg {
namespace {

// One work item of the combine kernel: up to kAccumChunk consecutive elements of one output
// block, with the matching element offsets in the old C and in the contraction result (-1:
// absent).
struct AccumItem {
  int64_t out_off, old_off, t_off;
  int32_t n, pad;
};
constexpr int kAccumChunk = 4096;

__device__ __forceinline__ double cmul(double a, double x) { return a * x; }
__device__ __forceinline__ double2 cmul(double2 a, double2 x) {
  return make_double2(fma(a.x, x.x, -a.y * x.y), fma(a.x, x.y, a.y * x.x));
}
__device__ __forceinline__ double cadd(double a, double b) { return a + b; }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double czero(double) { return 0.0; }
__device__ __forceinline__ double2 czero(double2) { return make_double2(0.0, 0.0); }

template <typename T>
__global__ void __launch_bounds__(256) k_accum_combine(const AccumItem* __restrict__ items, int nitems,
                                                       const T* __restrict__ old, const T* __restrict__ t,
                                                       T* __restrict__ out, T alpha, T beta, int read_old) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const AccumItem w = items[it];
    for (int e = threadIdx.x; e < w.n; e += blockDim.x) {
      T v = czero(T());
      if (read_old && w.old_off >= 0) v = cmul(beta, old[w.old_off + e]);
      if (w.t_off >= 0) v = cadd(v, cmul(alpha, t[w.t_off + e]));
      out[w.out_off + e] = v;
    }
  }
}


// Contracted axes and cyclic saved orders of a contiguous-axes contraction.
void contiguous_plan_axes(CtrctPlan& p, int64_t a0, int64_t b0, int32_t n) {
  const int ra = p.a.rank, rb = p.b.rank;
  QLTG_CHECK(n >= 1 && n <= ra && n <= rb, QLTG_ERR_INVALID, "contracted range length out of bounds");
  QLTG_CHECK(a0 >= 0 && a0 < ra && b0 >= 0 && b0 < rb, QLTG_ERR_INVALID, "contracted range start out of bounds");
  p.axa.clear();
  p.axb.clear();
  p.sa_order.clear();
  p.sb_order.clear();
  for (int i = 0; i < n; ++i) {
    p.axa.push_back((a0 + i) % ra);
    p.axb.push_back((b0 + i) % rb);
  }
  for (int i = 0; i < ra - n; ++i) p.sa_order.push_back((a0 + n + i) % ra);
  for (int i = 0; i < rb - n; ++i) p.sb_order.push_back((b0 + n + i) % rb);
}

void build_contiguous(CtrctPlan& p, qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b,
                      int64_t a0, int64_t b0, int32_t n) {
  p.ctx = ctx;
  p.a = meta_from_desc(a);
  p.b = meta_from_desc(b);
  contiguous_plan_axes(p, a0, b0, n);
  cudaStream_t s;
  QLTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  try {
    plan_contraction(p, s);
    finalize_plan(p, s);
  } catch (...) {
    cudaStreamDestroy(s);
    throw;
  }
  QLTG_CUDA(cudaStreamDestroy(s));
}

}  // namespace
}  // namespace qltg

struct qltg_accum_plan {
  qltg_ctx* ctx = nullptr;
  qltg::CtrctPlan ctr;            // T = A . B (contiguous axes)
  qltg::Meta out;                 // output topology
  bool has_c_in = false, expanded = false;
  std::vector<qltg::AccumItem> items;
  qltg::DevBuf d_items, t_buf;
};

using namespace qltg;

extern "C" {

int qltg_ctrct_plan_create_contiguous(qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b,
                                      int64_t a_start, int64_t b_start, int32_t n, int32_t a_side, int32_t b_side,
                                      qltg_ctrct_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    QLTG_CHECK((a_side == QLTG_SIDE_HEAD || a_side == QLTG_SIDE_TAIL) &&
                   (b_side == QLTG_SIDE_HEAD || b_side == QLTG_SIDE_TAIL),
               QLTG_ERR_INVALID, "side must be QLTG_SIDE_HEAD or QLTG_SIDE_TAIL");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_ctrct_plan>();
    build_contiguous(h->p, ctx, a, b, a_start, b_start, n);
    *plan = h.release();
  });
}

int qltg_accum_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b, int64_t a_start,
                           int64_t b_start, int32_t n, const qltg_tensor_desc* c_in, int32_t allow_expand,
                           qltg_accum_plan** plan, int32_t* expanded) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_accum_plan>();
    h->ctx = ctx;
    build_contiguous(h->ctr, ctx, a, b, a_start, b_start, n);
    const Meta& T = h->ctr.c;
    Meta cm;
    std::map<uint64_t, std::pair<int64_t, int64_t>> blocks;   // blk_idx -> (ordinal in C_in, in T)
    if (c_in) {
      cm = meta_from_desc(c_in);
      QLTG_CHECK(same_indexes(cm, T), QLTG_ERR_LAYOUT, "output indexes are not those of the contraction result");
      h->has_c_in = true;
      for (int64_t q = 0; q < cm.nblk; ++q) blocks[cm.rank ? cm.blk_idx(&cm.coords[q * cm.rank]) : 0] = {q, -1};
    }
    bool missing = false;
    for (int64_t q = 0; q < T.nblk; ++q) {
      const uint64_t k = T.rank ? T.blk_idx(&T.coords[q * T.rank]) : 0;
      auto it = blocks.find(k);
      if (it == blocks.end()) {
        blocks[k] = {-1, q};
        missing = true;
      } else {
        it->second.second = q;
      }
    }
    h->expanded = h->has_c_in && missing;
    QLTG_CHECK(!(h->expanded && !allow_expand), QLTG_ERR_LAYOUT,
               "output lacks blocks of the contraction result and expansion is not allowed");
    Meta& O = h->out;
    O = h->has_c_in ? cm : T;
    if (h->expanded) {   // union topology, ascending block index
      O.coords.clear();
      for (auto& kv : blocks) {
        const Meta& src = kv.second.first >= 0 ? cm : T;
        const int64_t ord = kv.second.first >= 0 ? kv.second.first : kv.second.second;
        O.coords.insert(O.coords.end(), src.coords.begin() + ord * O.rank, src.coords.begin() + (ord + 1) * O.rank);
      }
      O.nblk = (int64_t)blocks.size();
      O.refresh_offsets();
    }
    // combine work items over the output blocks
    auto add = [&](int64_t out_off, int64_t old_off, int64_t t_off, int64_t size) {
      for (int64_t e = 0; e < size; e += kAccumChunk)
        h->items.push_back(AccumItem{out_off + e, old_off >= 0 ? old_off + e : -1, t_off >= 0 ? t_off + e : -1,
                                     (int32_t)std::min<int64_t>(kAccumChunk, size - e), 0});
    };
    if (O.rank == 0) {   // scalar: always one value
      O.nblk = 1;
      O.size = 1;
      O.offsets.assign(1, 0);
      O.coords.clear();
      add(0, h->has_c_in && cm.size > 0 ? 0 : -1, T.size > 0 ? 0 : -1, 1);
    } else {
      int64_t q = 0;
      for (auto& kv : blocks) {
        const int64_t o = kv.second.first, t = kv.second.second;
        if (!h->has_c_in || h->expanded || o >= 0) {
          const int64_t out_q = h->expanded ? q : (h->has_c_in ? o : t);
          add(O.offsets[out_q], o >= 0 ? cm.offsets[o] : -1, t >= 0 ? T.offsets[t] : -1, O.blk_size(out_q));
        }
        ++q;
      }
    }
    if (expanded) *expanded = h->expanded ? 1 : 0;
    cudaStream_t s;
    QLTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    h->d_items = upload(h->items, s);
    QLTG_CUDA(cudaStreamSynchronize(s));
    QLTG_CUDA(cudaStreamDestroy(s));
    h->t_buf.alloc(std::max<int64_t>(T.size, 1) * T.elem_bytes());
    *plan = h.release();
  });
}

int qltg_accum_plan_result(const qltg_accum_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    if (rank) *rank = plan->out.rank;
    if (nblk) *nblk = plan->out.nblk;
    if (size) *size = plan->out.size;
  });
}

int qltg_accum_plan_result_blocks(const qltg_accum_plan* plan, int64_t* coords, int64_t* offsets) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    plan->out.export_arrays(nullptr, nullptr, nullptr, nullptr, coords, offsets);
  });
}

int qltg_accum_exec(qltg_accum_plan* plan, const void* a_dev, const void* b_dev, const void* c_in_dev,
                    void* c_out_dev, const double* alpha, const double* beta, int32_t mode, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan && a_dev && b_dev && c_out_dev && alpha && beta, QLTG_ERR_INVALID, "null argument");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    const bool cplx = plan->out.dtype == QLTG_C128;
    QLTG_CHECK(cplx || (alpha[1] == 0.0 && beta[1] == 0.0), QLTG_ERR_INVALID,
               "complex alpha or beta for a real tensor");
    const bool beta_zero = beta[0] == 0.0 && beta[1] == 0.0;
    QLTG_CHECK(plan->has_c_in || beta_zero, QLTG_ERR_INVALID, "accumulating into a default output needs beta == 0");
    QLTG_CHECK(!plan->has_c_in || beta_zero || c_in_dev, QLTG_ERR_INVALID, "null c_in_dev with nonzero beta");
    QLTG_CHECK(c_out_dev != a_dev && c_out_dev != b_dev, QLTG_ERR_INVALID, "output aliases an input");
    QLTG_CHECK(!(plan->expanded && c_in_dev && c_out_dev == c_in_dev), QLTG_ERR_INVALID,
               "an expanded output cannot be written over the input output");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (plan->ctr.c.size > 0) exec_contraction(plan->ctr, a_dev, b_dev, plan->t_buf.get(), mode, s);
    const int ni = (int)plan->items.size();
    if (!ni) return;
    const int grid = std::min(ni, std::max(1, plan->ctx->num_sms) * 8);
    const int read_old = beta_zero ? 0 : 1;
    if (cplx)
      k_accum_combine<double2><<<grid, 256, 0, s>>>(
          plan->d_items.as<AccumItem>(), ni, static_cast<const double2*>(c_in_dev), plan->t_buf.as<double2>(),
          static_cast<double2*>(c_out_dev), make_double2(alpha[0], alpha[1]), make_double2(beta[0], beta[1]), read_old);
    else
      k_accum_combine<double><<<grid, 256, 0, s>>>(plan->d_items.as<AccumItem>(), ni,
                                                   static_cast<const double*>(c_in_dev), plan->t_buf.as<double>(),
                                                   static_cast<double*>(c_out_dev), alpha[0], beta[0], read_old);
    QLTG_CUDA(cudaGetLastError());
  });
}

int qltg_accum_plan_device_status(qltg_accum_plan* plan, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    QLTG_CHECK(split_device_error(plan->ctr, static_cast<cudaStream_t>(stream)) == 0, QLTG_ERR_TIMEOUT,
               "a bounded tensor-core wait expired in the split-precision GEMM");
  });
}

int qltg_accum_plan_destroy(qltg_accum_plan* plan) {
  delete plan;
  return QLTG_OK;
}

}  // extern "C"
