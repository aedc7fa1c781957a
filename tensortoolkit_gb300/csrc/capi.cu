// C ABI: contexts, error reporting, descriptor validation, contraction and transpose.
#include <algorithm>
#include <memory>
#include <numeric>

#include "ctrct.h"
#include "split.h"

namespace qltg {

namespace {
thread_local std::string t_last_error;
}

void set_last_error(const std::string& msg) { t_last_error = msg; }

void Meta::refresh_offsets() {
  offsets.resize(nblk);
  int64_t off = 0;
  for (int64_t b = 0; b < nblk; ++b) { offsets[b] = off; off += blk_size(b); }
  size = off;
}

void Meta::export_arrays(int32_t* d, int32_t* ns, int32_t* q, int64_t* dm, int64_t* c, int64_t* o) const {
  int64_t qp = 0, dp = 0;
  for (int l = 0; l < rank; ++l) {
    if (d) d[l] = dirs[l];
    if (ns) ns[l] = (int32_t)dims[l].size();
    if (q) for (auto x : qns[l]) q[qp++] = x;
    if (dm) for (auto x : dims[l]) dm[dp++] = x;
  }
  if (c) std::copy(coords.begin(), coords.end(), c);
  if (o) std::copy(offsets.begin(), offsets.end(), o);
}

Meta meta_from_desc(const qltg_tensor_desc* d) {
  QLTG_CHECK(d != nullptr, QLTG_ERR_INVALID, "null tensor descriptor");
  Meta m;
  QLTG_CHECK(d->rank >= 0 && d->rank <= kMaxRank, QLTG_ERR_UNSUPPORTED, "tensor rank outside 0..8");
  QLTG_CHECK(d->dtype == QLTG_F64 || d->dtype == QLTG_C128, QLTG_ERR_INVALID, "unknown element type");
  QLTG_CHECK(d->qn_ncomp >= 1 && d->qn_ncomp <= 4, QLTG_ERR_INVALID, "qn_ncomp outside 1..4");
  QLTG_CHECK(d->parity_comp >= -1 && d->parity_comp < d->qn_ncomp, QLTG_ERR_INVALID, "parity_comp out of range");
  QLTG_CHECK(d->nblk >= 0, QLTG_ERR_INVALID, "negative block count");
  m.rank = d->rank;
  m.dtype = d->dtype;
  m.ncomp = d->qn_ncomp;
  m.parity_comp = d->parity_comp;
  m.nblk = d->nblk;
  if (m.rank == 0) {
    QLTG_CHECK(m.nblk <= 1, QLTG_ERR_INVALID, "a scalar tensor holds at most one block");
    m.refresh_offsets();
    return m;
  }
  QLTG_CHECK(d->dirs && d->nsct && d->qns && d->dims, QLTG_ERR_INVALID, "null leg arrays in descriptor");
  QLTG_CHECK(m.nblk == 0 || d->coords, QLTG_ERR_INVALID, "null block coordinates");
  int64_t qp = 0, dp = 0;
  for (int l = 0; l < m.rank; ++l) {
    QLTG_CHECK(d->dirs[l] == QLTG_IN || d->dirs[l] == QLTG_OUT, QLTG_ERR_INVALID, "leg direction must be IN or OUT");
    QLTG_CHECK(d->nsct[l] >= 1, QLTG_ERR_INVALID, "a leg needs at least one sector");
    m.dirs.push_back(d->dirs[l]);
    m.qns.emplace_back(d->qns + qp, d->qns + qp + (int64_t)d->nsct[l] * m.ncomp);
    m.dims.emplace_back(d->dims + dp, d->dims + dp + d->nsct[l]);
    for (auto x : m.dims.back()) QLTG_CHECK(x >= 1, QLTG_ERR_INVALID, "sector degeneracy must be >= 1");
    qp += (int64_t)d->nsct[l] * m.ncomp;
    dp += d->nsct[l];
  }
  m.coords.assign(d->coords, d->coords + m.nblk * m.rank);
  for (int64_t b = 0; b < m.nblk; ++b)
    for (int l = 0; l < m.rank; ++l) {
      const int64_t c = m.coords[b * m.rank + l];
      QLTG_CHECK(c >= 0 && c < m.nsct(l), QLTG_ERR_INVALID, "block coordinate out of range");
    }
  for (int64_t b = 1; b < m.nblk; ++b)
    QLTG_CHECK(m.blk_idx(&m.coords[(b - 1) * m.rank]) < m.blk_idx(&m.coords[b * m.rank]), QLTG_ERR_INVALID,
               "blocks must be unique and in ascending block index order");
  m.refresh_offsets();
  return m;
}

bool same_leg(const Meta& a, int la, const Meta& b, int lb) {
  return a.dirs[la] == b.dirs[lb] && a.qns[la] == b.qns[lb] && a.dims[la] == b.dims[lb];
}

bool inverse_leg(const Meta& a, int la, const Meta& b, int lb) {
  return a.dirs[la] != b.dirs[lb] && a.qns[la] == b.qns[lb] && a.dims[la] == b.dims[lb];
}

bool same_indexes(const Meta& x, const Meta& y) {
  if (x.rank != y.rank || x.dtype != y.dtype || x.ncomp != y.ncomp || x.parity_comp != y.parity_comp) return false;
  for (int l = 0; l < x.rank; ++l)
    if (!same_leg(x, l, y, l)) return false;
  return true;
}


// FermionicInplaceReorder (reference utility/utils_inl.h:52-75): sign of moving the legs
// into `order` by the cycle-following in-place reorder, counting odd legs passed over.
int reorder_sign(std::vector<uint8_t> par, const std::vector<int>& order) {
  std::vector<int> idx(order);
  int ex = 0;
  for (int i = 0; i < (int)idx.size(); ++i) {
    int cur = i;
    while (i != idx[cur]) {
      const int nxt = idx[cur];
      int between = 0;
      for (int j = std::min(cur, nxt) + 1; j < std::max(cur, nxt); ++j) between += par[j];
      ex += between * (par[cur] + par[nxt]) + par[cur] * par[nxt];
      std::swap(par[cur], par[nxt]);
      idx[cur] = cur;
      cur = nxt;
    }
    idx[cur] = cur;
  }
  return (ex & 1) ? -1 : 1;
}

// Destination layout of QLTensor::Transpose: blocks in ascending block index of the permuted
// sector counts, each multiplied by its FermionicInplaceReorder sign.
void transpose_layout(const Meta& m, const std::vector<int>& order, std::vector<double>& signs,
                      std::vector<int64_t>& dst_off) {
  std::vector<std::pair<uint64_t, int64_t>> keyed(m.nblk);
  signs.assign(m.nblk, 1.0);
  for (int64_t b = 0; b < m.nblk; ++b) {
    uint64_t idx = 0;
    for (int i = 0; i < m.rank; ++i) idx = idx * (uint64_t)m.nsct(order[i]) + (uint64_t)m.coords[b * m.rank + order[i]];
    keyed[b] = {idx, b};
    if (m.parity_comp >= 0) {
      std::vector<uint8_t> par(m.rank);
      for (int l = 0; l < m.rank; ++l) par[l] = m.parity(l, m.coords[b * m.rank + l]);
      signs[b] = reorder_sign(par, order);
    }
  }
  std::sort(keyed.begin(), keyed.end());
  dst_off.assign(m.nblk, 0);
  int64_t off = 0;
  for (auto& kv : keyed) { dst_off[kv.second] = off; off += m.blk_size(kv.second); }
}

}  // namespace qltg

using namespace qltg;

extern "C" {

const char* qltg_last_error(void) { return t_last_error.c_str(); }

int qltg_create(int device, qltg_ctx** ctx) {
  return guarded([&] {
    QLTG_CHECK(ctx != nullptr, QLTG_ERR_INVALID, "null ctx out-pointer");
    int n = 0;
    QLTG_CUDA(cudaGetDeviceCount(&n));
    QLTG_CHECK(device >= 0 && device < n, QLTG_ERR_INVALID, "no such CUDA device");
    QLTG_CUDA(cudaSetDevice(device));
    auto* c = new qltg_ctx;
    c->device = device;
    cudaDeviceProp prop;
    QLTG_CUDA(cudaGetDeviceProperties(&prop, device));
    c->num_sms = prop.multiProcessorCount;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    *ctx = c;
  });
}

int qltg_destroy(qltg_ctx* ctx) {
  delete ctx;
  return QLTG_OK;
}

int qltg_ctrct_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* a, const qltg_tensor_desc* b,
                           const int64_t* axes_a, const int64_t* axes_b, int32_t naxes, qltg_ctrct_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    QLTG_CHECK(naxes >= 0 && naxes <= kMaxRank, QLTG_ERR_INVALID, "naxes out of range");
    QLTG_CHECK(naxes == 0 || (axes_a && axes_b), QLTG_ERR_INVALID, "null axes");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_ctrct_plan>();
    CtrctPlan& p = h->p;
    p.ctx = ctx;
    p.a = meta_from_desc(a);
    p.b = meta_from_desc(b);
    p.axa.assign(axes_a, axes_a + naxes);
    p.axb.assign(axes_b, axes_b + naxes);
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
    *plan = h.release();
  });
}

int qltg_ctrct_plan_result(const qltg_ctrct_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    if (rank) *rank = plan->p.c.rank;
    if (nblk) *nblk = plan->p.c.nblk;
    if (size) *size = plan->p.c.size;
  });
}

int qltg_ctrct_plan_result_blocks(const qltg_ctrct_plan* plan, int64_t* coords, int64_t* offsets) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    plan->p.c.export_arrays(nullptr, nullptr, nullptr, nullptr, coords, offsets);
  });
}

int qltg_ctrct_plan_tasks(const qltg_ctrct_plan* plan, int64_t* ntasks, int64_t* tasks) {
  return guarded([&] {
    QLTG_CHECK(plan && ntasks, QLTG_ERR_INVALID, "null plan or ntasks");
    *ntasks = (int64_t)plan->p.tasks_gen.size() / 8;
    if (tasks) std::copy(plan->p.tasks_gen.begin(), plan->p.tasks_gen.end(), tasks);
  });
}

int qltg_ctrct_plan_stats(const qltg_ctrct_plan* plan, double* flops, double* bytes) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    if (flops) *flops = plan->p.flops;
    if (bytes) *bytes = plan->p.bytes;
  });
}

int qltg_ctrct_exec(qltg_ctrct_plan* plan, const void* a_dev, const void* b_dev, void* c_dev, int32_t mode,
                    void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    QLTG_CUDA(cudaSetDevice(plan->p.ctx->device));
    exec_contraction(plan->p, a_dev, b_dev, c_dev, mode, static_cast<cudaStream_t>(stream));
  });
}

int qltg_ctrct_exec_stage(qltg_ctrct_plan* plan, const void* a_dev, const void* b_dev, void* c_dev, int32_t mode,
                          int32_t stage, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    QLTG_CUDA(cudaSetDevice(plan->p.ctx->device));
    exec_contraction(plan->p, a_dev, b_dev, c_dev, mode, static_cast<cudaStream_t>(stream), stage);
  });
}

int qltg_ctrct_plan_device_status(qltg_ctrct_plan* plan, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    QLTG_CUDA(cudaSetDevice(plan->p.ctx->device));
    QLTG_CHECK(split_device_error(plan->p, static_cast<cudaStream_t>(stream)) == 0, QLTG_ERR_TIMEOUT,
               "a bounded tensor-core wait expired in the split-precision GEMM");
  });
}

int qltg_ctrct_plan_destroy(qltg_ctrct_plan* plan) {
  delete plan;
  return QLTG_OK;
}

int qltg_ctrct_plan_set_schedule(qltg_ctrct_plan* plan, int32_t f64_tile_rows, int32_t split_stack, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    QLTG_CHECK(f64_tile_rows == 0 || f64_tile_rows == 32 || f64_tile_rows == 64, QLTG_ERR_INVALID,
               "f64_tile_rows must be 0, 32 or 64");
    QLTG_CHECK(split_stack >= -1 && split_stack <= 1, QLTG_ERR_INVALID, "split_stack must be -1, 0 or 1");
    QLTG_CUDA(cudaSetDevice(plan->p.ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CtrctPlan& p = plan->p;
    if (f64_tile_rows) set_f64_tile(p, f64_tile_rows, 32, s);
    if (split_stack >= 0) {
      TuneChoice c;
      c.f64_bm = p.sched.bm;
      c.split_stack = split_stack != 0;
      if (p.split) apply_choice(p, QLTG_MODE_SPLIT, c, s);
      else p.split_cfg.stack = c.split_stack;
    }
  });
}

int qltg_ctrct_plan_get_schedule(const qltg_ctrct_plan* plan, int32_t* f64_tile_rows, int32_t* split_stack,
                                 int32_t* tuned, float* ms) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    const CtrctPlan& p = plan->p;
    if (f64_tile_rows) *f64_tile_rows = p.sched.bm;
    if (split_stack) *split_stack = p.split_cfg.stack ? 1 : 0;
    for (int m = 0; m < 2; ++m) {
      if (tuned) tuned[m] = p.is_tuned[m] ? 1 : 0;
      if (ms) {
        ms[2 * m] = p.tuned[m].ms;
        ms[2 * m + 1] = p.tuned[m].other_ms;
      }
    }
  });
}

int qltg_ctrct_plan_split_stats(const qltg_ctrct_plan* plan, int64_t* tile_stages, double* useful_frac) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    const bool has = plan->p.split && plan->p.split->built;
    if (tile_stages) *tile_stages = has ? plan->p.split->tile_stages : 0;
    if (useful_frac) *useful_frac = has ? plan->p.split->useful_frac : 0.0;
  });
}

int qltg_ctrct_plan_tune(qltg_ctrct_plan* plan, const void* a_dev, const void* b_dev, void* c_dev, int32_t mode,
                         void* stream, int32_t* from_cache) {
  return guarded([&] {
    QLTG_CHECK(plan && a_dev && b_dev && c_dev, QLTG_ERR_INVALID, "null plan or buffer");
    QLTG_CUDA(cudaSetDevice(plan->p.ctx->device));
    bool cached = false;
    tune_plan(plan->p, a_dev, b_dev, c_dev, mode, static_cast<cudaStream_t>(stream), &cached);
    if (from_cache) *from_cache = cached ? 1 : 0;
  });
}

int qltg_transpose(qltg_ctx* ctx, const qltg_tensor_desc* a, const void* src_dev, const int32_t* perm,
                   void* dst_dev, void* stream) {
  return guarded([&] {
    QLTG_CHECK(ctx, QLTG_ERR_INVALID, "null ctx");
    Meta m = meta_from_desc(a);
    if (m.rank == 0 || m.nblk == 0) return;
    QLTG_CHECK(perm && src_dev && dst_dev, QLTG_ERR_INVALID, "null perm or buffer");
    QLTG_CHECK(src_dev != dst_dev, QLTG_ERR_INVALID, "in-place transpose is not supported");
    std::vector<int> order(perm, perm + m.rank);
    {
      std::vector<int> chk(order);
      std::sort(chk.begin(), chk.end());
      for (int i = 0; i < m.rank; ++i) QLTG_CHECK(chk[i] == i, QLTG_ERR_INVALID, "perm is not a permutation");
    }
    QLTG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<double> signs;
    std::vector<int64_t> dst_off;
    transpose_layout(m, order, signs, dst_off);
    TransposeList tl;
    tl.build(m, order, signs, &dst_off, s);
    tl.launch(src_dev, dst_dev, (int)m.elem_bytes(), s);
    // the work list is freed on return: wait for the kernel that reads it
    QLTG_CUDA(cudaStreamSynchronize(s));
  });
}

int qltg_transpose_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* a, const int32_t* perm, void* stream,
                               qltg_transpose_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    Meta m = meta_from_desc(a);
    QLTG_CHECK(m.rank == 0 || perm, QLTG_ERR_INVALID, "null perm");
    std::vector<int> order(perm, perm + m.rank);
    {
      std::vector<int> chk(order);
      std::sort(chk.begin(), chk.end());
      for (int i = 0; i < m.rank; ++i) QLTG_CHECK(chk[i] == i, QLTG_ERR_INVALID, "perm is not a permutation");
    }
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_transpose_plan>();
    h->ctx = ctx;
    h->elem_bytes = (int)m.elem_bytes();
    if (m.rank && m.nblk) {
      std::vector<double> signs;
      std::vector<int64_t> dst_off;
      transpose_layout(m, order, signs, dst_off);
      h->tl.build(m, order, signs, &dst_off, static_cast<cudaStream_t>(stream));
      QLTG_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    }
    *plan = h.release();
  });
}

int qltg_transpose_plan_exec(qltg_transpose_plan* plan, const void* src_dev, void* dst_dev, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    if (plan->tl.ntiles == 0) return;
    QLTG_CHECK(src_dev && dst_dev && src_dev != dst_dev, QLTG_ERR_INVALID, "null or identical buffers");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    plan->tl.launch(src_dev, dst_dev, plan->elem_bytes, static_cast<cudaStream_t>(stream));
  });
}

int qltg_transpose_plan_destroy(qltg_transpose_plan* plan) {
  delete plan;
  return QLTG_OK;
}

int qltg_transpose_noalloc(qltg_ctx* ctx, const qltg_tensor_desc* a, const void* src_dev, const int32_t* perm,
                           void* dst_dev, void* stream) {
  return guarded([&] {
    QLTG_CHECK(ctx, QLTG_ERR_INVALID, "null ctx");
    Meta m = meta_from_desc(a);
    if (m.rank == 0 || m.nblk == 0) return;
    QLTG_CHECK(perm && src_dev && dst_dev, QLTG_ERR_INVALID, "null perm or buffer");
    QLTG_CHECK(src_dev != dst_dev, QLTG_ERR_INVALID, "in-place transpose is not supported");
    QLTG_CHECK(m.nblk <= kNoAllocPermBlocks, QLTG_ERR_INVALID,
               "qltg_transpose_noalloc: at most 4096 blocks per call (use qltg_transpose)");
    std::vector<int> order(perm, perm + m.rank);
    {
      std::vector<int> chk(order);
      std::sort(chk.begin(), chk.end());
      for (int i = 0; i < m.rank; ++i) QLTG_CHECK(chk[i] == i, QLTG_ERR_INVALID, "perm is not a permutation");
    }
    QLTG_CUDA(cudaSetDevice(ctx->device));
    std::vector<double> signs;
    std::vector<int64_t> dst_off;
    transpose_layout(m, order, signs, dst_off);
    TransposeList tl;
    tl.describe(m, order, signs, &dst_off);
    launch_permute_noalloc(ctx->device, tl, src_dev, dst_dev, (int)m.elem_bytes(), static_cast<cudaStream_t>(stream));
  });
}

}  // extern "C"

extern "C" int qltg_selftest_bounded_wait(qltg_ctx* ctx, int64_t limit_cycles, void* stream) {
  return qltg::guarded([&] {
    QLTG_CHECK(ctx, QLTG_ERR_INVALID, "null ctx");
    QLTG_CHECK(limit_cycles >= 1 && limit_cycles <= ((int64_t)1 << 31), QLTG_ERR_INVALID,
               "wait limit must be 1 .. 2^31 cycles");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    const int expired = qltg::wait_selftest(limit_cycles, static_cast<cudaStream_t>(stream));
    QLTG_CHECK(expired == 0 || expired == 1, QLTG_ERR_CUDA, "self-test kernel did not report");
    QLTG_CHECK(!expired, QLTG_ERR_TIMEOUT, "the bounded wait expired after its limit, as intended");
  });
}

extern "C" int qltg_selftest_fp64_rates(qltg_ctx* ctx, double* dfma_tflops, double* dmma_tflops, void* stream) {
  return qltg::guarded([&] {
    QLTG_CHECK(ctx && dfma_tflops && dmma_tflops, QLTG_ERR_INVALID, "null ctx or out-pointer");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    qltg::fp64_rates(ctx->num_sms, static_cast<cudaStream_t>(stream), dfma_tflops, dmma_tflops);
  });
}
