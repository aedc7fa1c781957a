// Two-site effective-Hamiltonian matvec: four planned contractions captured as one CUDA
// graph.
//
// The reference's chain is four independent Contract calls, each rebuilding its task
// list on the host and issuing per-block transposes and per-task GEMMs on the default
// stream (tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257). The block
// topology of a Lanczos matvec never changes, so here the four plans (device pairing,
// schedules, operand scratch) are built once, the intermediates t1..t3 live in HBM for
// the life of the object, and the whole chain replays as one graph launch.
#include <algorithm>
#include <map>
#include <memory>

#include "matvec.h"
#include "split.h"

using namespace qltg;

namespace {

// Split mode: when every A block of the last step's slices is written by the second MPO
// step's skinny kernel in the layout the slices read (no transpose; each block's row length
// a multiple of the skinny block's n), that kernel folds the row scales while it writes them
// and the last step skips its row-scale pass.
void link_row_fields(qltg_matvec& mv, cudaStream_t s) {
  for (CtrctPlan* q : {&mv.step[2], &mv.mpo12}) {   // unlink both possible producers first
    q->d_fuse.release();
    q->fuse_fields = nullptr;
  }
  if (mv.step[3].split) mv.step[3].split->a_fields_external = false;
  mv.fused_fields = false;
  CtrctPlan& p2 = mv.mpo_producer();
  CtrctPlan& p3 = mv.step[3];
  if (!p2.split || !p3.split || p3.split->a_ops.empty() || p3.split->a_static) return;
  if (p3.a_tl.ntiles || !p2.split->tiles.empty()) return;
  // a complex operand row of the last step is the real 2k-wide view of k complex values
  const int cw = p3.a.dtype == QLTG_C128 ? 2 : 1;
  const auto& ops = p3.split->a_ops;
  std::map<int64_t, int> op_of;
  for (int i = 0; i < (int)ops.size(); ++i) op_of[ops[i].src_off & ~qltg::kFromSrc] = i;
  const qltg::GemmSchedule& g = p2.sched;
  std::vector<qltg::SkinnyFuse> fz(std::max<size_t>(g.cblk.size(), 1), qltg::SkinnyFuse{-1, 1});
  size_t covered = 0;
  for (size_t q = 0; q < g.cblk.size(); ++q) {
    auto it = op_of.find(cw * g.cblk[q].c_off);   // operand offsets count real values
    if (it == op_of.end()) continue;
    const qltg::SplitOperand& o = ops[it->second];
    if (!qltg::skinny_cblk(g, (int32_t)q) || o.cols % (cw * g.cblk[q].n) != 0 ||
        (int64_t)o.rows * o.cols != (int64_t)cw * g.cblk[q].m * g.cblk[q].n)
      return;
    fz[q] = qltg::SkinnyFuse{o.exp_off, o.cols / cw};
    ++covered;
  }
  if (covered != ops.size()) return;
  p2.d_fuse = qltg::upload(fz, s);
  QLTG_CUDA(cudaStreamSynchronize(s));
  p2.fuse_fields = p3.split->a_exps.as<int32_t>();
  p3.split->a_fields_external = true;
  mv.fused_fields = true;
}

// Median ms of `reps` runs of fn on s (after one unmeasured run).
template <typename F>
float time_ms(F&& fn, cudaStream_t s, int reps = 5) {
  fn();
  std::vector<cudaEvent_t> ev(2 * reps);
  for (auto& e : ev) QLTG_CUDA(cudaEventCreate(&e));
  for (int r = 0; r < reps; ++r) {
    QLTG_CUDA(cudaEventRecord(ev[2 * r], s));
    fn();
    QLTG_CUDA(cudaEventRecord(ev[2 * r + 1], s));
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
  std::vector<float> ms(reps);
  for (int r = 0; r < reps; ++r) cudaEventElapsedTime(&ms[r], ev[2 * r], ev[2 * r + 1]);
  for (auto e : ev) cudaEventDestroy(e);
  std::sort(ms.begin(), ms.end());
  return ms[reps / 2];
}

// Plan the fused MPO form (W12 = W1 . W2 on the device, then t1 . W12 over t1's (w, p1, p2)
// legs), check that it yields t3's exact layout, and time it against the two MPO steps.
void plan_mpo_fusion(qltg_matvec& mv, cudaStream_t s) {
  CtrctPlan wp;
  wp.ctx = mv.ctx;
  wp.a = mv.step[1].b;
  wp.b = mv.step[2].b;
  wp.axa = {3};
  wp.axb = {0};
  plan_contraction(wp, s);
  finalize_plan(wp, s);
  if (wp.c.rank != 6 || wp.c.size == 0) return;
  mv.w12.alloc(wp.c.size * wp.c.elem_bytes());
  exec_contraction(wp, mv.mpo1, mv.mpo2, mv.w12.get(), QLTG_MODE_FP64, s);
  QLTG_CUDA(cudaStreamSynchronize(s));   // W12 is final before its plan's buffers go
  CtrctPlan& f = mv.mpo12;
  f.ctx = mv.ctx;
  f.a = mv.step[0].c;
  f.b = wp.c;
  f.axa = {0, 2, 3};
  f.axb = {0, 1, 3};
  plan_contraction(f, s);
  finalize_plan(f, s);
  const Meta& t3 = mv.step[2].c;
  if (f.c.size != t3.size || f.c.nblk != t3.nblk || f.c.coords != t3.coords || f.c.offsets != t3.offsets) return;
  tune_plan(f, mv.t[0].get(), mv.w12.get(), mv.t[2].get(), mv.mode, s, nullptr);
  if (mv.mode == QLTG_MODE_SPLIT) prepare_split(f, s);
  mv.mpo_fusable = true;
  mv.mpo_fused = false;
  mv.mid_ms[0] = time_ms([&] { mv.enqueue_mid(s); }, s);
  mv.mpo_fused = true;
  mv.mid_ms[1] = time_ms([&] { mv.enqueue_mid(s); }, s);
  mv.mpo_fused = mv.mid_ms[1] < mv.mid_ms[0];
}

}  // namespace

extern "C" {

int qltg_matvec_create(qltg_ctx* ctx, const qltg_tensor_desc* lenv, const void* lenv_dev,
                       const qltg_tensor_desc* psi, const qltg_tensor_desc* mpo1, const void* mpo1_dev,
                       const qltg_tensor_desc* mpo2, const void* mpo2_dev, const qltg_tensor_desc* renv,
                       const void* renv_dev, int32_t mode, void* stream, qltg_matvec** mv) {
  return guarded([&] {
    QLTG_CHECK(ctx && mv, QLTG_ERR_INVALID, "null ctx or matvec out-pointer");
    QLTG_CHECK(lenv_dev && mpo1_dev && mpo2_dev && renv_dev, QLTG_ERR_INVALID, "null operator buffer");
    QLTG_CHECK(mode == QLTG_MODE_FP64 || mode == QLTG_MODE_SPLIT, QLTG_ERR_INVALID, "unknown arithmetic mode");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_matvec>();
    h->ctx = ctx;
    h->mode = mode;
    h->lenv = lenv_dev; h->mpo1 = mpo1_dev; h->mpo2 = mpo2_dev; h->renv = renv_dev;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    QLTG_CUDA(cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking));
    const Meta ml = meta_from_desc(lenv), mp = meta_from_desc(psi), m1 = meta_from_desc(mpo1),
               m2 = meta_from_desc(mpo2), mr = meta_from_desc(renv);
    QLTG_CHECK(ml.rank == 3 && mp.rank == 4 && m1.rank == 4 && m2.rank == 4 && mr.rank == 3, QLTG_ERR_INVALID,
               "matvec expects lenv rank 3, psi rank 4, mpo rank 4, renv rank 3");
    h->psi_size = mp.size;
    const int64_t ax[4][2][2] = {{{0, -1}, {0, -1}}, {{0, 2}, {0, 1}}, {{4, 1}, {0, 1}}, {{4, 1}, {1, 0}}};
    const int nax[4] = {1, 2, 2, 2};
    const Meta* rhs[4] = {&mp, &m1, &m2, &mr};
    for (int i = 0; i < 4; ++i) {
      CtrctPlan& p = h->step[i];
      p.ctx = ctx;
      p.a = (i == 0) ? ml : h->step[i - 1].c;
      p.b = *rhs[i];
      p.axa.assign(ax[i][0], ax[i][0] + nax[i]);
      p.axb.assign(ax[i][1], ax[i][1] + nax[i]);
      plan_contraction(p, s);
      finalize_plan(p, s);
      if (i < 3) {
        h->t[i].alloc(std::max<int64_t>(1, p.c.size) * p.c.elem_bytes());
        QLTG_CUDA(cudaMemsetAsync(h->t[i].get(), 0, std::max<int64_t>(1, p.c.size) * p.c.elem_bytes(), s));
      }
      {
        // the GEMM schedule of this step from the tuner, timed on the step's own operands
        // (psi and the result as zero-filled scratch; t0..t2 hold the earlier steps' output)
        if (i == 0) {
          h->psi_stage.alloc(std::max<int64_t>(1, mp.size) * mp.elem_bytes());
          QLTG_CUDA(cudaMemsetAsync(h->psi_stage.get(), 0, std::max<int64_t>(1, mp.size) * mp.elem_bytes(), s));
        }
        if (i == 3) h->out_stage.alloc(std::max<int64_t>(1, p.c.size) * p.c.elem_bytes());
        const void* ta = i == 0 ? h->lenv : h->t[i - 1].get();
        const void* tb = i == 0 ? h->psi_stage.get() : (i == 1 ? h->mpo1 : (i == 2 ? h->mpo2 : h->renv));
        void* tc = i < 3 ? h->t[i].get() : h->out_stage.get();
        tune_plan(p, ta, tb, tc, mode, s, nullptr);
      }
      if (mode == QLTG_MODE_SPLIT) {
        prepare_split(p, s);
        // lenv (A of the first step), the MPO tensors and renv (B of the later steps) are
        // constant for the matvec's life
        if (i == 0) split_prepack_static(p, h->lenv, nullptr, s);
        if (i == 1) split_prepack_static(p, nullptr, h->mpo1, s);
        if (i == 2) split_prepack_static(p, nullptr, h->mpo2, s);
        if (i == 3) split_prepack_static(p, nullptr, h->renv, s);
      }
    }
    plan_mpo_fusion(*h, s);
    if (h->mpo_fused) h->t[1].release();   // t2 is never written in the fused form
    if (mode == QLTG_MODE_SPLIT) link_row_fields(*h, s);
    *mv = h.release();
  });
}

int qltg_matvec_result(const qltg_matvec* mv, int64_t* nblk, int64_t* size) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    if (nblk) *nblk = mv->step[3].c.nblk;
    if (size) *size = mv->step[3].c.size;
  });
}

int qltg_matvec_result_blocks(const qltg_matvec* mv, int64_t* coords, int64_t* offsets) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    mv->step[3].c.export_arrays(nullptr, nullptr, nullptr, nullptr, coords, offsets);
  });
}

int qltg_matvec_schedule(const qltg_matvec* mv, int32_t step, int32_t* f64_tile_rows, int32_t* split_stack,
                         int32_t* tuned, float* ms, int64_t* tile_stages, double* useful_frac) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    QLTG_CHECK(step >= 0 && step < 4, QLTG_ERR_INVALID, "step must be 0 .. 3");
    const CtrctPlan& p = mv->step[step];
    if (f64_tile_rows) *f64_tile_rows = p.sched.bm;
    if (split_stack) *split_stack = p.split_cfg.stack ? 1 : 0;
    for (int m = 0; m < 2; ++m) {
      if (tuned) tuned[m] = p.is_tuned[m] ? 1 : 0;
      if (ms) {
        ms[2 * m] = p.tuned[m].ms;
        ms[2 * m + 1] = p.tuned[m].other_ms;
      }
    }
    const bool has = p.split && p.split->built;
    if (tile_stages) *tile_stages = has ? p.split->tile_stages : 0;
    if (useful_frac) *useful_frac = has ? p.split->useful_frac : 0.0;
  });
}

int qltg_matvec_mpo_form(const qltg_matvec* mv, int32_t* fused, int32_t* fusable, float* ms) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    if (fused) *fused = mv->mpo_fused ? 1 : 0;
    if (fusable) *fusable = mv->mpo_fusable ? 1 : 0;
    if (ms) {
      ms[0] = mv->mid_ms[0];
      ms[1] = mv->mid_ms[1];
    }
  });
}

int qltg_matvec_set_mpo_form(qltg_matvec* mv, int32_t fused, void* stream) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    QLTG_CHECK(fused == 0 || fused == 1, QLTG_ERR_INVALID, "fused must be 0 or 1");
    QLTG_CHECK(!fused || mv->mpo_fusable, QLTG_ERR_UNSUPPORTED, "the MPO steps of this matvec cannot be fused");
    QLTG_CHECK(!mv->frozen && mv->graphs.empty(), QLTG_ERR_INVALID,
               "the MPO form is fixed once the matvec was applied or a Lanczos was created on it");
    if ((fused != 0) == mv->mpo_fused) return;
    QLTG_CUDA(cudaSetDevice(mv->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    mv->mpo_fused = fused != 0;
    if (!mv->mpo_fused && !mv->t[1].get())
      mv->t[1].alloc(std::max<int64_t>(1, mv->step[1].c.size) * mv->step[1].c.elem_bytes());
    if (mv->mode == QLTG_MODE_SPLIT) link_row_fields(*mv, s);
  });
}

int qltg_matvec_stats(const qltg_matvec* mv, double* flops, int64_t* launches) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    double f = 0;
    int64_t l = 0;
    const CtrctPlan* plans[4] = {&mv->step[0], &mv->step[1], &mv->step[2], &mv->step[3]};
    const int np = mv->mpo_fused ? 3 : 4;
    if (mv->mpo_fused) {
      plans[1] = &mv->mpo12;
      plans[2] = &mv->step[3];
    }
    for (int i = 0; i < np; ++i) {
      const CtrctPlan& p = *plans[i];
      f += p.flops;
      l += mv->mode == QLTG_MODE_SPLIT && p.split ? exec_launches_split(p) : p.launches_per_exec;
    }
    if (mv->fused_fields) ++l;   // the zero fill of the folded row scales
    if (flops) *flops = f;
    if (launches) *launches = l;
  });
}

int qltg_matvec_apply(qltg_matvec* mv, const void* psi_dev, void* out_dev, void* stream) {
  return guarded([&] {
    QLTG_CHECK(mv && psi_dev && out_dev, QLTG_ERR_INVALID, "null matvec or buffer");
    QLTG_CUDA(cudaSetDevice(mv->ctx->device));
    cudaGraphExec_t g = mv->graph_for(psi_dev, out_dev);
    QLTG_CUDA(cudaGraphLaunch(g, static_cast<cudaStream_t>(stream)));
  });
}

int qltg_matvec_apply_host(qltg_matvec* mv, const void* psi_host, void* out_host, void* stream) {
  return guarded([&] {
    QLTG_CHECK(mv && psi_host && out_host, QLTG_ERR_INVALID, "null matvec or buffer");
    QLTG_CUDA(cudaSetDevice(mv->ctx->device));
    for (const void* p : {psi_host, static_cast<const void*>(out_host)}) {
      cudaPointerAttributes at{};
      QLTG_CUDA(cudaPointerGetAttributes(&at, p));
      QLTG_CHECK(at.type == cudaMemoryTypeHost && at.devicePointer == p, QLTG_ERR_INVALID,
                 "host buffers must be page-locked and mapped at their host address (cudaMallocHost, cudaHostAlloc)");
    }
    const Meta& pm = mv->step[0].b;
    const Meta& om = mv->step[3].c;
    const int64_t in_bytes = pm.size * (int64_t)pm.elem_bytes(), out_bytes = om.size * (int64_t)om.elem_bytes();
    if (!mv->psi_stage.get()) mv->psi_stage.alloc(std::max<int64_t>(in_bytes, 16));
    if (!mv->out_stage.get()) mv->out_stage.alloc(std::max<int64_t>(out_bytes, 16));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // copy engine both ways: the last step storing straight into host memory measured slower
    // (its scattered 64-byte row stores over the host link stall the epilogue)
    if (in_bytes) QLTG_CUDA(cudaMemcpyAsync(mv->psi_stage.get(), psi_host, in_bytes, cudaMemcpyHostToDevice, s));
    QLTG_CUDA(cudaGraphLaunch(mv->graph_for(mv->psi_stage.get(), mv->out_stage.get()), s));
    if (out_bytes) QLTG_CUDA(cudaMemcpyAsync(out_host, mv->out_stage.get(), out_bytes, cudaMemcpyDeviceToHost, s));
  });
}

int qltg_matvec_device_status(qltg_matvec* mv, void* stream) {
  return guarded([&] {
    QLTG_CHECK(mv, QLTG_ERR_INVALID, "null matvec");
    QLTG_CUDA(cudaSetDevice(mv->ctx->device));
    for (const CtrctPlan* p : {&mv->step[0], &mv->step[1], &mv->step[2], &mv->step[3], &mv->mpo12})
      QLTG_CHECK(split_device_error(*p, static_cast<cudaStream_t>(stream)) == 0, QLTG_ERR_TIMEOUT,
                 "a bounded tensor-core wait expired in the split-precision GEMM");
  });
}

int qltg_matvec_destroy(qltg_matvec* mv) {
  delete mv;
  return QLTG_OK;
}

}  // extern "C"
