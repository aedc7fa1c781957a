// Schedule tuner for the grouped GEMM stage of a contraction plan.
//
// The reference issues one cublasDgemm per task (framework/hp_numeric/blas_level3.h:797-856)
// and has no schedule to choose. Here all tasks of a contraction go out in one persistent
// launch, and how they are cut into tiles is a choice that depends on the block shapes:
//  * FP64 (DFMA) tiles of 32 x 32 or 64 x 32 outputs - the taller tile reuses each staged
//    operand value for twice the FMAs, the smaller one wastes less on small blocks;
//  * split precision: row stacking on or off - stacking packs the A blocks of output blocks
//    with the same task structure into shared 128-row tiles (less padding, one row-map load
//    per output row), off keeps one block per tile.
// tune_plan times every candidate of a mode once on the plan's own operands (CUDA events on
// the caller's stream, the GEMM stage alone, median of a few runs) and keeps the fastest.
// The choice is remembered per device and block-structure signature (a hash of every
// non-skinny output block's shape and its tasks' k, operand blocks and signs), so later
// plans of the same layouts - the next Contract of a sweep, the matvec of the next Lanczos
// - take it without timing.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "ctrct.h"
#include "split.h"

namespace qltg {
namespace {

std::mutex g_tune_mu;
std::map<std::tuple<int, int, uint64_t>, TuneChoice> g_tune_cache;   // (device, mode, signature)

uint64_t fnv(uint64_t h, int64_t v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (uint64_t)((v >> (8 * i)) & 0xFF);
    h *= 1099511628211ull;
  }
  return h;
}

// Median time in ms of `reps` runs of stage `stage` of the plan (after one full run).
float time_stage(CtrctPlan& p, const void* a, const void* b, void* c, int mode, int stage, cudaStream_t s,
                 int reps = 5) {
  exec_contraction(p, a, b, c, mode, s, 0);
  std::vector<cudaEvent_t> ev(2 * reps);
  for (auto& e : ev) QLTG_CUDA(cudaEventCreate(&e));
  struct Free {
    std::vector<cudaEvent_t>& ev;
    ~Free() {
      for (auto e : ev) cudaEventDestroy(e);
    }
  } free_ev{ev};
  for (int r = 0; r < reps; ++r) {
    QLTG_CUDA(cudaEventRecord(ev[2 * r], s));
    exec_contraction(p, a, b, c, mode, s, stage);
    QLTG_CUDA(cudaEventRecord(ev[2 * r + 1], s));
  }
  QLTG_CUDA(cudaStreamSynchronize(s));
  std::vector<float> ms(reps);
  for (int r = 0; r < reps; ++r) QLTG_CUDA(cudaEventElapsedTime(&ms[r], ev[2 * r], ev[2 * r + 1]));
  std::sort(ms.begin(), ms.end());
  return ms[reps / 2];
}

}  // namespace

uint64_t plan_signature(const CtrctPlan& p, int mode) {
  const GemmSchedule& g = p.sched;
  uint64_t h = 1469598103934665603ull;
  h = fnv(h, mode);
  h = fnv(h, p.a.dtype);
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q) {
    if (skinny_cblk(g, q)) continue;
    const GemmCBlk& cb = g.cblk[q];
    h = fnv(h, cb.m);
    h = fnv(h, cb.n);
    for (int32_t t = cb.t0; t < cb.t1; ++t) {
      const GemmTask& tk = g.task[t];
      h = fnv(h, tk.k);
      h = fnv(h, tk.a_off & ~kFromSrc);
      h = fnv(h, tk.b_off & ~kFromSrc);
      h = fnv(h, tk.sign);
    }
  }
  return h;
}

void apply_choice(CtrctPlan& p, int mode, const TuneChoice& c, cudaStream_t s) {
  if (mode == QLTG_MODE_FP64) {
    set_f64_tile(p, c.f64_bm, 32, s);
  } else {
    QLTG_CHECK(!(p.split && (p.split->a_static || p.split->b_static)), QLTG_ERR_INVALID,
               "the split schedule of a plan with operands packed once cannot change");
    if (p.split && p.split->built && p.split_cfg.stack == c.split_stack) return;
    p.split_cfg.stack = c.split_stack;
    p.split.reset();
    prepare_split(p, s);
  }
}

TuneChoice tune_plan(CtrctPlan& p, const void* a, const void* b, void* c, int mode, cudaStream_t s, bool* cached) {
  QLTG_CHECK(mode == QLTG_MODE_FP64 || mode == QLTG_MODE_SPLIT, QLTG_ERR_INVALID, "unknown arithmetic mode");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  QLTG_CUDA(cudaStreamIsCapturing(s, &cs));
  QLTG_CHECK(cs == cudaStreamCaptureStatusNone, QLTG_ERR_INVALID, "tuning times kernels: not inside a stream capture");
  TuneChoice best{p.sched.bm, p.split_cfg.stack, 0.f, 0.f};
  if (cached) *cached = false;
  bool any_tiles = false;
  for (int32_t q = 0; q < (int32_t)p.sched.cblk.size() && !any_tiles; ++q) any_tiles = !skinny_cblk(p.sched, q);
  if (!any_tiles) return best;   // skinny blocks only: nothing to choose
  const auto key = std::make_tuple(p.ctx->device, mode, plan_signature(p, mode));
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      apply_choice(p, mode, it->second, s);
      if (cached) *cached = true;
      p.tuned[mode] = it->second;
      p.is_tuned[mode] = true;
      return it->second;
    }
  }
  std::vector<TuneChoice> cands;
  if (mode == QLTG_MODE_FP64) {
    cands.push_back(TuneChoice{32, p.split_cfg.stack, 0.f, 0.f});
    cands.push_back(TuneChoice{64, p.split_cfg.stack, 0.f, 0.f});
  } else {
    cands.push_back(TuneChoice{p.sched.bm, true, 0.f, 0.f});
    cands.push_back(TuneChoice{p.sched.bm, false, 0.f, 0.f});
  }
  float best_ms = 0.f;
  std::vector<float> times;
  for (size_t i = 0; i < cands.size(); ++i) {
    apply_choice(p, mode, cands[i], s);
    // the GEMM stage alone: FP64 stage 2 (the transposes are the same for every tile),
    // split stage 3 (operands packed by the full run before the timed ones)
    const float ms = time_stage(p, a, b, c, mode, mode == QLTG_MODE_FP64 ? 2 : 3, s);
    times.push_back(ms);
    if (i == 0 || ms < best_ms) {
      best_ms = ms;
      best = cands[i];
    }
  }
  best.ms = best_ms;
  best.other_ms = times.size() > 1 ? *std::max_element(times.begin(), times.end()) : best_ms;
  apply_choice(p, mode, best, s);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = best;
  }
  p.tuned[mode] = best;
  p.is_tuned[mode] = true;
  return best;
}

}  // namespace qltg
