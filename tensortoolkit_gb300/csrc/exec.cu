// Contraction execution: schedule construction after device pairing, and the launch
// sequence (operand transposes, then one grouped GEMM).
#include <algorithm>

#include "ctrct.h"
#include "split.h"

namespace qltg {

void finalize_plan(CtrctPlan& p, cudaStream_t s) {
  GemmSchedule& g = p.sched;
  g.tile.clear();
  g.skinny.clear();
  const int rows_per_item = skinny_rows_per_item();
  struct Cand { GemmTile t; int64_t cost; };
  std::vector<Cand> cands;
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q) {
    const GemmCBlk& cb = g.cblk[q];
    if (skinny_cblk(g, q)) {
      for (int32_t c = 0; c * (int64_t)rows_per_item < cb.m; ++c) g.skinny.push_back(GemmRowChunk{q, c});
      continue;
    }
    int64_t ksum = 0;
    for (int32_t t = cb.t0; t < cb.t1; ++t) ksum += g.task[t].k;
    const int tm = (cb.m + g.bm - 1) / g.bm, tn = (cb.n + g.bn - 1) / g.bn;
    QLTG_CHECK(tm < 32768 && tn < 32768, QLTG_ERR_UNSUPPORTED, "output block too large for the tile grid");
    for (int i = 0; i < tm; ++i)
      for (int j = 0; j < tn; ++j) {
        const int64_t rows = std::min(g.bm, cb.m - i * g.bm), cols = std::min(g.bn, cb.n - j * g.bn);
        cands.push_back({GemmTile{q, (int16_t)i, (int16_t)j}, ksum * rows * cols});
      }
  }
  std::stable_sort(cands.begin(), cands.end(), [](const Cand& x, const Cand& y) { return x.cost > y.cost; });
  g.tile.reserve(cands.size());
  for (auto& c : cands) g.tile.push_back(c.t);
  // operand transposes: blocks whose layout the permutation leaves unchanged are read from
  // the operand itself (flagged in the task offsets) and get no transpose work
  const size_t eb = p.a.elem_bytes();
  const bool any_work = !g.tile.empty() || !g.skinny.empty();
  auto flag_identity = [&](const Meta& m, const TransposeList& tl, bool side_a) {
    for (auto& tk : g.task) {
      int64_t& off = side_a ? tk.a_off : tk.b_off;
      const int64_t b = std::lower_bound(m.offsets.begin(), m.offsets.end(), off) - m.offsets.begin();
      QLTG_CHECK(b < m.nblk && m.offsets[b] == off, QLTG_ERR_INVALID, "internal: task operand offset is no block start");
      if (tl.identity[b]) off |= kFromSrc;
    }
  };
  p.a_tl = TransposeList();
  p.b_tl = TransposeList();
  if (p.a_trans && p.a.size && any_work) {
    p.a_tl.build(p.a, p.a_order, {}, nullptr, s, /*skip_identity=*/true);
    flag_identity(p.a, p.a_tl, true);
    if (p.a_tl.ntiles) p.a_t.alloc(p.a.size * eb);
  }
  if (p.b_trans && p.b.size && any_work) {
    p.b_tl.build(p.b, p.b_order, {}, nullptr, s, /*skip_identity=*/true);
    flag_identity(p.b, p.b_tl, false);
    if (p.b_tl.ntiles) p.b_t.alloc(p.b.size * eb);
  }
  g.d_cblk = upload(g.cblk, s);
  g.d_task = upload(g.task, s);
  g.d_tile = upload(g.tile, s);
  g.d_skinny = upload(g.skinny, s);
  g.d_counter.alloc(sizeof(int));
  p.launches_per_exec = (g.tile.empty() ? 0 : 2) + (g.skinny.empty() ? 0 : 1) +   // memset + GEMM
                         (p.a_tl.ntiles ? 1 : 0) + (p.b_tl.ntiles ? 1 : 0);
  QLTG_CUDA(cudaStreamSynchronize(s));
}

// Kernel launches of one split-mode execution: operand transposes plus the split stage.
int64_t exec_launches_split(const CtrctPlan& p) {
  int64_t n = split_launches(p);
  if (p.a_tl.ntiles && !(p.split && p.split->a_static)) n += 1;
  if (p.b_tl.ntiles && !(p.split && p.split->b_static)) n += 1;
  return n;
}

void exec_contraction(CtrctPlan& p, const void* a, const void* b, void* c, int mode, cudaStream_t s, int stage) {
  if (p.sched.tile.empty() && p.sched.skinny.empty()) return;
  QLTG_CHECK(a && b && c, QLTG_ERR_INVALID, "null device buffer");
  QLTG_CHECK(stage >= 0 && stage <= 3, QLTG_ERR_INVALID, "stage must be 0, 1, 2 or 3");
  QLTG_CHECK(mode == QLTG_MODE_FP64 || mode == QLTG_MODE_SPLIT, QLTG_ERR_INVALID, "unknown arithmetic mode");
  const int eb = (int)p.a.elem_bytes();
  // operand scratch (transposed blocks) and the operands themselves (blocks flagged
  // kFromSrc); untransposed operands are their own scratch
  Operands op{a, a, b, b};
  // operands packed once for the split path (constant for the plan's life) need no transpose
  const bool a_packed = mode == QLTG_MODE_SPLIT && p.split && p.split->a_static && p.split->a_ready;
  const bool b_packed = mode == QLTG_MODE_SPLIT && p.split && p.split->b_static && p.split->b_ready;
  if (p.a_tl.ntiles) {
    if (stage < 2 && !a_packed) p.a_tl.launch(a, p.a_t.get(), eb, s);
    op.a = p.a_t.get();
  }
  if (p.b_tl.ntiles) {
    if (stage < 2 && !b_packed) p.b_tl.launch(b, p.b_t.get(), eb, s);
    op.b = p.b_t.get();
  }
  if (stage == 1) return;
  if (mode == QLTG_MODE_FP64)
    launch_gemm_f64(p.sched, op, c, p.a.dtype == QLTG_C128, p.ctx->num_sms, s);
  else
    launch_gemm_split(p, op, c, s, /*pack=*/stage != 3);
}

}  // namespace qltg
