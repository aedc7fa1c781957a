// Contraction execution: schedule construction after device pairing, and the launch
// sequence (operand transposes, then one grouped GEMM).
#include <algorithm>

#include "ctrct.h"
#include "split.h"

namespace qltg {

// FP64 output tiles of g.bm x g.bn, longest first (the DFMA kernel takes them in this order).
static void f64_tile_list(GemmSchedule& g) {
  g.tile.clear();
  struct Cand { GemmTile t; int64_t cost; };
  std::vector<Cand> cands;
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q) {
    const GemmCBlk& cb = g.cblk[q];
    if (skinny_cblk(g, q)) continue;
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
}

void set_f64_tile(CtrctPlan& p, int bm, int bn, cudaStream_t s) {
  QLTG_CHECK((bm == 32 && bn == 32) || (bm == 64 && bn == 32), QLTG_ERR_INVALID, "FP64 tiles are 32 x 32 or 64 x 32");
  GemmSchedule& g = p.sched;
  if (g.bm == bm && g.bn == bn && g.d_tile.get()) return;
  g.bm = bm;
  g.bn = bn;
  f64_tile_list(g);
  g.d_tile = upload(g.tile, s);
  QLTG_CUDA(cudaStreamSynchronize(s));
}

void finalize_plan(CtrctPlan& p, cudaStream_t s) {
  GemmSchedule& g = p.sched;
  g.skinny.clear();
  g.skinny_maxn = 1;
  const int rows_per_item = skinny_rows_per_item();
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q) {
    const GemmCBlk& cb = g.cblk[q];
    if (skinny_cblk(g, q)) {
      g.skinny_maxn = std::max(g.skinny_maxn, (int)cb.n);
      for (int32_t c = 0; c * (int64_t)rows_per_item < cb.m; ++c) g.skinny.push_back(GemmRowChunk{q, c});
    }
  }
  f64_tile_list(g);
  // Operand transposes. A task reads its operand block from the transposed scratch unless
  // (a) the permutation leaves the block's layout unchanged, or (b) it is a skinny task and
  // the block, read in place, is a strided matrix (rows and columns each one stride); such
  // tasks read the operand itself (offset flag kFromSrc) and blocks nobody reads from the
  // scratch get no transpose work.
  const size_t eb = p.a.elem_bytes();
  const bool any_work = !g.tile.empty() || !g.skinny.empty();
  std::vector<uint8_t> skinny_task(g.task.size(), 0);
  for (int32_t q = 0; q < (int32_t)g.cblk.size(); ++q)
    if (skinny_cblk(g, q))
      for (int32_t t = g.cblk[q].t0; t < g.cblk[q].t1; ++t) skinny_task[t] = 1;
  auto block_of = [](const Meta& m, int64_t off) {
    const int64_t b = std::lower_bound(m.offsets.begin(), m.offsets.end(), off) - m.offsets.begin();
    QLTG_CHECK(b < m.nblk && m.offsets[b] == off, QLTG_ERR_INVALID, "internal: task operand offset is no block start");
    return b;
  };
  // (row stride, column stride) of block b of A read in place, rows = saved legs, columns =
  // contracted legs in the transposed order; false if either needs more than one stride
  auto strided_a = [&](int64_t b, int32_t& rs, int32_t& cs) {
    const int r = p.a.rank, ns = (int)p.sa.size();
    std::vector<int64_t> sstr(r);
    if (r) sstr[r - 1] = 1;
    for (int i = r - 2; i >= 0; --i) sstr[i] = sstr[i + 1] * p.a.dim(b, i + 1);
    auto merge = [&](int lo, int hi, int32_t& stride) {
      int64_t run_dim = 0, run_stride = 1;
      int n = 0;
      for (int i = lo; i < hi; ++i) {
        const int leg = p.a_order[i];
        const int64_t d = p.a.dim(b, leg);
        if (d == 1) continue;
        if (n && run_stride == sstr[leg] * d) {
          run_dim *= d;
          run_stride = sstr[leg];
        } else {
          if (n) return false;
          run_dim = d;
          run_stride = sstr[leg];
          n = 1;
        }
      }
      if (run_stride >= ((int64_t)1 << 31)) return false;
      stride = (int32_t)(n ? run_stride : 0);
      return true;
    };
    return merge(0, ns, rs) && merge(ns, r, cs);
  };
  p.a_tl = TransposeList();
  p.b_tl = TransposeList();
  if (p.a_trans && p.a.size && any_work) {
    TransposeList probe;
    probe.describe(p.a, p.a_order, {}, nullptr);
    std::vector<uint8_t> need(p.a.nblk, 0);
    for (size_t t = 0; t < g.task.size(); ++t) {
      GemmTask& tk = g.task[t];
      const int64_t b = block_of(p.a, tk.a_off);
      int32_t rs = 0, cs = 0;
      if (probe.identity[b]) {
        tk.a_off |= kFromSrc;
      } else if (skinny_task[t] && strided_a(b, rs, cs)) {
        tk.a_off |= kFromSrc;
        tk.a_rs = rs;
        tk.a_cs = cs;
      } else {
        need[b] = 1;
      }
    }
    std::vector<uint8_t> skip(p.a.nblk);
    for (int64_t b = 0; b < p.a.nblk; ++b) skip[b] = !need[b];
    p.a_tl.build(p.a, p.a_order, {}, nullptr, s, false, &skip);
    if (p.a_tl.ntiles) p.a_t.alloc(p.a.size * eb);
  }
  if (p.b_trans && p.b.size && any_work) {
    p.b_tl.build(p.b, p.b_order, {}, nullptr, s, /*skip_identity=*/true);
    for (auto& tk : g.task)
      if (p.b_tl.identity[block_of(p.b, tk.b_off)]) tk.b_off |= kFromSrc;
    if (p.b_tl.ntiles) p.b_t.alloc(p.b.size * eb);
  }
  if (!g.skinny.empty()) (void)skinny_grid((int)g.skinny.size(), p.a.dtype == QLTG_C128, g.skinny_maxn, p.ctx->num_sms);
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
