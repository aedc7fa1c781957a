// The reference's bosonic DMRG axis primitives (qlten::dmrg, tensor_manipulation/dmrg/
// axis_ops.h) on device buffers.
//
//  * ApplyAxisDiagonal (axis_ops.h:2370-2547) / ApplyAxisDiagonalInPlace (:2549-2582):
//      out = beta out + alpha D(in), D multiplying every degeneracy slice of `axis` by its
//      value; the topology is the input's. One streaming kernel over (block, chunk) items;
//      the axis coordinate of an element is (index / stride) mod dim inside its block.
//  * ApplyAxisSectorScalarsPreserveOrder (:2655-2744): a block times the value of its sector
//      on `axis` (the same kernel with one value per sector).
//  * ApplyRank2ToAxisPreserveOrder (:2862-2993): contract `axis` with the operator's index
//      0; index 1 takes the axis' place. The contraction's grouped GEMM writes (other legs,
//      new leg); one batched permute puts the new leg back at `axis` (none when it is the
//      last axis).
//  * ApplyTwoRank2ToAxesPreserveOrder (:2995-3126): op1 on axis1, then op2 on axis2.
//  * ApplyAxisMonomial (:2746-2860; topology :2241-2269; slice add :2306-2332): entries map an
//      input degeneracy slice (in_sector, in_offset) of `axis` to an output slice (out_sector,
//      out_offset) with a coefficient. The plan builds the output topology and, per output
//      slice, the list of contributing input slices in the reference's order (input blocks
//      ascending, entries in order); one kernel writes every output slice once:
//      out = beta out + sum alpha coef in_slice. No atomics, deterministic.
// All are bosonic-only, as in the reference (fermionic tensors: QLTG_ERR_UNSUPPORTED).
#include <algorithm>
#include <memory>
#include <numeric>

#include "ctrct.h"
#include "split.h"

namespace qltg {
namespace {

struct AxisItem {
  int64_t off;        // element offset of the chunk's block
  int32_t e0, n;      // first element of the chunk inside the block, element count
  int32_t stride;     // elements per step of the axis inside the block
  int32_t dim;        // the axis' extent inside the block
  int32_t vbase;      // index of the block's first axis value
  int32_t pad;
};
constexpr int kAxisChunk = 4096;

__device__ __forceinline__ double amul(double a, double x) { return a * x; }
__device__ __forceinline__ double2 amul(double2 a, double2 x) {
  return make_double2(fma(a.x, x.x, -a.y * x.y), fma(a.x, x.y, a.y * x.x));
}
__device__ __forceinline__ double aadd(double a, double b) { return a + b; }
__device__ __forceinline__ double2 aadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

template <typename T>
__global__ void __launch_bounds__(256) k_axis_scale(const AxisItem* __restrict__ items, int nitems,
                                                    const T* __restrict__ values, const T* in, T* out, T alpha,
                                                    T beta, int read_out) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const AxisItem w = items[it];
    for (int e = threadIdx.x; e < w.n; e += blockDim.x) {
      const int64_t g = (int64_t)w.e0 + e;
      const T v = values[w.vbase + (int32_t)((g / w.stride) % w.dim)];
      T r = amul(alpha, amul(v, in[w.off + g]));
      if (read_out) r = aadd(r, amul(beta, out[w.off + g]));
      out[w.off + g] = r;
    }
  }
}

struct MonoMap {             // one contributing input slice
  int64_t in_off;            // element offset of the input block
  int32_t in_axis_dim, in_offset;
  double coef_re, coef_im;
};
struct MonoItem {            // one output slice
  int64_t out_off;           // element offset of the output block
  int32_t out_axis_dim, out_offset;
  int32_t outer, inner;      // elements before / after the axis inside the block
  int32_t map0, map1;        // its maps
};

__device__ __forceinline__ double azero(double) { return 0.0; }
__device__ __forceinline__ double2 azero(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double mcoef(double re, double, double) { return re; }
__device__ __forceinline__ double2 mcoef(double re, double im, double2) { return make_double2(re, im); }

template <typename T>
__global__ void __launch_bounds__(256) k_axis_monomial(const MonoItem* __restrict__ items, int nitems,
                                                       const MonoMap* __restrict__ maps, const T* __restrict__ in,
                                                       T* __restrict__ out, T alpha, T beta, int read_out) {
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const MonoItem w = items[it];
    const int64_t n = (int64_t)w.outer * w.inner;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      const int64_t o = e / w.inner, i = e - o * w.inner;
      const int64_t dst = w.out_off + (o * w.out_axis_dim + w.out_offset) * w.inner + i;
      T acc = read_out ? amul(beta, out[dst]) : azero(T());
      for (int mi = w.map0; mi < w.map1; ++mi) {
        const MonoMap m = maps[mi];
        const T c = amul(alpha, mcoef(m.coef_re, m.coef_im, T()));
        acc = aadd(acc, amul(c, in[m.in_off + (o * m.in_axis_dim + m.in_offset) * w.inner + i]));
      }
      out[dst] = acc;
    }
  }
}

std::vector<AxisItem> axis_items(const Meta& m, int axis) {
  std::vector<int64_t> sstart(m.nsct(axis), 0);
  for (int64_t s = 1; s < m.nsct(axis); ++s) sstart[s] = sstart[s - 1] + m.dims[axis][s - 1];
  std::vector<AxisItem> items;
  for (int64_t b = 0; b < m.nblk; ++b) {
    int64_t stride = 1;
    for (int l = axis + 1; l < m.rank; ++l) stride *= m.dim(b, l);
    const int64_t size = m.blk_size(b);
    QLTG_CHECK(size < ((int64_t)1 << 31), QLTG_ERR_UNSUPPORTED, "block above 2^31 elements");
    for (int64_t e = 0; e < size; e += kAxisChunk)
      items.push_back(AxisItem{m.offsets[b], (int32_t)e, (int32_t)std::min<int64_t>(kAxisChunk, size - e),
                               (int32_t)stride, (int32_t)m.dim(b, axis),
                               (int32_t)sstart[m.coords[b * m.rank + axis]], 0});
  }
  return items;
}

// out = beta out + alpha D(in) with per-degeneracy values (host, complex interleaved)
void axis_scale(qltg_ctx* ctx, const Meta& m, int axis, const std::vector<double>& values, const void* in, void* out,
                const double* alpha, const double* beta, cudaStream_t s) {
  if (m.nblk == 0) return;
  QLTG_CHECK(in && out, QLTG_ERR_INVALID, "null buffer");
  const bool cplx = m.dtype == QLTG_C128;
  QLTG_CHECK(cplx || (alpha[1] == 0.0 && beta[1] == 0.0), QLTG_ERR_INVALID, "complex alpha or beta for a real tensor");
  const auto items = axis_items(m, axis);
  DevBuf d_items = upload(items, s);
  DevBuf d_vals = upload(values, s);
  const int ni = (int)items.size();
  const int grid = std::min(ni, std::max(1, ctx->num_sms) * 8);
  const int read_out = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
  if (cplx)
    k_axis_scale<double2><<<grid, 256, 0, s>>>(d_items.as<AxisItem>(), ni, d_vals.as<double2>(),
                                               static_cast<const double2*>(in), static_cast<double2*>(out),
                                               make_double2(alpha[0], alpha[1]), make_double2(beta[0], beta[1]),
                                               read_out);
  else
    k_axis_scale<double><<<grid, 256, 0, s>>>(d_items.as<AxisItem>(), ni, d_vals.as<double>(),
                                              static_cast<const double*>(in), static_cast<double*>(out), alpha[0],
                                              beta[0], read_out);
  QLTG_CUDA(cudaGetLastError());
  // the work list and values are freed on return
  QLTG_CUDA(cudaStreamSynchronize(s));
}

void require_bosonic_axis(const Meta& m, int axis) {
  QLTG_CHECK(m.parity_comp < 0, QLTG_ERR_UNSUPPORTED, "the dmrg axis primitives are bosonic-only");
  QLTG_CHECK(m.rank >= 1 && axis >= 0 && axis < m.rank, QLTG_ERR_INVALID, "axis out of range");
}

// Legs and blocks of m with its legs reordered to `order` (bosonic transpose).
Meta permuted_meta(const Meta& c, const std::vector<int>& order) {
  Meta m = c;
  const int r = c.rank;
  for (int l = 0; l < r; ++l) {
    m.dirs[l] = c.dirs[order[l]];
    m.qns[l] = c.qns[order[l]];
    m.dims[l] = c.dims[order[l]];
  }
  std::vector<std::vector<int64_t>> blocks(c.nblk, std::vector<int64_t>(r));
  for (int64_t b = 0; b < c.nblk; ++b)
    for (int l = 0; l < r; ++l) blocks[b][l] = c.coords[b * r + order[l]];
  std::sort(blocks.begin(), blocks.end(), [&](const std::vector<int64_t>& x, const std::vector<int64_t>& y) {
    return m.blk_idx(x.data()) < m.blk_idx(y.data());
  });
  m.coords.clear();
  for (auto& v : blocks) m.coords.insert(m.coords.end(), v.begin(), v.end());
  m.refresh_offsets();
  return m;
}

// One rank-2 application: contraction (in . op over axis <-> op index 0) and the permute
// that puts the new leg back at `axis`.
struct Rank2Step {
  CtrctPlan c;
  bool permute = false;
  TransposeList tl;
  Meta out;
  DevBuf scratch;

  void build(qltg_ctx* ctx, const Meta& in, const Meta& op, int axis, cudaStream_t s) {
    require_bosonic_axis(in, axis);
    QLTG_CHECK(op.rank == 2, QLTG_ERR_INVALID, "the axis operator must have rank 2");
    QLTG_CHECK(op.parity_comp < 0, QLTG_ERR_UNSUPPORTED, "the dmrg axis primitives are bosonic-only");
    c.ctx = ctx;
    c.a = in;
    c.b = op;
    c.axa = {axis};
    c.axb = {0};
    plan_contraction(c, s);
    finalize_plan(c, s);
    const int r = in.rank;
    permute = axis != r - 1;
    if (!permute) {
      out = c.c;
      return;
    }
    std::vector<int> order;
    for (int l = 0; l < axis; ++l) order.push_back(l);
    order.push_back(r - 1);
    for (int l = axis; l < r - 1; ++l) order.push_back(l);
    out = permuted_meta(c.c, order);
    std::vector<double> signs;
    std::vector<int64_t> dst_off;
    transpose_layout(c.c, order, signs, dst_off);
    tl.build(c.c, order, signs, &dst_off, s);
    scratch.alloc(std::max<int64_t>(c.c.size, 1) * c.c.elem_bytes());
  }
  void exec(const void* in, const void* op, void* dst, int mode, cudaStream_t s) {
    if (c.c.size == 0) return;
    if (!permute) {
      exec_contraction(c, in, op, dst, mode, s);
      return;
    }
    exec_contraction(c, in, op, scratch.get(), mode, s);
    tl.launch(scratch.get(), dst, (int)c.c.elem_bytes(), s);
  }
};

}  // namespace
}  // namespace qltg

struct qltg_axis_plan {
  qltg_ctx* ctx = nullptr;
  qltg::Rank2Step s1, s2;
  bool two = false;
  qltg::DevBuf mid;   // the single-axis intermediate of the two-operator form
  // monomial form
  bool mono = false;
  qltg::Meta mono_out;
  int mono_items = 0;
  qltg::DevBuf d_mono_items, d_mono_maps;
  const qltg::Meta& out() const { return mono ? mono_out : (two ? s2.out : s1.out); }
};

using namespace qltg;

extern "C" {

int qltg_axis_diagonal(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis, const double* values,
                       const void* in_dev, void* out_dev, const double* alpha, const double* beta, void* stream) {
  return guarded([&] {
    QLTG_CHECK(ctx && values && alpha && beta, QLTG_ERR_INVALID, "null argument");
    const Meta m = meta_from_desc(t);
    require_bosonic_axis(m, axis);
    QLTG_CUDA(cudaSetDevice(ctx->device));
    int64_t dim = 0;
    for (auto d : m.dims[axis]) dim += d;
    const int per = m.dtype == QLTG_C128 ? 2 : 1;
    axis_scale(ctx, m, axis, std::vector<double>(values, values + dim * per), in_dev, out_dev, alpha, beta,
               static_cast<cudaStream_t>(stream));
  });
}

int qltg_axis_sector_scalars(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis, const double* values_by_sector,
                             const void* in_dev, void* out_dev, void* stream) {
  return guarded([&] {
    QLTG_CHECK(ctx && values_by_sector, QLTG_ERR_INVALID, "null argument");
    const Meta m = meta_from_desc(t);
    require_bosonic_axis(m, axis);
    QLTG_CUDA(cudaSetDevice(ctx->device));
    const int per = m.dtype == QLTG_C128 ? 2 : 1;
    std::vector<double> v;   // one value per degeneracy: the sector's
    for (int64_t s = 0; s < m.nsct(axis); ++s)
      for (int64_t d = 0; d < m.dims[axis][s]; ++d)
        for (int c = 0; c < per; ++c) v.push_back(values_by_sector[s * per + c]);
    const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
    axis_scale(ctx, m, axis, v, in_dev, out_dev, one, zero, static_cast<cudaStream_t>(stream));
  });
}

int qltg_axis_rank2_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, const qltg_tensor_desc* op, int32_t axis,
                                qltg_axis_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_axis_plan>();
    h->ctx = ctx;
    cudaStream_t s;
    QLTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    try {
      h->s1.build(ctx, meta_from_desc(t), meta_from_desc(op), axis, s);
      QLTG_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      cudaStreamDestroy(s);
      throw;
    }
    QLTG_CUDA(cudaStreamDestroy(s));
    *plan = h.release();
  });
}

int qltg_axis_two_rank2_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, const qltg_tensor_desc* op1,
                                    int32_t axis1, const qltg_tensor_desc* op2, int32_t axis2,
                                    qltg_axis_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    QLTG_CHECK(axis1 != axis2, QLTG_ERR_INVALID, "axis1 and axis2 must differ");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    auto h = std::make_unique<qltg_axis_plan>();
    h->ctx = ctx;
    h->two = true;
    cudaStream_t s;
    QLTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    try {
      h->s1.build(ctx, meta_from_desc(t), meta_from_desc(op1), axis1, s);
      h->s2.build(ctx, h->s1.out, meta_from_desc(op2), axis2, s);
      QLTG_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      cudaStreamDestroy(s);
      throw;
    }
    QLTG_CUDA(cudaStreamDestroy(s));
    h->mid.alloc(std::max<int64_t>(h->s1.out.size, 1) * h->s1.out.elem_bytes());
    *plan = h.release();
  });
}

int qltg_axis_monomial_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis, int32_t out_nsct,
                                   const int32_t* out_qns, const int64_t* out_dims, const int32_t* flux,
                                   int64_t nentries, const int64_t* entries, const double* coefs,
                                   qltg_axis_plan** plan) {
  return guarded([&] {
    QLTG_CHECK(ctx && plan, QLTG_ERR_INVALID, "null ctx or plan out-pointer");
    const Meta m = meta_from_desc(t);
    require_bosonic_axis(m, axis);
    QLTG_CHECK(out_nsct >= 1 && out_qns && out_dims && flux, QLTG_ERR_INVALID, "null or empty output index");
    QLTG_CHECK(nentries >= 0 && (nentries == 0 || (entries && coefs)), QLTG_ERR_INVALID, "null entries");
    QLTG_CUDA(cudaSetDevice(ctx->device));
    const int nc = m.ncomp, per = m.dtype == QLTG_C128 ? 2 : 1;
    auto h = std::make_unique<qltg_axis_plan>();
    h->ctx = ctx;
    h->mono = true;
    // output index: the axis replaced (same direction)
    Meta& O = h->mono_out;
    O = m;
    O.qns[axis].assign(out_qns, out_qns + (int64_t)out_nsct * nc);
    O.dims[axis].assign(out_dims, out_dims + out_nsct);
    for (auto d : O.dims[axis]) QLTG_CHECK(d >= 1, QLTG_ERR_INVALID, "output degeneracy must be >= 1");
    // entries: range and flux checks (output qn = input qn + flux)
    for (int64_t e = 0; e < nentries; ++e) {
      const int64_t is = entries[4 * e], io = entries[4 * e + 1], os = entries[4 * e + 2], oo = entries[4 * e + 3];
      QLTG_CHECK(is >= 0 && is < m.nsct(axis) && os >= 0 && os < out_nsct, QLTG_ERR_INVALID,
                 "monomial entry sector out of range");
      QLTG_CHECK(io >= 0 && io < m.dims[axis][is] && oo >= 0 && oo < out_dims[os], QLTG_ERR_INVALID,
                 "monomial entry degeneracy offset out of range");
      for (int c = 0; c < nc; ++c)
        QLTG_CHECK(out_qns[os * nc + c] == m.qns[axis][is * nc + c] + flux[c], QLTG_ERR_INVALID,
                   "monomial entry quantum numbers are inconsistent with the flux");
    }
    // output topology: input blocks mapped through every matching entry, ascending block index
    std::vector<std::vector<int64_t>> oc;
    std::vector<uint64_t> okey;
    for (int64_t b = 0; b < m.nblk; ++b)
      for (int64_t e = 0; e < nentries; ++e) {
        if (entries[4 * e] != m.coords[b * m.rank + axis]) continue;
        std::vector<int64_t> c(m.coords.begin() + b * m.rank, m.coords.begin() + (b + 1) * m.rank);
        c[axis] = entries[4 * e + 2];
        const uint64_t k = O.blk_idx(c.data());
        if (std::find(okey.begin(), okey.end(), k) == okey.end()) {
          okey.push_back(k);
          oc.push_back(c);
        }
      }
    std::vector<size_t> ord(oc.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return okey[x] < okey[y]; });
    O.coords.clear();
    for (size_t i : ord) O.coords.insert(O.coords.end(), oc[i].begin(), oc[i].end());
    O.nblk = (int64_t)oc.size();
    O.refresh_offsets();
    // per output slice (block, out_offset): its maps, in the reference's order
    std::vector<int64_t> slice_base(O.nblk + 1, 0);
    for (int64_t q = 0; q < O.nblk; ++q) slice_base[q + 1] = slice_base[q] + O.dim(q, axis);
    std::vector<std::vector<MonoMap>> slices(slice_base[O.nblk]);
    auto find_block = [&](const std::vector<int64_t>& c) {
      const uint64_t k = O.blk_idx(c.data());
      int64_t lo = 0, hi = O.nblk - 1;
      while (lo <= hi) {
        const int64_t mid = (lo + hi) / 2;
        const uint64_t km = O.blk_idx(&O.coords[mid * O.rank]);
        if (km == k) return mid;
        if (km < k) lo = mid + 1; else hi = mid - 1;
      }
      return (int64_t)-1;
    };
    for (int64_t b = 0; b < m.nblk; ++b)
      for (int64_t e = 0; e < nentries; ++e) {
        if (entries[4 * e] != m.coords[b * m.rank + axis]) continue;
        const double cr = coefs[e * per], ci = per == 2 ? coefs[e * per + 1] : 0.0;
        if (cr == 0.0 && ci == 0.0) continue;
        std::vector<int64_t> c(m.coords.begin() + b * m.rank, m.coords.begin() + (b + 1) * m.rank);
        c[axis] = entries[4 * e + 2];
        const int64_t q = find_block(c);
        slices[slice_base[q] + entries[4 * e + 3]].push_back(
            MonoMap{m.offsets[b], (int32_t)m.dim(b, axis), (int32_t)entries[4 * e + 1], cr, ci});
      }
    std::vector<MonoItem> items;
    std::vector<MonoMap> maps;
    for (int64_t q = 0; q < O.nblk; ++q) {
      int64_t outer = 1, inner = 1;
      for (int l = 0; l < axis; ++l) outer *= O.dim(q, l);
      for (int l = axis + 1; l < O.rank; ++l) inner *= O.dim(q, l);
      QLTG_CHECK(outer * inner < ((int64_t)1 << 31), QLTG_ERR_UNSUPPORTED, "block slice above 2^31 elements");
      for (int64_t o = 0; o < O.dim(q, axis); ++o) {
        auto& v = slices[slice_base[q] + o];
        items.push_back(MonoItem{O.offsets[q], (int32_t)O.dim(q, axis), (int32_t)o, (int32_t)outer, (int32_t)inner,
                                 (int32_t)maps.size(), (int32_t)(maps.size() + v.size())});
        maps.insert(maps.end(), v.begin(), v.end());
      }
    }
    cudaStream_t s;
    QLTG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    h->d_mono_items = upload(items, s);
    h->d_mono_maps = upload(maps, s);
    QLTG_CUDA(cudaStreamSynchronize(s));
    QLTG_CUDA(cudaStreamDestroy(s));
    h->mono_items = (int)items.size();
    *plan = h.release();
  });
}

int qltg_axis_project_plan_create(qltg_ctx* ctx, const qltg_tensor_desc* t, int32_t axis, const int64_t* kept_counts,
                                  const int64_t* kept, qltg_axis_plan** plan) {
  // ProjectAxis (dmrg/axis_ops.h:2469-2532) is the monomial with one unit entry per kept
  // degeneracy: (s, kept_s[j]) -> (s', j), s' counting the sectors that keep something
  std::vector<int32_t> oq;
  std::vector<int64_t> od, ent;
  std::vector<double> cf;
  int nc = 0, per = 1;
  int32_t out_nsct = 0;
  const int rc = guarded([&] {
    QLTG_CHECK(t && kept_counts, QLTG_ERR_INVALID, "null argument");
    const Meta m = meta_from_desc(t);
    require_bosonic_axis(m, axis);
    nc = m.ncomp;
    per = m.dtype == QLTG_C128 ? 2 : 1;
    int64_t pos = 0;
    for (int64_t s = 0; s < m.nsct(axis); ++s) {
      const int64_t cnt = kept_counts[s];
      QLTG_CHECK(cnt >= 0 && cnt <= m.dims[axis][s], QLTG_ERR_INVALID, "projector keeps more degeneracies than a sector has");
      QLTG_CHECK(cnt == 0 || kept, QLTG_ERR_INVALID, "null kept offsets");
      std::vector<int64_t> seen;
      for (int64_t j = 0; j < cnt; ++j) {
        const int64_t d = kept[pos + j];
        QLTG_CHECK(d >= 0 && d < m.dims[axis][s], QLTG_ERR_INVALID, "projector offset out of range");
        QLTG_CHECK(std::find(seen.begin(), seen.end(), d) == seen.end(), QLTG_ERR_INVALID,
                   "projector offset repeated within a sector");
        seen.push_back(d);
        ent.insert(ent.end(), {s, d, (int64_t)out_nsct, j});
        cf.push_back(1.0);
        if (per == 2) cf.push_back(0.0);
      }
      if (cnt > 0) {
        oq.insert(oq.end(), m.qns[axis].begin() + s * nc, m.qns[axis].begin() + (s + 1) * nc);
        od.push_back(cnt);
        ++out_nsct;
      }
      pos += cnt;
    }
    QLTG_CHECK(out_nsct > 0, QLTG_ERR_INVALID, "projector keeps no degeneracy");
  });
  if (rc != QLTG_OK) return rc;
  const std::vector<int32_t> flux(nc, 0);
  return qltg_axis_monomial_plan_create(ctx, t, axis, out_nsct, oq.data(), od.data(), flux.data(),
                                        (int64_t)ent.size() / 4, ent.data(), cf.data(), plan);
}

int qltg_axis_monomial_exec(qltg_axis_plan* plan, const void* in_dev, void* out_dev, const double* alpha,
                            const double* beta, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan && plan->mono, QLTG_ERR_INVALID, "not a monomial plan");
    QLTG_CHECK(in_dev && out_dev && alpha && beta, QLTG_ERR_INVALID, "null argument");
    QLTG_CHECK(in_dev != out_dev, QLTG_ERR_INVALID, "output aliases the input");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    if (!plan->mono_items) return;
    const bool cplx = plan->mono_out.dtype == QLTG_C128;
    QLTG_CHECK(cplx || (alpha[1] == 0.0 && beta[1] == 0.0), QLTG_ERR_INVALID, "complex alpha or beta for a real tensor");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int grid = std::min(plan->mono_items, std::max(1, plan->ctx->num_sms) * 8);
    const int read_out = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
    if (cplx)
      k_axis_monomial<double2><<<grid, 256, 0, s>>>(
          plan->d_mono_items.as<MonoItem>(), plan->mono_items, plan->d_mono_maps.as<MonoMap>(),
          static_cast<const double2*>(in_dev), static_cast<double2*>(out_dev), make_double2(alpha[0], alpha[1]),
          make_double2(beta[0], beta[1]), read_out);
    else
      k_axis_monomial<double><<<grid, 256, 0, s>>>(plan->d_mono_items.as<MonoItem>(), plan->mono_items,
                                                   plan->d_mono_maps.as<MonoMap>(), static_cast<const double*>(in_dev),
                                                   static_cast<double*>(out_dev), alpha[0], beta[0], read_out);
    QLTG_CUDA(cudaGetLastError());
  });
}

int qltg_axis_plan_result(const qltg_axis_plan* plan, int32_t* rank, int64_t* nblk, int64_t* size) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    if (rank) *rank = plan->out().rank;
    if (nblk) *nblk = plan->out().nblk;
    if (size) *size = plan->out().size;
  });
}

int qltg_axis_plan_result_blocks(const qltg_axis_plan* plan, int64_t* coords, int64_t* offsets) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    plan->out().export_arrays(nullptr, nullptr, nullptr, nullptr, coords, offsets);
  });
}

int qltg_axis_plan_exec(qltg_axis_plan* plan, const void* in_dev, const void* op1_dev, const void* op2_dev,
                        void* out_dev, int32_t mode, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan && in_dev && op1_dev && out_dev, QLTG_ERR_INVALID, "null argument");
    QLTG_CHECK(!plan->mono, QLTG_ERR_INVALID, "a monomial plan runs through qltg_axis_monomial_exec");
    QLTG_CHECK(!plan->two || op2_dev, QLTG_ERR_INVALID, "null second operator");
    QLTG_CHECK(out_dev != in_dev, QLTG_ERR_INVALID, "output aliases the input");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!plan->two) {
      plan->s1.exec(in_dev, op1_dev, out_dev, mode, s);
      return;
    }
    plan->s1.exec(in_dev, op1_dev, plan->mid.get(), mode, s);
    plan->s2.exec(plan->mid.get(), op2_dev, out_dev, mode, s);
  });
}

int qltg_axis_plan_device_status(qltg_axis_plan* plan, void* stream) {
  return guarded([&] {
    QLTG_CHECK(plan, QLTG_ERR_INVALID, "null plan");
    QLTG_CUDA(cudaSetDevice(plan->ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (plan->mono) return;
    QLTG_CHECK(split_device_error(plan->s1.c, s) == 0 && (!plan->two || split_device_error(plan->s2.c, s) == 0),
               QLTG_ERR_TIMEOUT, "a bounded tensor-core wait expired in the split-precision GEMM");
  });
}

int qltg_axis_plan_destroy(qltg_axis_plan* plan) {
  delete plan;
  return QLTG_OK;
}

}  // extern "C"
