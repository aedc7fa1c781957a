// CPU restatement of the reference's block-sparse Contract / SVD / QR, used ONLY as
// the correctness oracle and as the timed CPU baseline. It is test infrastructure:
// the GPU library never links, loads or calls it.
//
// Parity pinned against the reference itself: oracle/ref/ref_driver.cc runs the
// reference's own code on the same generated inputs, and the committed fixtures in
// tests/golden/ hold its outputs; tests/test_oracle_golden.py checks this file
// against them.
//
// Each step follows the reference (paths relative to the reference tree):
//  * pairing by VecPartHasher of contracted block coordinates, A blocks outer, B blocks
//    inner, m/k/n from block shapes, beta = 0 for the first pair that creates an output
//    block, fermion exchange sign per pair
//      qltensor/blk_spar_data_ten/data_blk_operations.h:411-578, :351-401
//      framework/vec_hash.h:39-51
//  * output legs = saved A legs ++ saved B legs (tensor_manipulation/ten_ctrct.h:372-394);
//    a transposes to (saved, contracted), b to (contracted, saved) only when those orders
//    are not already the identity (ten_ctrct.h:396-443)
//  * tasks sorted by (output block, beta) then executed as
//    C_blk = sign * A_t B_t + beta * C_blk with a row-major dgemm/zgemm
//      raw_data_operation_tasks.h:250-269, global_operations.h:895-992,
//      raw_data_operations.h:530-548, framework/hp_numeric/blas_level3.h:35-56
//  * contiguous-axes contraction: contracted axes (start + i) mod rank, saved axes in the
//    cyclic order from the end of the contracted range; a fermionic block whose saved legs
//    come out of ascending order takes the sign of that reordering (-1 per pair of odd legs
//    that trade places: the residue sign of the reference's rotated matrix view)
//      tensor_manipulation/contract_contiguous_axes.h:305-472, :849-868,
//      qltensor/blk_spar_data_ten/data_blk_operations.h:580-611
//  * accumulate: C = beta C + alpha A.B over the union of C's blocks and the contraction's;
//    beta = 0 never reads C; a missing block is an error unless expansion is allowed
//      tensor_manipulation/contract_contiguous_axes.h:557-783, :953-1040
//  * SVD: block-matrices grouped by (left flux, right flux) in first-appearance order,
//    dense gather, LAPACKE ?gesvd('S','S'), global descending sort, keep from Dmin while
//    kept_sv2 <= (1 - eps) total and <= Dmax, result tensors U / S / Vt
//      tensor_manipulation/ten_decomp/ten_decomp_basic.h:68-106,
//      qltensor/blk_spar_data_ten/data_blk_mat.h:39-131, raw_data_operations.h:550-575,
//      framework/hp_numeric/lapack.h:41-82, tensor_manipulation/ten_decomp/ten_svd.h:281-582,
//      data_blk_operations.h:969-1021
//  * QR: same grouping, ?geqrf + ?orgqr/?ungqr, Q / R scatter
//      framework/hp_numeric/lapack.h:332-366, tensor_manipulation/ten_decomp/ten_qr.h:125-291,
//      data_blk_operations.h:1048-1078
//
// BLAS/LAPACK come from an OpenBLAS shared library opened at run time (the one bundled
// with SciPy or NumPy), so the arithmetic kernels are the same OpenBLAS routines the
// reference CPU build calls.
#include <dlfcn.h>

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cplx = std::complex<double>;

// ------------------------------------------------------------------ BLAS binding
struct Blas {
  bool ilp64 = false;
  void* h = nullptr;
  void* dgemm = nullptr;
  void* zgemm = nullptr;
  void* dgesvd = nullptr;
  void* zgesvd = nullptr;
  void* dgeqrf = nullptr;
  void* dorgqr = nullptr;
  void* zgeqrf = nullptr;
  void* zungqr = nullptr;
  void* set_threads = nullptr;
} g_blas;

std::string g_err;

template <typename I>
struct Fn {
  using dgemm_t = void (*)(int, int, int, I, I, I, double, const double*, I, const double*, I, double, double*, I);
  using zgemm_t = void (*)(int, int, int, I, I, I, const void*, const void*, I, const void*, I, const void*, void*, I);
  using dgesvd_t = I (*)(int, char, char, I, I, double*, I, double*, double*, I, double*, I, double*);
  using zgesvd_t = I (*)(int, char, char, I, I, cplx*, I, double*, cplx*, I, cplx*, I, double*);
  using dgeqrf_t = I (*)(int, I, I, double*, I, double*);
  using dorgqr_t = I (*)(int, I, I, I, double*, I, const double*);
  using zgeqrf_t = I (*)(int, I, I, cplx*, I, cplx*);
  using zungqr_t = I (*)(int, I, I, I, cplx*, I, const cplx*);
};

constexpr int kRowMajor = 101, kNoTrans = 111;

void need_blas() {
  if (!g_blas.dgemm) throw std::runtime_error("oracle: BLAS library not loaded (orc_load_blas)");
}

void dgemm(int64_t m, int64_t n, int64_t k, double alpha, const double* a, const double* b, double beta,
           double* c) {
  need_blas();
  if (g_blas.ilp64)
    ((Fn<int64_t>::dgemm_t)g_blas.dgemm)(kRowMajor, kNoTrans, kNoTrans, m, n, k, alpha, a, k, b, n, beta, c, n);
  else
    ((Fn<int>::dgemm_t)g_blas.dgemm)(kRowMajor, kNoTrans, kNoTrans, (int)m, (int)n, (int)k, alpha, a, (int)k, b,
                                    (int)n, beta, c, (int)n);
}

void gemm(int64_t m, int64_t n, int64_t k, double alpha, const cplx* a, const cplx* b, double beta, cplx* c) {
  need_blas();
  cplx al(alpha, 0.0), be(beta, 0.0);
  if (g_blas.ilp64)
    ((Fn<int64_t>::zgemm_t)g_blas.zgemm)(kRowMajor, kNoTrans, kNoTrans, m, n, k, &al, a, k, b, n, &be, c, n);
  else
    ((Fn<int>::zgemm_t)g_blas.zgemm)(kRowMajor, kNoTrans, kNoTrans, (int)m, (int)n, (int)k, &al, a, (int)k, b,
                                    (int)n, &be, c, (int)n);
}
void gemm(int64_t m, int64_t n, int64_t k, double alpha, const double* a, const double* b, double beta,
          double* c) {
  dgemm(m, n, k, alpha, a, b, beta, c);
}

template <typename I, typename T>
int64_t gesvd_t(int64_t m, int64_t n, T* a, double* s, T* u, T* vt) {
  const int64_t k = std::min(m, n);
  std::vector<double> superb(std::max<int64_t>(1, m));
  if constexpr (std::is_same<T, double>::value)
    return ((typename Fn<I>::dgesvd_t)g_blas.dgesvd)(kRowMajor, 'S', 'S', (I)m, (I)n, a, (I)n, s, u, (I)k, vt,
                                                      (I)n, superb.data());
  else
    return ((typename Fn<I>::zgesvd_t)g_blas.zgesvd)(kRowMajor, 'S', 'S', (I)m, (I)n, a, (I)n, s, u, (I)k, vt,
                                                      (I)n, superb.data());
}
template <typename T>
int64_t gesvd(int64_t m, int64_t n, T* a, double* s, T* u, T* vt) {
  need_blas();
  return g_blas.ilp64 ? gesvd_t<int64_t, T>(m, n, a, s, u, vt) : gesvd_t<int, T>(m, n, a, s, u, vt);
}

template <typename I, typename T>
void geqr_t(int64_t m, int64_t n, T* a, T* tau, bool orth, int64_t k) {
  if constexpr (std::is_same<T, double>::value) {
    if (!orth) ((typename Fn<I>::dgeqrf_t)g_blas.dgeqrf)(kRowMajor, (I)m, (I)n, a, (I)n, tau);
    else ((typename Fn<I>::dorgqr_t)g_blas.dorgqr)(kRowMajor, (I)m, (I)k, (I)k, a, (I)n, tau);
  } else {
    if (!orth) ((typename Fn<I>::zgeqrf_t)g_blas.zgeqrf)(kRowMajor, (I)m, (I)n, a, (I)n, tau);
    else ((typename Fn<I>::zungqr_t)g_blas.zungqr)(kRowMajor, (I)m, (I)k, (I)k, a, (I)n, tau);
  }
}
template <typename T>
void geqrf(int64_t m, int64_t n, T* a, T* tau) {
  need_blas();
  g_blas.ilp64 ? geqr_t<int64_t, T>(m, n, a, tau, false, 0) : geqr_t<int, T>(m, n, a, tau, false, 0);
}
template <typename T>
void orgqr(int64_t m, int64_t n, int64_t k, T* a, const T* tau) {
  need_blas();
  g_blas.ilp64 ? geqr_t<int64_t, T>(m, n, a, const_cast<T*>(tau), true, k)
               : geqr_t<int, T>(m, n, a, const_cast<T*>(tau), true, k);
}

// ------------------------------------------------------------------ tensors
struct Leg {
  int32_t dir = 0;                 // 0 IN, 1 OUT
  std::vector<int32_t> qns;        // nsct * ncomp
  std::vector<int64_t> dims;
};

struct Tensor {
  int ncomp = 1;
  int parity_comp = -1;
  bool is_complex = false;
  std::vector<Leg> legs;
  std::vector<int64_t> coords;     // nblk * rank, ascending block index
  std::vector<int64_t> offsets;
  int64_t size = 0;
  std::vector<double> data;       // size or 2 * size

  int rank() const { return (int)legs.size(); }
  int64_t nblk() const { return rank() ? (int64_t)coords.size() / rank() : (size ? 1 : 0); }
  int64_t dim(int64_t b, int l) const { return legs[l].dims[coords[b * rank() + l]]; }
  int64_t blk_size(int64_t b) const {
    int64_t s = 1;
    for (int l = 0; l < rank(); ++l) s *= dim(b, l);
    return s;
  }
  bool parity(int l, int64_t sct) const {
    return parity_comp >= 0 && (legs[l].qns[sct * ncomp + parity_comp] % 2) != 0;
  }
  void refresh_offsets() {
    offsets.resize(nblk());
    int64_t off = 0;
    for (int64_t b = 0; b < nblk(); ++b) { offsets[b] = off; off += blk_size(b); }
    size = off;
  }
  // blk_idx = row-major linearisation of the sector coordinates
  uint64_t blk_idx(const int64_t* c) const {
    uint64_t idx = 0;
    for (int l = 0; l < rank(); ++l) idx = idx * (uint64_t)legs[l].dims.size() + (uint64_t)c[l];
    return idx;
  }
};

// ------------------------------------------------------------------ hashing
constexpr uint64_t kP1 = 11400714785074694791ULL, kP2 = 14029467366897019727ULL, kP5 = 2870177450012600261ULL;
inline uint64_t rot31(uint64_t x) { return (x << 31) | (x >> 33); }

uint64_t part_hash(const int64_t* coords, const std::vector<int64_t>& sel) {
  uint64_t h = kP5;
  for (auto i : sel) {
    h += (uint64_t)coords[i] * kP2;
    h = rot31(h);
    h *= kP1;
  }
  h += (uint64_t)sel.size() ^ kP5;
  return h;
}

// ------------------------------------------------------------------ fermion sign
int exchange_sign(const std::vector<bool>& pa, const std::vector<bool>& pb, const std::vector<int64_t>& axa,
                  const std::vector<int64_t>& axb, const std::vector<int32_t>& a_ctrct_dir) {
  int exchanges = 0;
  std::vector<bool> par = pa;
  par.insert(par.end(), pb.begin(), pb.end());
  const size_t ra = pa.size(), nc = axa.size();
  std::vector<int64_t> ax(2 * nc);
  for (size_t i = 0; i < nc; ++i) { ax[2 * i] = axa[i]; ax[2 * i + 1] = axb[i] + (int64_t)ra; }
  for (size_t i = 0; i < nc; ++i) {
    const int64_t x1 = ax[2 * i], x2 = ax[2 * i + 1];
    const bool p1 = par[x1], p2 = par[x2];
    if (p1 != p2) throw std::runtime_error("oracle: contracted legs with different parity");
    if (p2) exchanges += (int)std::count(par.begin() + x1 + 1, par.begin() + x2, true);
    std::rotate(par.begin() + x1 + 1, par.begin() + x2, par.begin() + x2 + 1);
    for (auto& a : ax)
      if (a > x1 && a < x2) a++;
    ax[2 * i + 1] = x1 + 1;
    exchanges += (p1 && a_ctrct_dir[i] == 0) ? 1 : 0;
  }
  return (exchanges & 1) ? -1 : 1;
}

// ------------------------------------------------------------------ transpose
template <typename T>
void transpose(const T* src, const std::vector<int64_t>& shape, const std::vector<int64_t>& order, T* dst) {
  const int r = (int)shape.size();
  std::vector<int64_t> sstride(r, 1);
  for (int i = r - 2; i >= 0; --i) sstride[i] = sstride[i + 1] * shape[i + 1];
  std::vector<int64_t> dshape(r), dstr(r);
  for (int i = 0; i < r; ++i) { dshape[i] = shape[order[i]]; dstr[i] = sstride[order[i]]; }
  int64_t n = 1;
  for (auto s : shape) n *= s;
  const int64_t inner = r ? dshape[r - 1] : 1, inner_st = r ? dstr[r - 1] : 0;
  const int64_t outer = inner ? n / inner : 0;
#pragma omp parallel for schedule(static) if (n > (1 << 16))
  for (int64_t o = 0; o < outer; ++o) {
    int64_t rem = o, src_off = 0;
    for (int i = r - 2; i >= 0; --i) { src_off += (rem % dshape[i]) * dstr[i]; rem /= dshape[i]; }
    T* d = dst + o * inner;
    for (int64_t j = 0; j < inner; ++j) d[j] = src[src_off + j * inner_st];
  }
}

// ------------------------------------------------------------------ contraction
struct Task {
  int64_t a, b;          // block ordinals in A / B
  uint64_t c_idx;        // output blk_idx
  int64_t m, k, n;
  int sign;
  int beta;
};

struct CtrctOut {
  Tensor c;
  std::vector<Task> tasks;   // generation order
};

std::vector<int64_t> saved_axes(int rank, const std::vector<int64_t>& ctrct) {
  std::vector<int64_t> s;
  for (int i = 0; i < rank; ++i)
    if (std::find(ctrct.begin(), ctrct.end(), i) == ctrct.end()) s.push_back(i);
  return s;
}

// Sign of reordering a block's saved legs from ascending leg order to `order`.
int saved_order_sign(const std::vector<bool>& par, const std::vector<int64_t>& order) {
  int n = 0;
  for (size_t i = 0; i < order.size(); ++i)
    for (size_t j = i + 1; j < order.size(); ++j)
      if (order[i] > order[j] && par[order[i]] && par[order[j]]) ++n;
  return (n & 1) ? -1 : 1;
}

bool is_identity(const std::vector<int64_t>& first, const std::vector<int64_t>& second) {
  for (size_t i = 0; i < first.size(); ++i) if (first[i] != (int64_t)i) return false;
  for (size_t i = 0; i < second.size(); ++i) if (second[i] != (int64_t)(i + first.size())) return false;
  return true;
}

template <typename T>
void run_tasks(const Tensor& a, const Tensor& b, const std::vector<int64_t>& axa, const std::vector<int64_t>& axb,
               const std::vector<int64_t>& sa, const std::vector<int64_t>& sb, CtrctOut& out) {
  Tensor& c = out.c;
  std::vector<int64_t> a_order = sa, b_order = axb;
  a_order.insert(a_order.end(), axa.begin(), axa.end());
  b_order.insert(b_order.end(), sb.begin(), sb.end());
  const bool a_trans = !is_identity(sa, axa), b_trans = !is_identity(axb, sb);
  c.data.assign(c.is_complex ? 2 * c.size : c.size, 0.0);
  if (out.tasks.empty()) return;
  std::vector<Task> tasks = out.tasks;
  std::stable_sort(tasks.begin(), tasks.end(), [](const Task& x, const Task& y) {
    return x.c_idx < y.c_idx || (x.c_idx == y.c_idx && x.beta < y.beta);
  });
  std::map<uint64_t, int64_t> c_pos;   // blk_idx -> ordinal
  for (int64_t i = 0; i < c.nblk(); ++i) c_pos[c.rank() ? c.blk_idx(&c.coords[i * c.rank()]) : 0] = i;
  std::unordered_map<int64_t, std::vector<T>> a_cache, b_cache;
  const T* ad = reinterpret_cast<const T*>(a.data.data());
  const T* bd = reinterpret_cast<const T*>(b.data.data());
  T* cd = reinterpret_cast<T*>(c.data.data());
  auto shape_of = [](const Tensor& t, int64_t blk) {
    std::vector<int64_t> s(t.rank());
    for (int l = 0; l < t.rank(); ++l) s[l] = t.dim(blk, l);
    return s;
  };
  for (auto& t : tasks) {
    const T* ap = ad + a.offsets[t.a];
    const T* bp = bd + b.offsets[t.b];
    if (a_trans) {
      auto it = a_cache.find(t.a);
      if (it == a_cache.end()) {
        std::vector<T> buf(a.blk_size(t.a));
        transpose(ap, shape_of(a, t.a), a_order, buf.data());
        it = a_cache.emplace(t.a, std::move(buf)).first;
      }
      ap = it->second.data();
    }
    if (b_trans) {
      auto it = b_cache.find(t.b);
      if (it == b_cache.end()) {
        std::vector<T> buf(b.blk_size(t.b));
        transpose(bp, shape_of(b, t.b), b_order, buf.data());
        it = b_cache.emplace(t.b, std::move(buf)).first;
      }
      bp = it->second.data();
    }
    T* cp = cd + (c.rank() ? c.offsets[c_pos.at(t.c_idx)] : 0);
    gemm(t.m, t.n, t.k, (double)t.sign, ap, bp, (double)t.beta, cp);
  }
}

// sa_order / sb_order: the saved legs in the order they take in C (empty: ascending).
CtrctOut contract(const Tensor& a, const Tensor& b, const std::vector<int64_t>& axa, const std::vector<int64_t>& axb,
                  const std::vector<int64_t>& sa_order = {}, const std::vector<int64_t>& sb_order = {}) {
  if (axa.size() != axb.size()) throw std::runtime_error("oracle: axes size mismatch");
  if (a.is_complex != b.is_complex) throw std::runtime_error("oracle: mixed element types");
  CtrctOut out;
  Tensor& c = out.c;
  c.ncomp = a.ncomp;
  c.parity_comp = a.parity_comp;
  c.is_complex = a.is_complex;
  const auto sa = sa_order.empty() ? saved_axes(a.rank(), axa) : sa_order;
  const auto sb = sb_order.empty() ? saved_axes(b.rank(), axb) : sb_order;
  for (auto i : sa) c.legs.push_back(a.legs[i]);
  for (auto i : sb) c.legs.push_back(b.legs[i]);
  const bool fermionic = a.parity_comp >= 0;
  std::vector<int32_t> a_dir;
  for (auto i : axa) a_dir.push_back(a.legs[i].dir);
  std::vector<uint64_t> ha(a.nblk()), hb(b.nblk());
  for (int64_t i = 0; i < a.nblk(); ++i) ha[i] = part_hash(&a.coords[i * a.rank()], axa);
  for (int64_t j = 0; j < b.nblk(); ++j) hb[j] = part_hash(&b.coords[j * b.rank()], axb);
  auto parities = [&](const Tensor& t, int64_t blk) {
    std::vector<bool> p(t.rank());
    for (int l = 0; l < t.rank(); ++l) p[l] = t.parity(l, t.coords[blk * t.rank() + l]);
    return p;
  };
  auto finish = [&]() {
    if (c.is_complex) run_tasks<cplx>(a, b, axa, axb, sa, sb, out); else run_tasks<double>(a, b, axa, axb, sa, sb, out);
  };
  auto prod = [](const Tensor& t, int64_t blk, const std::vector<int64_t>& axes) {
    int64_t s = 1;
    for (auto l : axes) s *= t.dim(blk, (int)l);
    return s;
  };
  if (sa.empty() && sb.empty()) {
    // scalar result: first matching B block per A block only
    for (int64_t i = 0; i < a.nblk(); ++i)
      for (int64_t j = 0; j < b.nblk(); ++j)
        if (ha[i] == hb[j]) {
          int sign = fermionic ? exchange_sign(parities(a, i), parities(b, j), axa, axb, a_dir) : 1;
          out.tasks.push_back({i, j, 0, 1, prod(a, i, axa), 1, sign, 1});
          break;
        }
    if (!out.tasks.empty()) { out.tasks[0].beta = 0; c.size = 1; c.offsets = {0}; }
    finish();
    return out;
  }
  std::map<uint64_t, std::vector<int64_t>> cblocks;   // blk_idx -> coords
  std::vector<int64_t> cc(c.rank());
  for (int64_t i = 0; i < a.nblk(); ++i) {
    for (int64_t j = 0; j < b.nblk(); ++j) {
      if (ha[i] != hb[j]) continue;
      const int64_t m = prod(a, i, sa), k = prod(a, i, axa), n = prod(b, j, sb);
      size_t p = 0;
      for (auto l : sa) cc[p++] = a.coords[i * a.rank() + l];
      for (auto l : sb) cc[p++] = b.coords[j * b.rank() + l];
      const uint64_t cidx = c.blk_idx(cc.data());
      int beta = 1;
      if (!cblocks.count(cidx)) { cblocks[cidx] = cc; beta = 0; }
      int sign = 1;
      if (fermionic) {
        const auto pa = parities(a, i), pb = parities(b, j);
        sign = exchange_sign(pa, pb, axa, axb, a_dir) * saved_order_sign(pa, sa) * saved_order_sign(pb, sb);
      }
      out.tasks.push_back({i, j, cidx, m, k, n, sign, beta});
    }
  }
  for (auto& kv : cblocks) c.coords.insert(c.coords.end(), kv.second.begin(), kv.second.end());
  c.refresh_offsets();
  finish();
  return out;
}

// ------------------------------------------------------------------ decompositions
struct BlkMat {
  std::vector<int32_t> lflux, rflux, mid;
  int64_t rows = 0, cols = 0;
  std::vector<std::vector<int64_t>> rkeys, ckeys;
  std::vector<int64_t> roff, rdim, coff, cdim;
  std::vector<int64_t> eblk, erow, ecol;
};

std::vector<int32_t> tensor_div(const Tensor& t) {
  std::vector<int32_t> d(t.ncomp, 0);
  if (t.nblk() == 0 || t.rank() == 0) return d;
  for (int l = 0; l < t.rank(); ++l)
    for (int k = 0; k < t.ncomp; ++k) {
      int32_t q = t.legs[l].qns[t.coords[l] * t.ncomp + k];
      d[k] += t.legs[l].dir == 1 ? q : -q;
    }
  return d;
}

std::vector<BlkMat> group_blocks(const Tensor& t, int ldims, const std::vector<int32_t>& lqndiv) {
  std::vector<BlkMat> mats;
  const auto div = tensor_div(t);
  const int r = t.rank(), nc = t.ncomp;
  for (int64_t b = 0; b < t.nblk(); ++b) {
    std::vector<int32_t> lf(nc, 0), rf(nc), mid(nc);
    for (int l = 0; l < ldims; ++l)
      for (int k = 0; k < nc; ++k) {
        int32_t q = t.legs[l].qns[t.coords[b * r + l] * nc + k];
        lf[k] += t.legs[l].dir == 1 ? q : -q;
      }
    for (int k = 0; k < nc; ++k) { rf[k] = div[k] - lf[k]; mid[k] = lqndiv[k] - lf[k]; }
    int64_t m = 1, n = 1;
    for (int l = 0; l < ldims; ++l) m *= t.dim(b, l);
    for (int l = ldims; l < r; ++l) n *= t.dim(b, l);
    size_t g = 0;
    for (; g < mats.size(); ++g) if (mats[g].lflux == lf && mats[g].rflux == rf) break;
    if (g == mats.size()) { mats.emplace_back(); mats[g].lflux = lf; mats[g].rflux = rf; mats[g].mid = mid; }
    auto& M = mats[g];
    std::vector<int64_t> lk(t.coords.begin() + b * r, t.coords.begin() + b * r + ldims);
    std::vector<int64_t> rk(t.coords.begin() + b * r + ldims, t.coords.begin() + b * r + r);
    size_t i = 0;
    for (; i < M.rkeys.size(); ++i) if (M.rkeys[i] == lk) break;
    if (i == M.rkeys.size()) { M.rkeys.push_back(lk); M.roff.push_back(M.rows); M.rdim.push_back(m); M.rows += m; }
    size_t j = 0;
    for (; j < M.ckeys.size(); ++j) if (M.ckeys[j] == rk) break;
    if (j == M.ckeys.size()) { M.ckeys.push_back(rk); M.coff.push_back(M.cols); M.cdim.push_back(n); M.cols += n; }
    M.eblk.push_back(b); M.erow.push_back(i); M.ecol.push_back(j);
  }
  return mats;
}

template <typename T>
std::vector<T> dense_of(const Tensor& t, const BlkMat& M) {
  std::vector<T> d(M.rows * M.cols, T(0));
  const T* src = reinterpret_cast<const T*>(t.data.data());
  for (size_t e = 0; e < M.eblk.size(); ++e) {
    const int64_t b = M.eblk[e], ro = M.roff[M.erow[e]], rd = M.rdim[M.erow[e]];
    const int64_t co = M.coff[M.ecol[e]], cd = M.cdim[M.ecol[e]];
    for (int64_t i = 0; i < rd; ++i)
      for (int64_t j = 0; j < cd; ++j) d[(ro + i) * M.cols + co + j] = src[t.offsets[b] + i * cd + j];
  }
  return d;
}

Leg mid_leg(const std::vector<std::vector<int32_t>>& qns, const std::vector<int64_t>& dims, int dir) {
  Leg l;
  l.dir = dir;
  for (auto& q : qns) l.qns.insert(l.qns.end(), q.begin(), q.end());
  l.dims = dims;
  return l;
}

// Insert a block by coordinates keeping ascending blk_idx order; returns nothing, the
// caller refreshes offsets once all blocks exist.
void sort_blocks(Tensor& t) {
  const int r = t.rank();
  std::vector<std::pair<uint64_t, std::vector<int64_t>>> v;
  for (int64_t b = 0; b < t.nblk(); ++b) {
    std::vector<int64_t> c(t.coords.begin() + b * r, t.coords.begin() + b * r + r);
    v.push_back({t.blk_idx(c.data()), c});
  }
  std::sort(v.begin(), v.end());
  t.coords.clear();
  for (auto& x : v) t.coords.insert(t.coords.end(), x.second.begin(), x.second.end());
  t.refresh_offsets();
}

int64_t find_block(const Tensor& t, const std::vector<int64_t>& c) {
  const int r = t.rank();
  for (int64_t b = 0; b < t.nblk(); ++b)
    if (std::equal(c.begin(), c.end(), t.coords.begin() + b * r)) return b;
  return -1;
}

struct SvdOut {
  Tensor u, s, vt;
  double err = 0;
  int64_t D = 0;
};

template <typename T>
SvdOut svd_impl(const Tensor& t, int ldims, const std::vector<int32_t>& lqndiv, double trunc, int64_t dmin,
                int64_t dmax) {
  auto mats = group_blocks(t, ldims, lqndiv);
  struct Res { int64_t m, n, k; std::vector<T> u, vt; std::vector<double> s; };
  std::vector<Res> res(mats.size());
  for (size_t g = 0; g < mats.size(); ++g) {
    auto d = dense_of<T>(t, mats[g]);
    Res& R = res[g];
    R.m = mats[g].rows; R.n = mats[g].cols; R.k = std::min(R.m, R.n);
    R.u.resize(R.m * R.k); R.vt.resize(R.k * R.n); R.s.resize(R.k);
    if (gesvd<T>(R.m, R.n, d.data(), R.s.data(), R.u.data(), R.vt.data()) != 0)
      throw std::runtime_error("oracle: gesvd failed");
  }
  // (sv, group, in-group index, sv^2)
  struct SV { double sv; int64_t g, i; double sv2; };
  std::vector<SV> info;
  for (size_t g = 0; g < res.size(); ++g)
    for (int64_t i = 0; i < res[g].k; ++i)
      if (res[g].s[i] != 0.0) info.push_back({res[g].s[i], (int64_t)g, i, res[g].s[i] * res[g].s[i]});
  SvdOut out;
  const int64_t total = (int64_t)info.size();
  if (total <= dmin) {
    out.err = 0; out.D = total;
  } else {
    std::stable_sort(info.begin(), info.end(), [](const SV& x, const SV& y) { return x.sv > y.sv; });
    double total2 = 0;
    for (auto& x : info) total2 += x.sv2;
    const double target = total2 * (1 - trunc);
    int64_t kept = dmin;
    double kept2 = 0;
    for (int64_t i = 0; i < kept; ++i) kept2 += info[i].sv2;
    while (true) {
      if (kept2 > target) break;
      const int64_t next = kept + 1;
      if (next > total) break;
      const double next2 = kept2 + info[next - 1].sv2;
      if (next > dmax) break;
      kept = next; kept2 = next2;
    }
    const double e = 1 - kept2 / total2;
    out.err = e > 0 ? e : 0;
    out.D = kept;
    info.resize(kept);
    std::stable_sort(info.begin(), info.end(),
                     [](const SV& x, const SV& y) { return x.g < y.g || (x.g == y.g && x.i < y.i); });
  }
  if (info.empty()) throw std::runtime_error("EmptySVDResult");
  // group -> (mid sector coordinate, kept svs, kept in-group indices)
  std::map<int64_t, std::pair<std::vector<double>, std::vector<int64_t>>> kept;
  for (auto& x : info) { kept[x.g].first.push_back(x.sv); kept[x.g].second.push_back(x.i); }
  std::vector<std::vector<int32_t>> mq;
  std::vector<int64_t> md;
  for (auto& kv : kept) { mq.push_back(mats[kv.first].mid); md.push_back((int64_t)kv.second.first.size()); }
  Leg mout = mid_leg(mq, md, 1), min_ = mid_leg(mq, md, 0);
  for (Tensor* x : {&out.u, &out.s, &out.vt}) { x->ncomp = t.ncomp; x->parity_comp = t.parity_comp; }
  out.u.is_complex = out.vt.is_complex = t.is_complex;
  out.s.is_complex = false;
  out.u.legs.assign(t.legs.begin(), t.legs.begin() + ldims); out.u.legs.push_back(mout);
  out.vt.legs = {min_}; out.vt.legs.insert(out.vt.legs.end(), t.legs.begin() + ldims, t.legs.end());
  out.s.legs = {min_, mout};
  int64_t mc = 0;
  for (auto& kv : kept) {
    const auto& M = mats[kv.first];
    out.s.coords.insert(out.s.coords.end(), {mc, mc});
    for (auto& rk : M.rkeys) { out.u.coords.insert(out.u.coords.end(), rk.begin(), rk.end()); out.u.coords.push_back(mc); }
    for (auto& ck : M.ckeys) { out.vt.coords.push_back(mc); out.vt.coords.insert(out.vt.coords.end(), ck.begin(), ck.end()); }
    ++mc;
  }
  sort_blocks(out.u); sort_blocks(out.s); sort_blocks(out.vt);
  out.u.data.assign(out.u.is_complex ? 2 * out.u.size : out.u.size, 0.0);
  out.vt.data.assign(out.vt.is_complex ? 2 * out.vt.size : out.vt.size, 0.0);
  out.s.data.assign(out.s.size, 0.0);
  T* ud = reinterpret_cast<T*>(out.u.data.data());
  T* vd = reinterpret_cast<T*>(out.vt.data.data());
  mc = 0;
  for (auto& kv : kept) {
    const auto& M = mats[kv.first];
    const auto& R = res[kv.first];
    const auto& cols = kv.second.second;
    const int64_t kd = (int64_t)cols.size();
    int64_t sb = find_block(out.s, {mc, mc});
    for (int64_t i = 0; i < kd; ++i) out.s.data[out.s.offsets[sb] + i * kd + i] = kv.second.first[i];
    for (size_t ri = 0; ri < M.rkeys.size(); ++ri) {
      auto c = M.rkeys[ri]; c.push_back(mc);
      int64_t b = find_block(out.u, c);
      for (int64_t i = 0; i < M.rdim[ri]; ++i)
        for (int64_t j = 0; j < kd; ++j) ud[out.u.offsets[b] + i * kd + j] = R.u[(M.roff[ri] + i) * R.k + cols[j]];
    }
    for (size_t ci = 0; ci < M.ckeys.size(); ++ci) {
      std::vector<int64_t> c = {mc}; c.insert(c.end(), M.ckeys[ci].begin(), M.ckeys[ci].end());
      int64_t b = find_block(out.vt, c);
      for (int64_t i = 0; i < kd; ++i)
        for (int64_t j = 0; j < M.cdim[ci]; ++j) vd[out.vt.offsets[b] + i * M.cdim[ci] + j] = R.vt[cols[i] * R.n + M.coff[ci] + j];
    }
    ++mc;
  }
  return out;
}

struct QrOut { Tensor q, r; };

template <typename T>
QrOut qr_impl(const Tensor& t, int ldims, const std::vector<int32_t>& lqndiv) {
  auto mats = group_blocks(t, ldims, lqndiv);
  QrOut out;
  std::vector<std::vector<int32_t>> mq;
  std::vector<int64_t> md;
  for (auto& M : mats) { mq.push_back(M.mid); md.push_back(std::min(M.rows, M.cols)); }
  Leg mout = mid_leg(mq, md, 1), min_ = mid_leg(mq, md, 0);
  for (Tensor* x : {&out.q, &out.r}) { x->ncomp = t.ncomp; x->parity_comp = t.parity_comp; x->is_complex = t.is_complex; }
  out.q.legs.assign(t.legs.begin(), t.legs.begin() + ldims); out.q.legs.push_back(mout);
  out.r.legs = {min_}; out.r.legs.insert(out.r.legs.end(), t.legs.begin() + ldims, t.legs.end());
  for (int64_t g = 0; g < (int64_t)mats.size(); ++g) {
    for (auto& rk : mats[g].rkeys) { out.q.coords.insert(out.q.coords.end(), rk.begin(), rk.end()); out.q.coords.push_back(g); }
    for (auto& ck : mats[g].ckeys) { out.r.coords.push_back(g); out.r.coords.insert(out.r.coords.end(), ck.begin(), ck.end()); }
  }
  sort_blocks(out.q); sort_blocks(out.r);
  out.q.data.assign(t.is_complex ? 2 * out.q.size : out.q.size, 0.0);
  out.r.data.assign(t.is_complex ? 2 * out.r.size : out.r.size, 0.0);
  T* qd = reinterpret_cast<T*>(out.q.data.data());
  T* rd = reinterpret_cast<T*>(out.r.data.data());
  for (int64_t g = 0; g < (int64_t)mats.size(); ++g) {
    const auto& M = mats[g];
    auto a = dense_of<T>(t, M);
    const int64_t m = M.rows, n = M.cols, k = std::min(m, n);
    std::vector<T> tau(std::max<int64_t>(1, k));
    geqrf<T>(m, n, a.data(), tau.data());
    std::vector<T> R(k * n, T(0));
    for (int64_t i = 0; i < k; ++i)
      for (int64_t j = i; j < n; ++j) R[i * n + j] = a[i * n + j];
    orgqr<T>(m, n, k, a.data(), tau.data());
    for (size_t ri = 0; ri < M.rkeys.size(); ++ri) {
      auto c = M.rkeys[ri]; c.push_back(g);
      int64_t b = find_block(out.q, c);
      for (int64_t i = 0; i < M.rdim[ri]; ++i)
        for (int64_t j = 0; j < k; ++j) qd[out.q.offsets[b] + i * k + j] = a[(M.roff[ri] + i) * n + j];
    }
    for (size_t ci = 0; ci < M.ckeys.size(); ++ci) {
      std::vector<int64_t> c = {g}; c.insert(c.end(), M.ckeys[ci].begin(), M.ckeys[ci].end());
      int64_t b = find_block(out.r, c);
      for (int64_t i = 0; i < k; ++i)
        for (int64_t j = 0; j < M.cdim[ci]; ++j) rd[out.r.offsets[b] + i * M.cdim[ci] + j] = R[i * n + M.coff[ci] + j];
    }
  }
  return out;
}

// ------------------------------------------------------------------ C interface glue
struct Result {
  std::vector<std::unique_ptr<Tensor>> tensors;
  std::vector<double> scalars;
  std::vector<int64_t> tasks;    // generation order: a_blk_idx, b_blk_idx, c_blk_idx, m, k, n, sign, beta
};

}  // namespace

extern "C" {

struct OrcTensorIn {
  int32_t rank, ncomp, parity_comp, is_complex;
  const int32_t* dirs;
  const int32_t* nsct;
  const int32_t* qns;
  const int64_t* dims;
  int64_t nblk;
  const int64_t* coords;
  const double* data;
};

static Tensor from_in(const OrcTensorIn* in) {
  Tensor t;
  t.ncomp = in->ncomp;
  t.parity_comp = in->parity_comp;
  t.is_complex = in->is_complex != 0;
  int64_t qpos = 0, dpos = 0;
  for (int l = 0; l < in->rank; ++l) {
    Leg leg;
    leg.dir = in->dirs[l];
    leg.qns.assign(in->qns + qpos, in->qns + qpos + (int64_t)in->nsct[l] * in->ncomp);
    leg.dims.assign(in->dims + dpos, in->dims + dpos + in->nsct[l]);
    qpos += (int64_t)in->nsct[l] * in->ncomp;
    dpos += in->nsct[l];
    t.legs.push_back(std::move(leg));
  }
  t.coords.assign(in->coords, in->coords + in->nblk * in->rank);
  t.refresh_offsets();
  for (int64_t b = 1; b < t.nblk(); ++b)
    if (t.blk_idx(&t.coords[(b - 1) * t.rank()]) >= t.blk_idx(&t.coords[b * t.rank()]))
      throw std::runtime_error("oracle: blocks not in ascending block index order");
  t.data.assign(in->data, in->data + (t.is_complex ? 2 : 1) * t.size);
  return t;
}

const char* orc_last_error(void) { return g_err.c_str(); }

int orc_load_blas(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) { g_err = dlerror(); return 1; }
  auto sym = [&](const char* lp, const char* ilp) -> void* {
    void* p = dlsym(h, lp);
    if (p) return p;
    return ilp ? dlsym(h, ilp) : nullptr;
  };
  Blas b;
  b.h = h;
  const char* probe[][2] = {{"scipy_cblas_dgemm", nullptr}, {"cblas_dgemm", nullptr}};
  for (auto& p : probe) if ((b.dgemm = dlsym(h, p[0]))) break;
  std::string pre = dlsym(h, "scipy_cblas_dgemm") ? "scipy_" : "";
  std::string suf = "";
  if (!b.dgemm && dlsym(h, "scipy_cblas_dgemm64_")) { pre = "scipy_"; suf = "64_"; b.ilp64 = true; }
  auto get = [&](const std::string& n) { return sym((pre + n + suf).c_str(), nullptr); };
  b.dgemm = get("cblas_dgemm");
  b.zgemm = get("cblas_zgemm");
  b.dgesvd = get("LAPACKE_dgesvd");
  b.zgesvd = get("LAPACKE_zgesvd");
  b.dgeqrf = get("LAPACKE_dgeqrf");
  b.dorgqr = get("LAPACKE_dorgqr");
  b.zgeqrf = get("LAPACKE_zgeqrf");
  b.zungqr = get("LAPACKE_zungqr");
  b.set_threads = get("openblas_set_num_threads");
  if (!b.dgemm || !b.zgemm || !b.dgesvd || !b.zgesvd || !b.dgeqrf || !b.dorgqr || !b.zgeqrf || !b.zungqr) {
    g_err = "oracle: BLAS/LAPACKE symbols missing in " + std::string(path);
    return 1;
  }
  g_blas = b;
  return 0;
}

int orc_set_threads(int n) {
  if (g_blas.set_threads) ((void (*)(int))g_blas.set_threads)(n);
#ifdef _OPENMP
  omp_set_num_threads(n);
#endif
  return 0;
}

void* orc_contract(const OrcTensorIn* a, const OrcTensorIn* b, const int64_t* axa, const int64_t* axb, int n) {
  try {
    Tensor ta = from_in(a), tb = from_in(b);
    std::vector<int64_t> va(axa, axa + n), vb(axb, axb + n);
    auto out = contract(ta, tb, va, vb);
    auto* r = new Result;
    r->tensors.emplace_back(new Tensor(std::move(out.c)));
    for (auto& t : out.tasks)
      r->tasks.insert(r->tasks.end(), {(int64_t)ta.blk_idx(&ta.coords[t.a * ta.rank()]),
                                       (int64_t)tb.blk_idx(&tb.coords[t.b * tb.rank()]), (int64_t)t.c_idx, t.m,
                                       t.k, t.n, (int64_t)t.sign, (int64_t)t.beta});
    return r;
  } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

// ContractContiguousAxes: axes (start + i) mod rank, saved legs cyclic from the range end.
static void contiguous_axes(int ra, int rb, int64_t a0, int64_t b0, int n, std::vector<int64_t>& axa,
                            std::vector<int64_t>& axb, std::vector<int64_t>& sa, std::vector<int64_t>& sb) {
  if (n < 1 || n > ra || n > rb || a0 < 0 || a0 >= ra || b0 < 0 || b0 >= rb)
    throw std::runtime_error("oracle: contiguous axis range out of bounds");
  for (int i = 0; i < n; ++i) { axa.push_back((a0 + i) % ra); axb.push_back((b0 + i) % rb); }
  for (int i = 0; i < ra - n; ++i) sa.push_back((a0 + n + i) % ra);
  for (int i = 0; i < rb - n; ++i) sb.push_back((b0 + n + i) % rb);
}

void* orc_contract_contiguous(const OrcTensorIn* a, const OrcTensorIn* b, int64_t a0, int64_t b0, int n) {
  try {
    Tensor ta = from_in(a), tb = from_in(b);
    std::vector<int64_t> axa, axb, sa, sb;
    contiguous_axes(ta.rank(), tb.rank(), a0, b0, n, axa, axb, sa, sb);
    auto out = contract(ta, tb, axa, axb, sa, sb);
    auto* r = new Result;
    r->tensors.emplace_back(new Tensor(std::move(out.c)));
    return r;
  } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

// C = beta C + alpha A.B (tail/head contiguous contraction) over the union topology.
// c_in NULL: the default output (beta must be 0). *status: 0 done, 1 layout mismatch (the
// indexes differ, or blocks are missing and expansion is not allowed; nothing computed).
void* orc_accumulate(const OrcTensorIn* a, const OrcTensorIn* b, int64_t a0, int64_t b0, int n,
                     const double* alpha, const double* beta, const OrcTensorIn* c_in, int allow_expand,
                     int* status) {
  try {
    *status = 0;
    Tensor ta = from_in(a), tb = from_in(b);
    std::vector<int64_t> axa, axb, sa, sb;
    contiguous_axes(ta.rank(), tb.rank(), a0, b0, n, axa, axb, sa, sb);
    Tensor t = contract(ta, tb, axa, axb, sa, sb).c;
    const cplx al(alpha[0], alpha[1]), be(beta[0], beta[1]);
    if (!c_in && be != cplx(0.0)) throw std::runtime_error("oracle: accumulate into a default output needs beta == 0");
    Tensor c0;
    if (c_in) {
      c0 = from_in(c_in);
      bool same = c0.rank() == t.rank() && c0.ncomp == t.ncomp && c0.is_complex == t.is_complex;
      for (int l = 0; same && l < t.rank(); ++l)
        same = c0.legs[l].dir == t.legs[l].dir && c0.legs[l].qns == t.legs[l].qns && c0.legs[l].dims == t.legs[l].dims;
      if (!same) { *status = 1; return nullptr; }
    }
    // union topology
    std::map<uint64_t, std::pair<int64_t, int64_t>> blocks;   // blk_idx -> (ordinal in c0, ordinal in t)
    const int r = t.rank();
    if (c_in)
      for (int64_t i = 0; i < c0.nblk(); ++i) blocks[r ? c0.blk_idx(&c0.coords[i * r]) : 0] = {i, -1};
    bool missing = false;
    for (int64_t i = 0; i < t.nblk(); ++i) {
      const uint64_t k = r ? t.blk_idx(&t.coords[i * r]) : 0;
      auto it = blocks.find(k);
      if (it == blocks.end()) { blocks[k] = {-1, i}; missing = true; }
      else it->second.second = i;
    }
    if (c_in && missing && !allow_expand) { *status = 1; return nullptr; }
    Tensor c;
    c.ncomp = t.ncomp;
    c.parity_comp = t.parity_comp;
    c.is_complex = t.is_complex;
    c.legs = t.legs;
    if (r == 0) {   // scalar output: one value
      c.size = 1;
      c.offsets = {0};
    } else {
      for (auto& kv : blocks) {
        const Tensor& src = kv.second.first >= 0 ? c0 : t;
        const int64_t ord = kv.second.first >= 0 ? kv.second.first : kv.second.second;
        c.coords.insert(c.coords.end(), src.coords.begin() + ord * r, src.coords.begin() + (ord + 1) * r);
      }
      c.refresh_offsets();
    }
    const int per = c.is_complex ? 2 : 1;
    c.data.assign((size_t)per * c.size, 0.0);
    auto get = [&](const Tensor& x, int64_t e) {
      return x.is_complex ? cplx(x.data[2 * e], x.data[2 * e + 1]) : cplx(x.data[e], 0.0);
    };
    auto put = [&](int64_t e, cplx v) {
      if (c.is_complex) { c.data[2 * e] = v.real(); c.data[2 * e + 1] = v.imag(); } else c.data[e] = v.real();
    };
    auto combine = [&](int64_t dst, int64_t n_el, int64_t old_off, int64_t t_off) {
      for (int64_t e = 0; e < n_el; ++e) {
        cplx v(0.0);
        if (old_off >= 0 && be != cplx(0.0)) v += be * get(c0, old_off + e);
        if (t_off >= 0) v += al * get(t, t_off + e);
        put(dst + e, v);
      }
    };
    if (r == 0) {
      combine(0, 1, c_in && c0.size ? 0 : -1, t.size ? 0 : -1);
    } else {
      int64_t q = 0;
      for (auto& kv : blocks) {
        const int64_t o = kv.second.first, ti = kv.second.second;
        combine(c.offsets[q], c.blk_size(q), o >= 0 ? c0.offsets[o] : -1, ti >= 0 ? t.offsets[ti] : -1);
        ++q;
      }
    }
    auto* res = new Result;
    res->tensors.emplace_back(new Tensor(std::move(c)));
    return res;
  } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

void* orc_svd(const OrcTensorIn* t, int ldims, const int32_t* lqndiv, double trunc, int64_t dmin, int64_t dmax) {
  try {
    Tensor tt = from_in(t);
    std::vector<int32_t> div(lqndiv, lqndiv + tt.ncomp);
    SvdOut o = tt.is_complex ? svd_impl<cplx>(tt, ldims, div, trunc, dmin, dmax)
                             : svd_impl<double>(tt, ldims, div, trunc, dmin, dmax);
    auto* r = new Result;
    r->tensors.emplace_back(new Tensor(std::move(o.u)));
    r->tensors.emplace_back(new Tensor(std::move(o.s)));
    r->tensors.emplace_back(new Tensor(std::move(o.vt)));
    r->scalars = {o.err, (double)o.D};
    return r;
  } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

void* orc_qr(const OrcTensorIn* t, int ldims, const int32_t* lqndiv) {
  try {
    Tensor tt = from_in(t);
    std::vector<int32_t> div(lqndiv, lqndiv + tt.ncomp);
    QrOut o = tt.is_complex ? qr_impl<cplx>(tt, ldims, div) : qr_impl<double>(tt, ldims, div);
    auto* r = new Result;
    r->tensors.emplace_back(new Tensor(std::move(o.q)));
    r->tensors.emplace_back(new Tensor(std::move(o.r)));
    return r;
  } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

void orc_free(void* r) { delete static_cast<Result*>(r); }

int64_t orc_num_tasks(void* r) { return (int64_t)static_cast<Result*>(r)->tasks.size() / 8; }
void orc_tasks(void* r, int64_t* out) {
  auto& v = static_cast<Result*>(r)->tasks;
  std::copy(v.begin(), v.end(), out);
}
double orc_scalar(void* r, int i) { return static_cast<Result*>(r)->scalars.at(i); }

// info: rank, ncomp, parity_comp, is_complex, nblk, size, total sectors
void orc_tensor_info(void* r, int i, int64_t* info) {
  const Tensor& t = *static_cast<Result*>(r)->tensors.at(i);
  int64_t ts = 0;
  for (auto& l : t.legs) ts += (int64_t)l.dims.size();
  info[0] = t.rank(); info[1] = t.ncomp; info[2] = t.parity_comp; info[3] = t.is_complex;
  info[4] = t.nblk(); info[5] = t.size; info[6] = ts;
}

void orc_tensor_export(void* r, int i, int32_t* dirs, int32_t* nsct, int32_t* qns, int64_t* dims, int64_t* coords,
                       int64_t* offsets, double* data) {
  const Tensor& t = *static_cast<Result*>(r)->tensors.at(i);
  int64_t qp = 0, dp = 0;
  for (int l = 0; l < t.rank(); ++l) {
    dirs[l] = t.legs[l].dir;
    nsct[l] = (int32_t)t.legs[l].dims.size();
    for (auto q : t.legs[l].qns) qns[qp++] = q;
    for (auto d : t.legs[l].dims) dims[dp++] = d;
  }
  std::copy(t.coords.begin(), t.coords.end(), coords);
  std::copy(t.offsets.begin(), t.offsets.end(), offsets);
  std::copy(t.data.begin(), t.data.end(), data);
}

}  // extern "C"
