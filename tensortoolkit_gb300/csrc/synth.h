// Deterministic synthetic block-sparse workloads for the two-site H*psi matvec,
// the block-diagonal SVD/QR and the fermionic U(1)xU(1) Hubbard case.
//
// Header-only C++17 with no dependencies, so the same bytes are produced by the
// GPU library's workload helper, the CPU restatement used as oracle and the
// driver that runs the reference implementation.
//
// Layout rules mirrored from the reference's BlockSparseDataTensor:
//  * a block exists iff the quantum-number divergence of its sector coordinates
//    equals the requested divergence (QLTensor::Fill, qltensor/qltensor_impl.h:416-441;
//    CalcDiv, qltensor/index.h:267-285: OUT legs add their QN, IN legs subtract it);
//  * blocks are stored in ascending block index, blk_idx = row-major linearisation of
//    the sector coordinates (blk_spar_data_ten.h:380-382, utility/utils_inl.h:125-148),
//    each block row-major over its degeneracy dims, offsets cumulative
//    (data_blk_operations.h:137-145).
//
// Random numbers: std::mt19937_64 (its output sequence is fixed by the C++ standard)
// feeding an explicit Box-Muller transform, because std::normal_distribution is
// implementation-defined.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <random>
#include <stdexcept>
#include <vector>

namespace qltg_synth {

enum : int { DIR_IN = 0, DIR_OUT = 1 };

struct Leg {
  int dir = DIR_IN;
  int ncomp = 1;                 // components of one quantum number
  std::vector<int32_t> qns;      // [nsct * ncomp]
  std::vector<int64_t> dims;     // [nsct] sector degeneracies
  int parity_comp = -1;          // component whose oddness is the fermion parity; -1 = bosonic

  int64_t nsct() const { return (int64_t)dims.size(); }
  int64_t total_dim() const { return std::accumulate(dims.begin(), dims.end(), (int64_t)0); }
  bool parity(int64_t s) const {
    return parity_comp >= 0 && (qns[s * ncomp + parity_comp] % 2) != 0;
  }
  Leg inverse() const { Leg l = *this; l.dir = 1 - dir; return l; }
};

struct Tensor {
  std::vector<Leg> legs;
  bool is_complex = false;
  std::vector<int64_t> coords;   // [nblk * rank] in ascending block index
  std::vector<int64_t> offsets;  // [nblk] element offsets
  int64_t size = 0;              // number of elements
  std::vector<double> data;      // size (real) or 2*size (interleaved re,im)

  int rank() const { return (int)legs.size(); }
  int64_t nblk() const { return rank() ? (int64_t)coords.size() / rank() : 0; }
  int64_t blk_dim(int64_t b, int leg) const {
    return legs[leg].dims[coords[b * rank() + leg]];
  }
  int64_t blk_size(int64_t b) const {
    int64_t s = 1;
    for (int l = 0; l < rank(); ++l) s *= blk_dim(b, l);
    return s;
  }
  int ncomp() const { return legs.empty() ? 1 : legs[0].ncomp; }
  bool fermionic() const { return !legs.empty() && legs[0].parity_comp >= 0; }
};

// ---------------------------------------------------------------------------
// Random numbers
// ---------------------------------------------------------------------------
class Normal {
 public:
  explicit Normal(uint64_t seed) : g_(seed) {}
  double uniform01_open_left() {   // (0, 1]
    return (double)((g_() >> 11) + 1) * (1.0 / 9007199254740992.0);
  }
  double uniform01() {             // [0, 1)
    return (double)(g_() >> 11) * (1.0 / 9007199254740992.0);
  }
  double next() {
    if (has_spare_) { has_spare_ = false; return spare_; }
    const double u1 = uniform01_open_left();
    const double u2 = uniform01();
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double t = 6.283185307179586476925286766559 * u2;
    spare_ = r * std::sin(t);
    has_spare_ = true;
    return r * std::cos(t);
  }
  uint64_t raw() { return g_(); }

 private:
  std::mt19937_64 g_;
  bool has_spare_ = false;
  double spare_ = 0.0;
};

// ---------------------------------------------------------------------------
// Block structure
// ---------------------------------------------------------------------------
inline Leg make_u1_leg(int qlo, const std::vector<int64_t>& dims, int dir) {
  Leg l;
  l.dir = dir;
  l.ncomp = 1;
  l.dims = dims;
  for (size_t i = 0; i < dims.size(); ++i) l.qns.push_back(qlo + (int)i);
  return l;
}

// Enumerate every block whose divergence equals div (ncomp components), in row-major
// (= ascending block index) order, and lay out offsets.
inline Tensor make_tensor(const std::vector<Leg>& legs, const std::vector<int32_t>& div,
                          bool is_complex) {
  Tensor t;
  t.legs = legs;
  t.is_complex = is_complex;
  const int r = (int)legs.size();
  const int nc = legs.empty() ? 1 : legs[0].ncomp;
  std::vector<int64_t> c(r, 0);
  int64_t total = 1;
  for (auto& l : legs) total *= l.nsct();
  std::vector<int32_t> d(nc);
  for (int64_t lin = 0; lin < total; ++lin) {
    int64_t rem = lin;
    for (int i = r - 1; i >= 0; --i) { c[i] = rem % legs[i].nsct(); rem /= legs[i].nsct(); }
    std::fill(d.begin(), d.end(), 0);
    for (int i = 0; i < r; ++i) {
      for (int k = 0; k < nc; ++k) {
        int32_t q = legs[i].qns[c[i] * nc + k];
        d[k] += (legs[i].dir == DIR_OUT) ? q : -q;
      }
    }
    if (d == div) {
      t.coords.insert(t.coords.end(), c.begin(), c.end());
    }
  }
  t.offsets.resize(t.nblk());
  int64_t off = 0;
  for (int64_t b = 0; b < t.nblk(); ++b) { t.offsets[b] = off; off += t.blk_size(b); }
  t.size = off;
  t.data.assign(is_complex ? 2 * off : off, 0.0);
  return t;
}

inline void fill_normal(Tensor& t, Normal& rng) {
  for (auto& x : t.data) x = rng.next();
}

inline double frob_norm(const Tensor& t) {
  // Deterministic pairwise sum of squares.
  std::vector<double> v(t.data.size());
  for (size_t i = 0; i < v.size(); ++i) v[i] = t.data[i] * t.data[i];
  size_t n = v.size();
  while (n > 1) {
    size_t h = (n + 1) / 2;
    for (size_t i = 0; i + h < n; ++i) v[i] += v[i + h];
    n = h;
  }
  return n ? std::sqrt(v[0]) : 0.0;
}

inline void normalize(Tensor& t) {
  const double nrm = frob_norm(t);
  if (nrm > 0) for (auto& x : t.data) x /= nrm;
}

// Gaussian sector dims: w_q = exp(-q^2 / (2 sigma^2)), d_q = max(1, round(D w_q / sum w)),
// the q = 0 sector absorbs the rounding remainder so the dims sum to D exactly.
inline std::vector<int64_t> gauss_dims(int qmax, double sigma, int64_t D) {
  const int n = 2 * qmax + 1;
  std::vector<double> w(n);
  double s = 0;
  for (int i = 0; i < n; ++i) {
    const double q = i - qmax;
    w[i] = std::exp(-q * q / (2 * sigma * sigma));
    s += w[i];
  }
  std::vector<int64_t> d(n);
  int64_t tot = 0;
  for (int i = 0; i < n; ++i) {
    d[i] = std::max<int64_t>(1, (int64_t)std::llround(w[i] / s * (double)D));
    tot += d[i];
  }
  d[qmax] += D - tot;
  return d;
}

// ---------------------------------------------------------------------------
// Config 1: rank-3 U(1) tensors contracted over one leg (runs on a CPU in ms).
// ---------------------------------------------------------------------------
struct Pair { Tensor a, b; };

inline Pair config1(uint64_t seed = 0) {
  Leg l0 = make_u1_leg(-2, {4, 8, 12, 8, 4}, DIR_IN);
  Leg l1 = make_u1_leg(0, {1, 1}, DIR_IN);
  Leg l2 = make_u1_leg(-2, {4, 8, 12, 8, 4, 2}, DIR_OUT);
  Pair p;
  p.a = make_tensor({l0, l1, l2}, {0}, false);
  p.b = make_tensor({l2.inverse(), l1, l0.inverse()}, {0}, false);
  Normal rng(seed);
  fill_normal(p.a, rng);
  fill_normal(p.b, rng);
  return p;
}

// ---------------------------------------------------------------------------
// Two-site effective Hamiltonian operands.
//   psi  = (V IN, P IN, P IN, V OUT)     lenv = (V OUT, M IN, V IN)
//   mpo  = (M OUT, P OUT, P IN, M IN)    renv = (V IN, M OUT, V OUT)
// chain (reference tests/test_tensor_manipulation/test_ten_ctrct_1sct.cc:253-257):
//   t1 = lenv.psi {{0},{0}}; t2 = t1.mpo {{0,2},{0,1}}; t3 = t2.mpo {{4,1},{0,1}};
//   out = t3.renv {{4,1},{1,0}}
// ---------------------------------------------------------------------------
struct Matvec {
  Tensor lenv, psi, mpo1, mpo2, renv;
};

// U(1) spin-1/2 chain, random N(0,1) operands (Config 2 at D=2000, qmax 20, sigma 6;
// the D=4000 precision case at qmax 30, sigma 9).
inline Matvec heisenberg_u1_random(int qmax, double sigma, int64_t D, uint64_t seed) {
  auto dims = gauss_dims(qmax, sigma, D);
  Leg vin = make_u1_leg(-qmax, dims, DIR_IN);
  Leg pin = make_u1_leg(0, {1, 1}, DIR_IN);
  Leg min_ = make_u1_leg(-1, {1, 3, 1}, DIR_IN);
  Matvec m;
  m.psi = make_tensor({vin, pin, pin, vin.inverse()}, {0}, false);
  m.lenv = make_tensor({vin.inverse(), min_, vin}, {0}, false);
  m.mpo1 = make_tensor({min_.inverse(), pin.inverse(), pin, min_}, {0}, false);
  m.renv = make_tensor({vin, min_.inverse(), vin.inverse()}, {0}, false);
  Normal rng(seed);
  fill_normal(m.psi, rng);
  normalize(m.psi);
  fill_normal(m.lenv, rng);
  fill_normal(m.mpo1, rng);
  fill_normal(m.renv, rng);
  m.mpo2 = m.mpo1;
  return m;
}

// Locate the block with the given sector coordinates (binary search over the
// ascending coordinate list). Returns -1 if absent.
inline int64_t find_block(const Tensor& t, const std::vector<int64_t>& c) {
  int64_t lo = 0, hi = t.nblk();
  const int r = t.rank();
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    bool less = std::lexicographical_compare(t.coords.begin() + mid * r,
                                             t.coords.begin() + mid * r + r, c.begin(), c.end());
    if (less) lo = mid + 1; else hi = mid;
  }
  if (lo < t.nblk() && std::equal(c.begin(), c.end(), t.coords.begin() + lo * r)) return lo;
  return -1;
}

// Symmetrise a rank-3 environment E(a, w, a') so that E(a, w, a') = E(a', wbar, a),
// where wbar swaps the q=-1 and q=+1 MPO channels and fixes the q=0 channels.
inline void symmetrize_env(Tensor& e) {
  std::vector<double> out(e.data.size());
  const auto& wleg = e.legs[1];
  for (int64_t b = 0; b < e.nblk(); ++b) {
    int64_t c0 = e.coords[b * 3], c1 = e.coords[b * 3 + 1], c2 = e.coords[b * 3 + 2];
    int64_t cbar = wleg.nsct() - 1 - c1;   // channel sectors are q = -1, 0, +1
    int64_t p = find_block(e, {c2, cbar, c0});
    if (p < 0) throw std::runtime_error("symmetrize_env: partner block missing");
    const int64_t d0 = e.blk_dim(b, 0), d1 = e.blk_dim(b, 1), d2 = e.blk_dim(b, 2);
    const double* x = e.data.data() + e.offsets[b];
    const double* y = e.data.data() + e.offsets[p];
    double* o = out.data() + e.offsets[b];
    for (int64_t i = 0; i < d0; ++i)
      for (int64_t w = 0; w < d1; ++w)
        for (int64_t j = 0; j < d2; ++j)
          o[(i * d1 + w) * d2 + j] = 0.5 * (x[(i * d1 + w) * d2 + j] + y[(j * d1 + w) * d0 + i]);
  }
  e.data.swap(out);
}

// Heisenberg MPO (J = 1) in the (M OUT wl, P OUT s_in, P IN s_out, M IN wr) layout.
// Channels: q=-1 sector {S+ placed}, q=0 sector {start, Sz placed, done}, q=+1 {S- placed};
// P charges {0: down, 1: up}. Entry = <s_out| op |s_in>.
inline void fill_heisenberg_mpo(Tensor& w) {
  std::fill(w.data.begin(), w.data.end(), 0.0);
  // channel (sector, degeneracy) ids
  struct Ch { int64_t sct, deg; };
  const Ch start{1, 0}, szc{1, 1}, done{1, 2}, spc{0, 0}, smc{2, 0};
  const int64_t f = w.is_complex ? 2 : 1;   // doubles per element (real part first)
  auto set = [&](Ch wl, int64_t s_in, int64_t s_out, Ch wr, double v) {
    int64_t b = find_block(w, {wl.sct, s_in, s_out, wr.sct});
    if (b < 0) throw std::runtime_error("heisenberg mpo: block missing");
    const int64_t d3 = w.blk_dim(b, 3);
    w.data[(w.offsets[b] + wl.deg * d3 + wr.deg) * f] = v;   // P dims are 1
  };
  for (int s = 0; s < 2; ++s) { set(start, s, s, start, 1.0); set(done, s, s, done, 1.0); }
  set(start, 0, 1, spc, 1.0);          // S+ |down> = |up>
  set(start, 1, 0, smc, 1.0);          // S- |up> = |down>
  set(start, 0, 0, szc, -0.5);
  set(start, 1, 1, szc, 0.5);
  set(spc, 1, 0, done, 0.5);           // (1/2) S- completes S+ S-
  set(smc, 0, 1, done, 0.5);           // (1/2) S+ completes S- S+
  set(szc, 0, 0, done, -0.5);
  set(szc, 1, 1, done, 0.5);
}

// D=4000 precision case with a real-symmetric effective Hamiltonian (for Lanczos):
// Heisenberg MPO on both sites, symmetrised random environments.
inline Matvec heisenberg_u1_hermitian(int qmax, double sigma, int64_t D, uint64_t seed) {
  Matvec m = heisenberg_u1_random(qmax, sigma, D, seed);
  symmetrize_env(m.lenv);
  symmetrize_env(m.renv);
  fill_heisenberg_mpo(m.mpo1);
  m.mpo2 = m.mpo1;
  return m;
}

// Complex form of symmetrize_env: E(a, w, a') = conj(E(a', wbar, a)) (data interleaved re, im).
inline void hermitize_env(Tensor& e) {
  std::vector<double> out(e.data.size());
  const auto& wleg = e.legs[1];
  for (int64_t b = 0; b < e.nblk(); ++b) {
    int64_t c0 = e.coords[b * 3], c1 = e.coords[b * 3 + 1], c2 = e.coords[b * 3 + 2];
    int64_t p = find_block(e, {c2, wleg.nsct() - 1 - c1, c0});
    if (p < 0) throw std::runtime_error("hermitize_env: partner block missing");
    const int64_t d0 = e.blk_dim(b, 0), d1 = e.blk_dim(b, 1), d2 = e.blk_dim(b, 2);
    const double* x = e.data.data() + 2 * e.offsets[b];
    const double* y = e.data.data() + 2 * e.offsets[p];
    double* o = out.data() + 2 * e.offsets[b];
    for (int64_t i = 0; i < d0; ++i)
      for (int64_t w = 0; w < d1; ++w)
        for (int64_t j = 0; j < d2; ++j) {
          const int64_t u = (i * d1 + w) * d2 + j, v = (j * d1 + w) * d0 + i;
          o[2 * u] = 0.5 * (x[2 * u] + y[2 * v]);
          o[2 * u + 1] = 0.5 * (x[2 * u + 1] - y[2 * v + 1]);
        }
  }
  e.data.swap(out);
}

// Complex128 U(1) chain with a complex-Hermitian effective Hamiltonian (for the complex
// Lanczos): N(0,1)+iN(0,1) psi and environments, environments made Hermitian per MPO
// channel pair, the real Heisenberg MPO on both sites.
inline Matvec heisenberg_u1_hermitian_complex(int qmax, double sigma, int64_t D, uint64_t seed) {
  auto dims = gauss_dims(qmax, sigma, D);
  Leg vin = make_u1_leg(-qmax, dims, DIR_IN);
  Leg pin = make_u1_leg(0, {1, 1}, DIR_IN);
  Leg min_ = make_u1_leg(-1, {1, 3, 1}, DIR_IN);
  Matvec m;
  m.psi = make_tensor({vin, pin, pin, vin.inverse()}, {0}, true);
  m.lenv = make_tensor({vin.inverse(), min_, vin}, {0}, true);
  m.mpo1 = make_tensor({min_.inverse(), pin.inverse(), pin, min_}, {0}, true);
  m.renv = make_tensor({vin, min_.inverse(), vin.inverse()}, {0}, true);
  Normal rng(seed);
  fill_normal(m.psi, rng);
  normalize(m.psi);
  fill_normal(m.lenv, rng);
  fill_normal(m.renv, rng);
  hermitize_env(m.lenv);
  hermitize_env(m.renv);
  fill_heisenberg_mpo(m.mpo1);
  m.mpo2 = m.mpo1;
  return m;
}

// ---------------------------------------------------------------------------
// Config 5: spinful fermions, U(1)xU(1) (N, Sz), parity = N odd, complex128.
// ---------------------------------------------------------------------------
inline Leg make_u1u1_leg(const std::vector<std::pair<int, int>>& qn,
                         const std::vector<int64_t>& dims, int dir) {
  Leg l;
  l.dir = dir;
  l.ncomp = 2;
  l.parity_comp = 0;
  l.dims = dims;
  for (auto& q : qn) { l.qns.push_back(q.first); l.qns.push_back(q.second); }
  return l;
}

// Bond sectors (N, Sz) in [-half, half) x [-half, half); dims clip(round(D x / sum x), 1, 300)
// with x ~ LogNormal(3, 1); the largest sector absorbs the remainder so the dims sum to D.
inline Matvec hubbard_u1u1(int half, int64_t D, uint64_t seed) {
  Normal rng(seed);
  std::vector<std::pair<int, int>> vq;
  std::vector<double> x;
  for (int n = -half; n < half; ++n)
    for (int s = -half; s < half; ++s) {
      vq.push_back({n, s});
      x.push_back(std::exp(3.0 + 1.0 * rng.next()));
    }
  const double sx = std::accumulate(x.begin(), x.end(), 0.0);
  std::vector<int64_t> dims(x.size());
  int64_t tot = 0;
  for (size_t i = 0; i < x.size(); ++i) {
    dims[i] = std::min<int64_t>(300, std::max<int64_t>(1, (int64_t)std::llround(x[i] * (double)D / sx)));
    tot += dims[i];
  }
  // Distribute the remainder over the largest sectors without leaving [1, 300].
  std::vector<size_t> order(dims.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return dims[a] > dims[b]; });
  int64_t rem = D - tot;
  for (size_t k = 0; rem != 0 && k < order.size() * 300; ++k) {
    size_t i = order[k % order.size()];
    if (rem > 0 && dims[i] < 300) { int64_t t = std::min<int64_t>(rem, 300 - dims[i]); dims[i] += t; rem -= t; }
    else if (rem < 0 && dims[i] > 1) { int64_t t = std::min<int64_t>(-rem, dims[i] - 1); dims[i] -= t; rem += t; }
  }
  Leg vin = make_u1u1_leg(vq, dims, DIR_IN);
  Leg pin = make_u1u1_leg({{0, 0}, {1, 1}, {1, -1}, {2, 0}}, {1, 1, 1, 1}, DIR_IN);
  Leg min_ = make_u1u1_leg({{0, 0}, {1, 1}, {-1, -1}, {1, -1}, {-1, 1}}, {2, 1, 1, 1, 1}, DIR_IN);
  Matvec m;
  m.psi = make_tensor({vin, pin, pin, vin.inverse()}, {0, 0}, true);
  m.lenv = make_tensor({vin.inverse(), min_, vin}, {0, 0}, true);
  m.mpo1 = make_tensor({min_.inverse(), pin.inverse(), pin, min_}, {0, 0}, true);
  m.renv = make_tensor({vin, min_.inverse(), vin.inverse()}, {0, 0}, true);
  fill_normal(m.psi, rng);
  normalize(m.psi);
  fill_normal(m.lenv, rng);
  fill_normal(m.mpo1, rng);
  fill_normal(m.renv, rng);
  m.mpo2 = m.mpo1;
  return m;
}

// ---------------------------------------------------------------------------
// Block-matrix view for decompositions: blocks grouped by (left flux, right flux),
// group ids in order of first appearance over ascending blocks, row/col sectors in
// order of first appearance inside a group (the reference's GenIdxTenDecompDataBlkMats,
// tensor_manipulation/ten_decomp/ten_decomp_basic.h:68-106, and TenDecompDataBlkMat,
// qltensor/blk_spar_data_ten/data_blk_mat.h:39-131).
// ---------------------------------------------------------------------------
struct BlockMatrix {
  std::vector<int32_t> lflux;
  int64_t rows = 0, cols = 0;
  std::vector<std::vector<int64_t>> row_keys, col_keys;   // part coordinates
  std::vector<int64_t> row_off, row_dim, col_off, col_dim;
  std::vector<int64_t> elem_blk, elem_row, elem_col;       // tensor block -> (row sct, col sct)
};

inline std::vector<BlockMatrix> block_matrices(const Tensor& t, int ldims) {
  std::vector<BlockMatrix> mats;
  const int r = t.rank(), nc = t.ncomp();
  for (int64_t b = 0; b < t.nblk(); ++b) {
    std::vector<int32_t> lf(nc, 0);
    for (int i = 0; i < ldims; ++i)
      for (int k = 0; k < nc; ++k) {
        int32_t q = t.legs[i].qns[t.coords[b * r + i] * nc + k];
        lf[k] += (t.legs[i].dir == DIR_OUT) ? q : -q;
      }
    // right flux is determined by the left flux for a tensor of fixed divergence
    size_t g = 0;
    for (; g < mats.size(); ++g) if (mats[g].lflux == lf) break;
    if (g == mats.size()) { mats.emplace_back(); mats.back().lflux = lf; }
    auto& m = mats[g];
    std::vector<int64_t> lk(t.coords.begin() + b * r, t.coords.begin() + b * r + ldims);
    std::vector<int64_t> rk(t.coords.begin() + b * r + ldims, t.coords.begin() + b * r + r);
    int64_t rd = 1, cd = 1;
    for (int i = 0; i < ldims; ++i) rd *= t.blk_dim(b, i);
    for (int i = ldims; i < r; ++i) cd *= t.blk_dim(b, i);
    size_t i = 0;
    for (; i < m.row_keys.size(); ++i) if (m.row_keys[i] == lk) break;
    if (i == m.row_keys.size()) { m.row_keys.push_back(lk); m.row_off.push_back(m.rows); m.row_dim.push_back(rd); m.rows += rd; }
    size_t j = 0;
    for (; j < m.col_keys.size(); ++j) if (m.col_keys[j] == rk) break;
    if (j == m.col_keys.size()) { m.col_keys.push_back(rk); m.col_off.push_back(m.cols); m.col_dim.push_back(cd); m.cols += cd; }
    m.elem_blk.push_back(b); m.elem_row.push_back(i); m.elem_col.push_back(j);
  }
  return mats;
}

// Orthonormal columns (k of them) for an n x k matrix: two passes of modified
// Gram-Schmidt over N(0,1) columns. Row-major output [n * k].
inline std::vector<double> random_orthonormal(int64_t n, int64_t k, Normal& rng) {
  std::vector<double> q(n * k);
  for (auto& x : q) x = rng.next();
  for (int64_t j = 0; j < k; ++j) {
    for (int pass = 0; pass < 2; ++pass) {
      for (int64_t p = 0; p < j; ++p) {
        double dot = 0;
        for (int64_t i = 0; i < n; ++i) dot += q[i * k + p] * q[i * k + j];
        for (int64_t i = 0; i < n; ++i) q[i * k + j] -= dot * q[i * k + p];
      }
    }
    double nrm = 0;
    for (int64_t i = 0; i < n; ++i) nrm += q[i * k + j] * q[i * k + j];
    nrm = std::sqrt(nrm);
    for (int64_t i = 0; i < n; ++i) q[i * k + j] /= nrm;
  }
  return q;
}

// Fill a real tensor so that each block-matrix (ldims split) is Q1 diag(s_b) Q2^T with the
// global spectrum s_j = exp(-rate * j), j = 0 .. sum_b min(r_b, c_b) - 1, randomly
// partitioned across block-matrices and sorted descending inside each.
inline void fill_with_spectrum(Tensor& t, int ldims, double rate, uint64_t seed) {
  auto mats = block_matrices(t, ldims);
  Normal rng(seed);
  int64_t total = 0;
  for (auto& m : mats) total += std::min(m.rows, m.cols);
  std::vector<int64_t> perm(total);
  std::iota(perm.begin(), perm.end(), 0);
  for (int64_t i = total - 1; i > 0; --i) {     // Fisher-Yates with an explicit modulus
    int64_t j = (int64_t)(rng.raw() % (uint64_t)(i + 1));
    std::swap(perm[i], perm[j]);
  }
  int64_t pos = 0;
  std::fill(t.data.begin(), t.data.end(), 0.0);
  const int r = t.rank();
  for (auto& m : mats) {
    const int64_t k = std::min(m.rows, m.cols);
    std::vector<double> s(k);
    for (int64_t i = 0; i < k; ++i) s[i] = std::exp(-rate * (double)perm[pos + i]);
    pos += k;
    std::sort(s.begin(), s.end(), [](double a, double b) { return a > b; });
    auto q1 = random_orthonormal(m.rows, k, rng);
    auto q2 = random_orthonormal(m.cols, k, rng);
    std::vector<double> dense(m.rows * m.cols, 0.0);
    for (int64_t i = 0; i < m.rows; ++i)
      for (int64_t p = 0; p < k; ++p) {
        const double a = q1[i * k + p] * s[p];
        for (int64_t j = 0; j < m.cols; ++j) dense[i * m.cols + j] += a * q2[j * k + p];
      }
    for (size_t e = 0; e < m.elem_blk.size(); ++e) {
      const int64_t b = m.elem_blk[e];
      const int64_t ro = m.row_off[m.elem_row[e]], rd = m.row_dim[m.elem_row[e]];
      const int64_t co = m.col_off[m.elem_col[e]], cd = m.col_dim[m.elem_col[e]];
      double* dst = t.data.data() + t.offsets[b];
      for (int64_t i = 0; i < rd; ++i)
        for (int64_t j = 0; j < cd; ++j) dst[i * cd + j] = dense[(ro + i) * m.cols + co + j];
    }
    (void)r;
  }
}

// Config 3 on the two-site psi structure (ldims = 2).
inline Tensor svd_psi(int qmax, double sigma, int64_t D, uint64_t seed) {
  auto dims = gauss_dims(qmax, sigma, D);
  Leg vin = make_u1_leg(-qmax, dims, DIR_IN);
  Leg pin = make_u1_leg(0, {1, 1}, DIR_IN);
  Tensor psi = make_tensor({vin, pin, pin, vin.inverse()}, {0}, false);
  fill_with_spectrum(psi, 2, 0.01, seed);
  return psi;
}

// Stress variant: nb square blocks with sizes linearly spaced lo..hi on a rank-2 U(1)
// tensor (V IN, V OUT), same spectrum rule.
inline Tensor svd_stress(int nb, int64_t lo, int64_t hi, uint64_t seed) {
  std::vector<int64_t> dims(nb);
  for (int i = 0; i < nb; ++i)
    dims[i] = lo + (int64_t)std::llround((double)(hi - lo) * i / (double)std::max(1, nb - 1));
  Leg vin = make_u1_leg(0, dims, DIR_IN);
  Tensor t = make_tensor({vin, vin.inverse()}, {0}, false);
  fill_with_spectrum(t, 1, 0.01, seed);
  return t;
}

}  // namespace qltg_synth
