// Runs the reference implementation (header-only qlten, CPU path) on synthetic inputs
// from tensortoolkit_gb300/csrc/synth.h and writes inputs, task lists and results to a
// QTB1 file. Built only where the reference sources are present, by oracle/ref/Makefile;
// its outputs pin the CPU restatement (oracle/oracle.cc) and become the committed golden
// fixtures under tests/golden/. Test infrastructure only.
//
// Usage: ref_driver <case> <out.qtb> [args...]
//   cfg1                          Contract(A, B, {{2},{0}}) of the rank-3 U(1) case
//   matvec_u1 qmax sigma D seed   four-step two-site chain, U(1), FP64
//   matvec_f half D seed          four-step chain, fermionic U(1)xU(1), complex128
//   ctrct_misc seed               extra axis patterns incl. scalar results and IN-leg contractions
//   ctrct_contig seed             ContractContiguousAxes (all side pairs, wrapped and middle
//                                 ranges) and ContractTailHeadContiguousAccumulate /
//                                 TryContractTailHeadContiguousAccumulate (default, same,
//                                 expanded and superset outputs), U(1) real and fermionic complex
//   qlten_io seed dir             tensors written by the reference's QLTensor stream operator
//                                 (dir/<tag>.qlten) and dumped to <out>: U(1) real, fermionic
//                                 complex, a scalar, a tensor with no blocks
//   axis_ops seed                 qlten::dmrg axis primitives on a U(1) psi: ApplyAxisDiagonal
//                                 (out of place, accumulate), ApplyAxisSectorScalarsPreserveOrder,
//                                 ApplyRank2ToAxisPreserveOrder (boundary and middle axes),
//                                 ApplyTwoRank2ToAxesPreserveOrder
//   svd_u1 qmax sigma D seed trunc Dmin Dmax   SVD of a spectrum-controlled psi (ldims 2)
//   svd_stress nb lo hi seed trunc Dmin Dmax   SVD of a rank-2 block-diagonal tensor
//   svd_f half D seed trunc Dmin Dmax          SVD of a fermionic complex psi
//   qr_u1 qmax sigma D seed                     QR of psi (ldims 2)
//   qr_f half D seed                            QR of a fermionic complex psi
//   time_matvec_u1 qmax sigma D seed threads iters   wall time of the chain (no dump)
#include "qlten/qlten.h"
#include "qlten/tensor_manipulation/dmrg/axis_ops.h"
#include "synth.h"
#include "../qtb_io.h"

#include <array>
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

using namespace qlten;
using qlten::special_qn::U1QN;
using qlten::special_qn::fU1U1QN;
namespace sy = qltg_synth;

template <typename QNT> QNT make_qn(const int32_t* q);
template <> U1QN make_qn<U1QN>(const int32_t* q) { return U1QN(q[0]); }
template <> fU1U1QN make_qn<fU1U1QN>(const int32_t* q) { return fU1U1QN(q[0], q[1]); }

template <typename QNT> constexpr int qn_ncomp() { return std::is_same<QNT, U1QN>::value ? 1 : 2; }

template <typename QNT>
Index<QNT> to_index(const sy::Leg& l) {
  std::vector<QNSector<QNT>> s;
  for (int64_t i = 0; i < l.nsct(); ++i) s.emplace_back(make_qn<QNT>(&l.qns[i * l.ncomp]), (size_t)l.dims[i]);
  return Index<QNT>(s, l.dir == sy::DIR_IN ? TenIndexDirType::IN : TenIndexDirType::OUT);
}

template <typename ElemT, typename QNT>
QLTensor<ElemT, QNT> to_qlten(const sy::Tensor& t, const std::vector<int32_t>& div = {}) {
  IndexVec<QNT> idx;
  for (auto& l : t.legs) idx.push_back(to_index<QNT>(l));
  QLTensor<ElemT, QNT> q(idx);
  std::vector<int32_t> d(qn_ncomp<QNT>(), 0);
  for (size_t i = 0; i < div.size() && i < d.size(); ++i) d[i] = div[i];
  q.Fill(make_qn<QNT>(d.data()), ElemT(0));
  auto& bsdt = q.GetBlkSparDataTen();
  const auto& blks = bsdt.GetBlkIdxDataBlkMap();
  if ((int64_t)blks.size() != t.nblk()) throw std::runtime_error("block count mismatch");
  int64_t b = 0;
  for (auto& kv : blks) {
    if ((int64_t)kv.second.data_offset != t.offsets[b]) throw std::runtime_error("offset mismatch");
    for (int i = 0; i < t.rank(); ++i)
      if ((int64_t)kv.second.blk_coors[i] != t.coords[b * t.rank() + i]) throw std::runtime_error("coords mismatch");
    ++b;
  }
  if ((int64_t)bsdt.GetActualRawDataSize() != t.size) throw std::runtime_error("size mismatch");
  std::memcpy(bsdt.GetActualRawDataPtr(), t.data.data(), t.data.size() * sizeof(double));
  return q;
}

template <typename ElemT, typename QNT>
void dump(qtb::Writer& w, const std::string& name, const QLTensor<ElemT, QNT>& t) {
  const auto& idxs = t.GetIndexes();
  std::vector<int32_t> dirs, nsct, qns;
  std::vector<int64_t> dims;
  for (auto& ix : idxs) {
    dirs.push_back(ix.GetDir() == TenIndexDirType::IN ? sy::DIR_IN : sy::DIR_OUT);
    nsct.push_back((int32_t)ix.GetQNSctNum());
    for (auto& s : ix.GetQNScts()) {
      for (int k = 0; k < qn_ncomp<QNT>(); ++k) qns.push_back(s.GetQn().GetQNVal(k).GetVal());
      dims.push_back((int64_t)s.GetDegeneracy());
    }
  }
  w.i32(name + ".dirs", dirs);
  w.i32(name + ".nsct", nsct);
  w.i32(name + ".qns", qns);
  w.i64(name + ".dims", dims);
  w.scalar_i64(name + ".ncomp", qn_ncomp<QNT>());
  const auto& bsdt = t.GetBlkSparDataTen();
  std::vector<int64_t> coords, offsets;
  for (auto& kv : bsdt.GetBlkIdxDataBlkMap()) {
    for (auto c : kv.second.blk_coors) coords.push_back((int64_t)c);
    offsets.push_back((int64_t)kv.second.data_offset);
  }
  w.i64(name + ".coords", coords);
  w.i64(name + ".offsets", offsets);
  size_t n = bsdt.GetActualRawDataSize();
  if (t.IsScalar() && n == 0) n = 0;
  const double* p = reinterpret_cast<const double*>(bsdt.GetActualRawDataPtr());
  const size_t per = std::is_same<ElemT, double>::value ? 1 : 2;
  std::vector<double> data(p ? p : nullptr, p ? p + n * per : nullptr);
  w.f64(name + ".data", data);
}

// The task list the reference would execute: DataBlkGenForTenCtrct then
// SortTasksByCBlkIdx, as TensorContractionExecutor and CtrctTwoBSDTAndAssignIn do
// (tensor_manipulation/ten_ctrct.h:177-235; global_operations.h:895-992).
template <typename ElemT, typename QNT>
void dump_tasks(qtb::Writer& w, const std::string& name, const QLTensor<ElemT, QNT>& a,
                const QLTensor<ElemT, QNT>& b, const std::vector<std::vector<size_t>>& axes) {
  auto saved = TenCtrctGenSavedAxesSet(a.Rank(), b.Rank(), axes);
  QLTensor<ElemT, QNT> c;
  TenCtrctInitResTen(&a, &b, saved, &c);
  auto tasks = c.GetBlkSparDataTen().DataBlkGenForTenCtrct(a.GetBlkSparDataTen(), b.GetBlkSparDataTen(), axes, saved);
  std::vector<int64_t> gen;   // generation order (a_blk, b_blk, c_blk, m, k, n, sign, beta)
  for (auto& t : tasks) {
    gen.insert(gen.end(), {(int64_t)t.a_blk_idx, (int64_t)t.b_blk_idx, (int64_t)t.c_blk_idx, (int64_t)t.m,
                           (int64_t)t.k, (int64_t)t.n, (int64_t)t.f_ex_sign, (int64_t)t.beta});
  }
  w.put(name + ".tasks", 1, {tasks.size(), 8}, gen.data(), 8);
}

template <typename ElemT, typename QNT>
void contract_case(qtb::Writer& w, const std::string& tag, const QLTensor<ElemT, QNT>& a,
                   const QLTensor<ElemT, QNT>& b, const std::vector<std::vector<size_t>>& axes,
                   QLTensor<ElemT, QNT>* out = nullptr) {
  std::vector<int64_t> ax;
  for (auto x : axes[0]) ax.push_back((int64_t)x);
  for (auto x : axes[1]) ax.push_back((int64_t)x);
  w.i64(tag + ".axes", ax);
  dump(w, tag + ".A", a);
  dump(w, tag + ".B", b);
  dump_tasks(w, tag, a, b, axes);
  QLTensor<ElemT, QNT> c;
  Contract(&a, &b, axes, &c);
  dump(w, tag + ".C", c);
  if (out) *out = c;
}

static sy::Tensor random_like(const std::vector<sy::Leg>& legs, const std::vector<int32_t>& div, bool cplx,
                              sy::Normal& rng) {
  auto t = sy::make_tensor(legs, div, cplx);
  sy::fill_normal(t, rng);
  return t;
}

// ContractContiguousAxes<ASide, BSide> (tensor_manipulation/contract_contiguous_axes.h:849-868)
template <typename ElemT, typename QNT, CtrctSide SA, CtrctSide SB>
QLTensor<ElemT, QNT> contig(const QLTensor<ElemT, QNT>& a, const QLTensor<ElemT, QNT>& b, size_t a0, size_t b0,
                            size_t n) {
  QLTensor<ElemT, QNT> c;
  ContractContiguousAxes<ElemT, QNT, SA, SB>(a, b, a0, b0, n, c);
  return c;
}

template <typename ElemT, typename QNT>
void contig_case(qtb::Writer& w, const std::string& tag, const QLTensor<ElemT, QNT>& a,
                 const QLTensor<ElemT, QNT>& b, size_t a0, size_t b0, size_t n, bool a_tail, bool b_head) {
  w.i64(tag + ".params", {(int64_t)a0, (int64_t)b0, (int64_t)n, a_tail ? 1 : 0, b_head ? 1 : 0});
  dump(w, tag + ".A", a);
  dump(w, tag + ".B", b);
  QLTensor<ElemT, QNT> c;
  using S = CtrctSide;
  if (a_tail && b_head) c = contig<ElemT, QNT, S::Tail, S::Head>(a, b, a0, b0, n);
  else if (a_tail) c = contig<ElemT, QNT, S::Tail, S::Tail>(a, b, a0, b0, n);
  else if (b_head) c = contig<ElemT, QNT, S::Head, S::Head>(a, b, a0, b0, n);
  else c = contig<ElemT, QNT, S::Head, S::Tail>(a, b, a0, b0, n);
  dump(w, tag + ".C", c);
}

template <typename ElemT> std::vector<double> re_im(ElemT x);
template <> std::vector<double> re_im<double>(double x) { return {x, 0.0}; }
template <> std::vector<double> re_im<std::complex<double>>(std::complex<double> x) { return {x.real(), x.imag()}; }

// ContractTailHeadContiguousAccumulate / TryContractTailHeadContiguousAccumulate
// (tensor_manipulation/contract_contiguous_axes.h:953-1040). c0 == nullptr: default output.
template <typename ElemT, typename QNT>
void accum_case(qtb::Writer& w, const std::string& tag, const QLTensor<ElemT, QNT>& a,
                const QLTensor<ElemT, QNT>& b, size_t a0, size_t b0, size_t n, ElemT alpha, ElemT beta,
                const QLTensor<ElemT, QNT>* c0, bool try_only, QLTensor<ElemT, QNT>* out = nullptr) {
  w.i64(tag + ".params", {(int64_t)a0, (int64_t)b0, (int64_t)n, 1, 1});
  w.f64(tag + ".alpha", re_im(alpha));
  w.f64(tag + ".beta", re_im(beta));
  dump(w, tag + ".A", a);
  dump(w, tag + ".B", b);
  QLTensor<ElemT, QNT> c;
  if (c0) {
    dump(w, tag + ".C0", *c0);
    c = *c0;
  }
  if (try_only) {
    const bool ok = TryContractTailHeadContiguousAccumulate(a, b, a0, b0, n, alpha, beta, c);
    w.scalar_i64(tag + ".ok", ok ? 1 : 0);
  } else {
    ContractTailHeadContiguousAccumulate(a, b, a0, b0, n, alpha, beta, c);
  }
  dump(w, tag + ".C", c);
  if (out) *out = c;
}

template <typename ElemT, typename QNT>
void contig_suite(qtb::Writer& w, const std::string& pre, const sy::Matvec& mv, const std::vector<int32_t>& div0,
                  const std::vector<int32_t>& div1, ElemT alpha, ElemT beta, sy::Normal& rng) {
  const bool cplx = !std::is_same<ElemT, double>::value;
  auto P = to_qlten<ElemT, QNT>(mv.psi);
  auto L = to_qlten<ElemT, QNT>(mv.lenv);
  std::vector<sy::Leg> inv;
  for (auto& l : mv.psi.legs) inv.push_back(l.inverse());
  auto Pd = to_qlten<ElemT, QNT>(random_like(inv, div0, cplx, rng));
  const auto& pl = mv.psi.legs;
  auto Q = to_qlten<ElemT, QNT>(random_like({pl[2].inverse(), pl[3].inverse(), pl[0].inverse(), pl[1].inverse()},
                                            div0, cplx, rng));
  contig_case(w, pre + "hh", L, P, 0, 0, 1, false, true);     // lenv leg 0 . psi leg 0
  contig_case(w, pre + "wrap", P, Pd, 3, 3, 2, true, true);   // axes {3, 0} . {3, 0}
  contig_case(w, pre + "mid", P, Pd, 1, 1, 2, true, true);    // axes {1, 2}: saved order 3, 0
  contig_case(w, pre + "tt", P, Pd, 2, 2, 2, true, false);
  contig_case(w, pre + "ht", P, Q, 0, 2, 2, false, false);
  // accumulate: A = lenv with its legs rotated (last leg = inverse of psi leg 0), tail . head
  const auto& ll = mv.lenv.legs;
  auto A1 = to_qlten<ElemT, QNT>(random_like({ll[1], ll[2], ll[0]}, div0, cplx, rng));
  auto A2 = to_qlten<ElemT, QNT>(random_like({ll[1], ll[2], ll[0]}, div0, cplx, rng));
  std::vector<sy::Leg> cl = {ll[1], ll[2], pl[1], pl[2], pl[3]};
  auto Csame = contig<ElemT, QNT, CtrctSide::Tail, CtrctSide::Head>(A2, P, 2, 0, 1);
  auto Cother = to_qlten<ElemT, QNT>(random_like(cl, div1, cplx, rng), div1);
  accum_case(w, pre + "acc_default", A1, P, 2, 0, 1, alpha, ElemT(0), (const QLTensor<ElemT, QNT>*)nullptr, false);
  accum_case(w, pre + "acc_same", A1, P, 2, 0, 1, alpha, beta, &Csame, false);
  QLTensor<ElemT, QNT> Cunion;
  accum_case(w, pre + "acc_expand", A1, P, 2, 0, 1, alpha, beta, &Cother, false, &Cunion);
  accum_case(w, pre + "acc_superset", A2, P, 2, 0, 1, beta, alpha, &Cunion, false);
  accum_case(w, pre + "try_fail", A1, P, 2, 0, 1, alpha, beta, &Cother, true);
  accum_case(w, pre + "try_ok", A2, P, 2, 0, 1, alpha, beta, &Cunion, true);
}

template <typename ElemT, typename QNT>
void matvec_case(qtb::Writer& w, const sy::Matvec& mv) {
  auto L = to_qlten<ElemT, QNT>(mv.lenv);
  auto P = to_qlten<ElemT, QNT>(mv.psi);
  auto W1 = to_qlten<ElemT, QNT>(mv.mpo1);
  auto W2 = to_qlten<ElemT, QNT>(mv.mpo2);
  auto R = to_qlten<ElemT, QNT>(mv.renv);
  QLTensor<ElemT, QNT> t1, t2, t3, out;
  contract_case(w, "s1", L, P, {{0}, {0}}, &t1);
  contract_case(w, "s2", t1, W1, {{0, 2}, {0, 1}}, &t2);
  contract_case(w, "s3", t2, W2, {{4, 1}, {0, 1}}, &t3);
  contract_case(w, "s4", t3, R, {{4, 1}, {1, 0}}, &out);
}

template <typename ElemT, typename QNT>
void svd_case(qtb::Writer& w, const sy::Tensor& st, size_t ldims, double trunc, size_t dmin, size_t dmax) {
  auto t = to_qlten<ElemT, QNT>(st);
  dump(w, "T", t);
  std::vector<int32_t> zero(qn_ncomp<QNT>(), 0);
  QLTensor<ElemT, QNT> u, vt;
  QLTensor<QLTEN_Double, QNT> s;
  double err = 0;
  size_t D = 0;
  SVD(&t, ldims, make_qn<QNT>(zero.data()), trunc, dmin, dmax, &u, &s, &vt, &err, &D);
  dump(w, "U", u);
  dump(w, "S", s);
  dump(w, "Vt", vt);
  w.scalar_f64("err", err);
  w.scalar_i64("D", (int64_t)D);
  w.scalar_i64("ldims", (int64_t)ldims);
  w.scalar_f64("trunc", trunc);
  w.scalar_i64("Dmin", (int64_t)dmin);
  w.scalar_i64("Dmax", (int64_t)dmax);
}

template <typename ElemT, typename QNT>
void qr_case(qtb::Writer& w, const sy::Tensor& st, size_t ldims) {
  auto t = to_qlten<ElemT, QNT>(st);
  dump(w, "T", t);
  std::vector<int32_t> zero(qn_ncomp<QNT>(), 0);
  QLTensor<ElemT, QNT> q, r;
  QR(&t, ldims, make_qn<QNT>(zero.data()), &q, &r);
  dump(w, "Q", q);
  dump(w, "R", r);
  w.scalar_i64("ldims", (int64_t)ldims);
}

int main(int argc, char** argv) {
  if (argc < 3) { std::fprintf(stderr, "usage: ref_driver <case> <out> [args]\n"); return 2; }
  std::string cs = argv[1];
  auto A = [&](int i) { return std::string(argv[i]); };
  try {
    if (cs == "time_matvec_u1") {
      auto mv = sy::heisenberg_u1_random(std::stoi(A(2)), std::stod(A(3)), std::stoll(A(4)), std::stoull(A(5)));
      hp_numeric::SetTensorManipulationThreads(std::stoi(A(6)));
      int iters = std::stoi(A(7));
      auto L = to_qlten<double, U1QN>(mv.lenv);
      auto P = to_qlten<double, U1QN>(mv.psi);
      auto W = to_qlten<double, U1QN>(mv.mpo1);
      auto R = to_qlten<double, U1QN>(mv.renv);
      for (int it = 0; it < iters; ++it) {
        auto t0 = std::chrono::steady_clock::now();
        QLTensor<double, U1QN> t1, t2, t3, out;
        Contract(&L, &P, {{0}, {0}}, &t1);
        Contract(&t1, &W, {{0, 2}, {0, 1}}, &t2);
        Contract(&t2, &W, {{4, 1}, {0, 1}}, &t3);
        Contract(&t3, &R, {{4, 1}, {1, 0}}, &out);
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("iter %d %.6f s\n", it, dt);
      }
      return 0;
    }
    qtb::Writer w(argv[2]);
    if (cs == "cfg1") {
      auto p = sy::config1(0);
      contract_case(w, "c", to_qlten<double, U1QN>(p.a), to_qlten<double, U1QN>(p.b), {{2}, {0}});
    } else if (cs == "matvec_u1") {
      auto mv = sy::heisenberg_u1_random(std::stoi(A(3)), std::stod(A(4)), std::stoll(A(5)), std::stoull(A(6)));
      matvec_case<double, U1QN>(w, mv);
    } else if (cs == "matvec_u1h") {
      auto mv = sy::heisenberg_u1_hermitian(std::stoi(A(3)), std::stod(A(4)), std::stoll(A(5)), std::stoull(A(6)));
      matvec_case<double, U1QN>(w, mv);
    } else if (cs == "matvec_f") {
      auto mv = sy::hubbard_u1u1(std::stoi(A(3)), std::stoll(A(4)), std::stoull(A(5)));
      matvec_case<std::complex<double>, fU1U1QN>(w, mv);
    } else if (cs == "ctrct_misc") {
      sy::Normal rng(std::stoull(A(3)));
      // U(1): scalar result (full contraction), two-leg contraction with transposed B,
      // contraction over a middle leg.
      auto mv = sy::heisenberg_u1_random(3, 1.5, 20, std::stoull(A(3)));
      auto P = to_qlten<double, U1QN>(mv.psi);
      std::vector<sy::Leg> inv;
      for (auto& l : mv.psi.legs) inv.push_back(l.inverse());
      auto Pd = to_qlten<double, U1QN>(random_like(inv, {0}, false, rng));
      contract_case(w, "u_scalar", P, Pd, {{0, 1, 2, 3}, {0, 1, 2, 3}});
      contract_case(w, "u_perm", P, Pd, {{3, 1}, {3, 1}});
      auto L = to_qlten<double, U1QN>(mv.lenv);
      contract_case(w, "u_mid", L, P, {{2}, {3}});
      // Fermionic U(1)xU(1) complex: IN-direction contracted legs, several axis orders.
      auto fm = sy::hubbard_u1u1(1, 6, std::stoull(A(3)));
      auto FP = to_qlten<std::complex<double>, fU1U1QN>(fm.psi);
      std::vector<sy::Leg> finv;
      for (auto& l : fm.psi.legs) finv.push_back(l.inverse());
      auto FPd = to_qlten<std::complex<double>, fU1U1QN>(random_like(finv, {0, 0}, true, rng));
      contract_case(w, "f_scalar", FP, FPd, {{0, 1, 2, 3}, {0, 1, 2, 3}});
      contract_case(w, "f_in", FP, FPd, {{0, 2}, {0, 2}});
      contract_case(w, "f_rev", FP, FPd, {{3, 1, 0}, {3, 1, 0}});
      auto FL = to_qlten<std::complex<double>, fU1U1QN>(fm.lenv);
      auto FW = to_qlten<std::complex<double>, fU1U1QN>(fm.mpo1);
      contract_case(w, "f_env", FP, FL, {{0}, {0}});   // IN leg of A against OUT leg of B
      contract_case(w, "f_mpo", FW, FW, {{3}, {0}});
    } else if (cs == "ctrct_contig") {
      sy::Normal rng(std::stoull(A(3)));
      auto mv = sy::heisenberg_u1_random(3, 1.5, 20, std::stoull(A(3)));
      contig_suite<double, U1QN>(w, "u_", mv, {0}, {1}, 2.0, -1.5, rng);
      auto fm = sy::hubbard_u1u1(1, 6, std::stoull(A(3)));
      contig_suite<std::complex<double>, fU1U1QN>(w, "f_", fm, {0, 0}, {2, 0}, std::complex<double>(0.5, 0.25),
                                                  std::complex<double>(-1.0, 0.5), rng);
    } else if (cs == "qlten_io") {
      // QLTensor::StreamWrite (qltensor/qltensor_impl.h:825-830) through operator<<
      const std::string dir = A(4);
      auto save = [&](const std::string& tag, const auto& t) {
        std::ofstream ofs(dir + "/" + tag + ".qlten", std::ios::binary);
        ofs << t;
        dump(w, tag, t);
      };
      auto mv = sy::heisenberg_u1_random(2, 1.0, 8, std::stoull(A(3)));
      save("u_psi", to_qlten<double, U1QN>(mv.psi));
      save("u_lenv", to_qlten<double, U1QN>(mv.lenv));
      auto fm = sy::hubbard_u1u1(1, 4, std::stoull(A(3)));
      save("f_psi", to_qlten<std::complex<double>, fU1U1QN>(fm.psi));
      auto P = to_qlten<double, U1QN>(mv.psi);
      QLTensor<double, U1QN> sc;
      Contract(&P, &P, {{0, 1, 2, 3}, {0, 1, 2, 3}}, &sc);   // not a valid pairing: an empty scalar
      std::vector<sy::Leg> inv;
      for (auto& l : mv.psi.legs) inv.push_back(l.inverse());
      sy::Normal rng(std::stoull(A(3)));
      auto Pd = to_qlten<double, U1QN>(random_like(inv, {0}, false, rng));
      QLTensor<double, U1QN> sc2;
      Contract(&P, &Pd, {{0, 1, 2, 3}, {0, 1, 2, 3}}, &sc2);
      save("u_scalar", sc2);
    } else if (cs == "axis_ops") {
      using T = QLTensor<double, U1QN>;
      sy::Normal rng(std::stoull(A(3)));
      auto mv = sy::heisenberg_u1_random(2, 1.0, 10, std::stoull(A(3)));
      const auto& pl = mv.psi.legs;
      T P = to_qlten<double, U1QN>(mv.psi);
      dump(w, "psi", P);
      // diagonal values per (sector, degeneracy) of an axis
      auto diag_op = [&](size_t axis) {
        dmrg::AxisDiagonalOp<double, U1QN> op{P.GetIndex(axis), {}};
        for (auto& sct : op.index.GetQNScts()) {
          std::vector<double> v(sct.GetDegeneracy());
          for (auto& x : v) x = rng.next();
          op.values.push_back(v);
        }
        std::vector<double> flat;
        for (auto& v : op.values) flat.insert(flat.end(), v.begin(), v.end());
        return std::make_pair(op, flat);
      };
      for (size_t axis : {1u, 3u}) {
        auto [op, flat] = diag_op(axis);
        const std::string tag = "diag" + std::to_string(axis);
        w.f64(tag + ".values", flat);
        T out;
        dmrg::ApplyAxisDiagonal(P, axis, op, out, 1.5, 0.0);
        dump(w, tag + ".out", out);
        T acc = out;                         // accumulate: acc = 0.5 acc - 2 D(P)
        dmrg::ApplyAxisDiagonal(P, axis, op, acc, -2.0, 0.5);
        dump(w, tag + ".acc", acc);
      }
      {
        dmrg::AxisSectorScalar<double, U1QN> sc{0, {}};
        for (size_t s2 = 0; s2 < P.GetIndex(0).GetQNSctNum(); ++s2) sc.values_by_sector.push_back(rng.next());
        w.f64("sect.values", sc.values_by_sector);
        T out;
        dmrg::ApplyAxisSectorScalarsPreserveOrder(P, sc, out, dmrg::AxisApplyStorageMode::kOutOfPlace);
        dump(w, "sect.out", out);
      }
      // rank-2 operators {InverseIndex(axis leg), new leg}: the new leg keeps the charges with
      // other degeneracies
      auto rank2 = [&](size_t axis, int64_t grow) {
        sy::Leg in = pl[axis];
        sy::Leg nl = in;
        for (auto& d : nl.dims) d = std::max<int64_t>(1, d + grow);
        return to_qlten<double, U1QN>(random_like({in.inverse(), nl}, {0}, false, rng));
      };
      for (size_t axis : {0u, 2u, 3u}) {
        T op = rank2(axis, axis == 2 ? 1 : -1);
        const std::string tag = "r2_" + std::to_string(axis);
        dump(w, tag + ".op", op);
        T out;
        dmrg::ApplyRank2ToAxisPreserveOrder(P, op, axis, out);
        dump(w, tag + ".out", out);
      }
      // monomial operators: a raising map on the physical leg (flux +1) and a permuting,
      // accumulating map inside the sectors of the right bond leg (flux 0)
      auto monomial = [&](const std::string& tag, size_t axis, int flux,
                          const std::vector<std::array<size_t, 4>>& ent, const std::vector<double>& coefs) {
        dmrg::AxisMonomialOp<double, U1QN> op{P.GetIndex(axis), P.GetIndex(axis), U1QN(flux), {}};
        std::vector<int64_t> flat;
        for (size_t i = 0; i < ent.size(); ++i) {
          op.entries.push_back({ent[i][0], ent[i][1], ent[i][2], ent[i][3], coefs[i]});
          flat.insert(flat.end(), {(int64_t)ent[i][0], (int64_t)ent[i][1], (int64_t)ent[i][2], (int64_t)ent[i][3]});
        }
        w.i64(tag + ".entries", flat);
        w.f64(tag + ".coefs", coefs);
        w.i64(tag + ".params", {(int64_t)axis, flux});
        T out;
        dmrg::ApplyAxisMonomial(P, axis, op, out, 1.25, 0.0);
        dump(w, tag + ".out", out);
        dmrg::ApplyAxisMonomial(P, axis, op, out, -0.5, 2.0);   // accumulate onto it
        dump(w, tag + ".acc", out);
      };
      monomial("mono_p", 1, 1, {{0, 0, 1, 0}}, {1.0});
      monomial("mono_b", 3, 0, {{2, 0, 2, 3}, {2, 3, 2, 0}, {2, 1, 2, 1}, {2, 1, 2, 3}, {1, 0, 1, 1}, {3, 1, 3, 0}},
               {0.5, -1.0, 2.0, 0.25, 1.5, -0.75});
      {
        T op1 = rank2(0, 1), op2 = rank2(3, -1);
        dump(w, "two.op1", op1);
        dump(w, "two.op2", op2);
        T out;
        dmrg::ApplyTwoRank2ToAxesPreserveOrder(P, op1, 0, op2, 3, out);
        dump(w, "two.out", out);
      }
      auto scalars = [&](size_t axis) {
        dmrg::AxisSectorScalar<double, U1QN> sc{axis, {}};
        for (size_t s2 = 0; s2 < P.GetIndex(axis).GetQNSctNum(); ++s2) sc.values_by_sector.push_back(rng.next());
        return sc;
      };
      // a rank-2 operator restricted to the diagonal sector blocks listed in `keep`
      auto partial = [&](const T& op, const std::vector<size_t>& keep) {
        T o(op.GetIndexes());
        const auto& i0 = op.GetIndex(0);
        const auto& i1 = op.GetIndex(1);
        size_t b0 = 0, b1 = 0;
        for (size_t s2 = 0; s2 < i0.GetQNSctNum(); ++s2) {
          const size_t d0 = i0.GetQNSct(s2).GetDegeneracy(), d1 = i1.GetQNSct(s2).GetDegeneracy();
          if (std::find(keep.begin(), keep.end(), s2) != keep.end())
            for (size_t a = 0; a < d0; ++a)
              for (size_t b = 0; b < d1; ++b) o.SetElem({b0 + a, b1 + b}, op.GetElem({b0 + a, b1 + b}));
          b0 += d0;
          b1 += d1;
        }
        return o;
      };
      // projector on the right bond leg: sector 0 dropped, sector 1 keeps {0}, sector 2 keeps
      // {3, 1} (reordered), the others keep everything
      {
        const auto& ix = P.GetIndex(3);
        dmrg::AxisProjector<U1QN> pr{ix, {}};
        std::vector<int64_t> counts, flat;
        for (size_t s2 = 0; s2 < ix.GetQNSctNum(); ++s2) {
          std::vector<size_t> k;
          const size_t d = ix.GetQNSct(s2).GetDegeneracy();
          if (s2 == 1) k = {0};
          else if (s2 == 2 && d > 3) k = {3, 1};
          else if (s2 != 0) for (size_t j = 0; j < d; ++j) k.push_back(j);
          counts.push_back((int64_t)k.size());
          for (auto x : k) flat.push_back((int64_t)x);
          pr.kept_degeneracies.push_back(k);
        }
        w.i64("proj.counts", counts);
        w.i64("proj.kept", flat);
        T out;
        dmrg::ProjectAxis(P, 3, pr, out);
        dump(w, "proj.out", out);
      }
      {
        T op = rank2(0, -1);
        auto [dg, flat] = diag_op(3);
        dump(w, "r2diag.op", op);
        w.f64("r2diag.values", flat);
        T out;
        dmrg::ApplyRank2ThenAxisDiagonalPreserveOrder(P, op, 0, 3, dg, out);
        dump(w, "r2diag.out", out);
      }
      {
        T op = rank2(3, 1);
        auto sc = scalars(0);
        dump(w, "r2sect.op", op);
        w.f64("r2sect.values", sc.values_by_sector);
        T out;
        dmrg::ApplyRank2ThenAxisSectorScalarsPreserveOrder(P, op, 3, sc, out);
        dump(w, "r2sect.out", out);
      }
      // boundary rank-2 then sector scalars: fused (fresh output), accumulated onto it, and
      // accumulated onto an output lacking blocks (expansion); then the last-axis form
      {
        T op = rank2(0, -1);
        T opp = partial(op, {1, 2});
        auto sc = scalars(3);
        dump(w, "bnd.op", op);
        dump(w, "bnd.opp", opp);
        w.f64("bnd.values", sc.values_by_sector);
        T fused;
        dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder(P, op, 0, sc, fused);
        dump(w, "bnd.fused", fused);
        T acc = fused;
        dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder(P, op, 0, sc, -0.5, 2.0, acc);
        dump(w, "bnd.acc", acc);
        T part;
        dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder(P, opp, 0, sc, part);
        dump(w, "bnd.part", part);
        dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder(P, op, 0, sc, 1.25, 0.75, part);
        dump(w, "bnd.exp", part);
        T op3 = rank2(3, 1);
        auto sc0 = scalars(0);
        dump(w, "bnd.op3", op3);
        w.f64("bnd.values0", sc0.values_by_sector);
        T last;
        dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder(P, op3, 3, sc0, last);
        dump(w, "bnd.last", last);
      }
      {
        T op = rank2(0, -1);
        dmrg::AxisMonomialOp<double, U1QN> mo{P.GetIndex(3), P.GetIndex(3), U1QN(0), {}};
        const std::vector<std::array<size_t, 4>> ent = {{2, 0, 2, 3}, {2, 3, 2, 0}, {2, 1, 2, 1},
                                                        {2, 1, 2, 3}, {1, 0, 1, 1}, {3, 1, 3, 0}};
        const std::vector<double> cf = {0.5, -1.0, 2.0, 0.25, 1.5, -0.75};
        for (size_t i = 0; i < ent.size(); ++i)
          mo.entries.push_back({ent[i][0], ent[i][1], ent[i][2], ent[i][3], cf[i]});
        dump(w, "r2mono.op", op);
        T out;
        dmrg::ApplyRank2ThenAxisMonomialFusedPreserveOrder(P, op, 0, 3, mo, out);
        dump(w, "r2mono.out", out);
      }
      {
        T op1 = rank2(0, 1), op2 = rank2(3, -1);
        auto [dg, flat] = diag_op(1);
        auto sc = scalars(2);
        dump(w, "two2.op1", op1);
        dump(w, "two2.op2", op2);
        w.f64("two2.values", flat);
        w.f64("two2.scalars", sc.values_by_sector);
        T od, os;
        dmrg::ApplyTwoRank2ThenAxisDiagonalPreserveOrder(P, op1, 0, op2, 3, 1, dg, od);
        dump(w, "two2.diag", od);
        dmrg::ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder(P, op1, 0, op2, 3, sc, os);
        dump(w, "two2.sect", os);
      }
      {
        T out;
        dmrg::MoveHeadAxisToTail(P, out);
        dump(w, "move.out", out);
      }
      // LinearCombine over tensors with the same indexes and different block sets
      {
        T op = rank2(0, -1);
        T X, Y, Z;
        dmrg::ApplyRank2ToAxisPreserveOrder(P, partial(op, {0, 1, 2}), 0, X);
        dmrg::ApplyRank2ToAxisPreserveOrder(P, partial(op, {2, 3, 4}), 0, Y);
        dmrg::ApplyRank2ToAxisPreserveOrder(P, op, 0, Z);
        dump(w, "lc.X", X);
        dump(w, "lc.Y", Y);
        dump(w, "lc.Z", Z);
        T r1;
        LinearCombine<double, U1QN>({1.5, -2.0}, {&X, &Y}, 0.0, &r1);
        dump(w, "lc.r1", r1);
        T r2 = Z;
        LinearCombine<double, U1QN>({0.5, 0.0, 3.0}, {&X, &Y, &X}, 2.0, &r2);
        dump(w, "lc.r2", r2);
        T r3 = X;
        AddScaledAssign(r3, 0.25, Y);
        dump(w, "lc.r3", r3);
      }
    } else if (cs == "svd_u1") {
      auto t = sy::svd_psi(std::stoi(A(3)), std::stod(A(4)), std::stoll(A(5)), std::stoull(A(6)));
      svd_case<double, U1QN>(w, t, 2, std::stod(A(7)), std::stoull(A(8)), std::stoull(A(9)));
    } else if (cs == "svd_stress") {
      auto t = sy::svd_stress(std::stoi(A(3)), std::stoll(A(4)), std::stoll(A(5)), std::stoull(A(6)));
      svd_case<double, U1QN>(w, t, 1, std::stod(A(7)), std::stoull(A(8)), std::stoull(A(9)));
    } else if (cs == "svd_f") {
      auto mv = sy::hubbard_u1u1(std::stoi(A(3)), std::stoll(A(4)), std::stoull(A(5)));
      svd_case<std::complex<double>, fU1U1QN>(w, mv.psi, 2, std::stod(A(6)), std::stoull(A(7)), std::stoull(A(8)));
    } else if (cs == "qr_u1") {
      auto mv = sy::heisenberg_u1_random(std::stoi(A(3)), std::stod(A(4)), std::stoll(A(5)), std::stoull(A(6)));
      qr_case<double, U1QN>(w, mv.psi, 2);
    } else if (cs == "qr_f") {
      auto mv = sy::hubbard_u1u1(std::stoi(A(3)), std::stoll(A(4)), std::stoull(A(5)));
      qr_case<std::complex<double>, fU1U1QN>(w, mv.psi, 2);
    } else {
      std::fprintf(stderr, "unknown case %s\n", cs.c_str());
      return 2;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
