/*
 * qlten_gb300.h - drop-in GB300 backend for qlten's Contract / SVD / QR.
 *
 * Header-only C++17 glue that a qlten user (or a qlten maintainer) includes after
 * "qlten/qlten.h". It keeps the reference's signatures and QLTensor objects and routes the
 * arithmetic through the C ABI in qltg.h (libqltg.so):
 *
 *   qlten::Contract(&A, &B, axes, &C)        (tensor_manipulation/ten_ctrct.h:276-290)
 *     -> qlten_gb300::Contract(&A, &B, axes, &C, ctx [, mode])
 *   qlten::SVD(&T, ldims, lqndiv, eps, Dmin, Dmax, &U, &S, &Vt, &err, &D)  (ten_svd.h:244-263)
 *     -> qlten_gb300::SVD(..., ctx)
 *   qlten::QR(&T, ldims, lqndiv, &Q, &R)      (ten_decomp/ten_qr.h:152-162)
 *     -> qlten_gb300::QR(..., ctx)
 *   qlten::ContractContiguousAxes<..., ASide, BSide>(A, B, a0, b0, n, C)
 *     -> qlten_gb300::ContractContiguousAxes(A, B, a0, b0, n, C, ctx [, mode, a_side, b_side])
 *   qlten::ContractTailHeadContiguousAccumulate / TryContract...(A, B, a0, b0, n, alpha, beta, C)
 *     -> the same names with (..., C, ctx [, mode])  (contract_contiguous_axes.h:953-1040)
 *   qlten::LinearCombine(coefs, tens, beta, &res)   (ten_linear_combine.h:186-197)
 *     -> qlten_gb300::LinearCombine(coefs, tens, beta, &res, ctx)
 *
 * With the reference built for the GPU (USE_GPU) the QLTensor raw buffers already live in
 * device memory and are passed straight through. With the CPU build they are staged
 * through device buffers (one copy in, one copy out per call).
 *
 * Contract keeps its plans: the Context caches one plan per (A layout, B layout, axes) - the
 * device pairing, task list, operand-transpose work lists and the GEMM schedule the tuner
 * picked on the plan's first use - so the repeated contractions of a sweep pay the planning
 * once.
 *
 * Supported quantum numbers: U1QN, U1U1QN, fU1QN, fU1U1QN (integer-additive components;
 * the fermionic ones take their parity from the particle-number component).
 */
#ifndef QLTEN_GB300_H_
#define QLTEN_GB300_H_

#include <cuda_runtime.h>

#include <deque>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "qltg.h"

namespace qlten_gb300 {

inline void check(int rc) {
  if (rc != QLTG_OK) {
    if (rc == QLTG_ERR_EMPTY_SVD) throw qlten::EmptySVDResultError(qltg_last_error());
    throw std::runtime_error(std::string("qltg: ") + qltg_last_error());
  }
}

// ------------------------------------------------------------------ QN traits
template <typename QNT> struct QNTraits;
template <> struct QNTraits<qlten::special_qn::U1QN> {
  static constexpr int ncomp = 1, parity_comp = -1;
  static qlten::special_qn::U1QN make(const int32_t* v) { return qlten::special_qn::U1QN(v[0]); }
};
template <> struct QNTraits<qlten::special_qn::U1U1QN> {
  static constexpr int ncomp = 2, parity_comp = -1;
  static qlten::special_qn::U1U1QN make(const int32_t* v) { return qlten::special_qn::U1U1QN(v[0], v[1]); }
};
template <> struct QNTraits<qlten::special_qn::fU1QN> {
  static constexpr int ncomp = 1, parity_comp = 0;
  static qlten::special_qn::fU1QN make(const int32_t* v) { return qlten::special_qn::fU1QN(v[0]); }
};
template <> struct QNTraits<qlten::special_qn::fU1U1QN> {
  static constexpr int ncomp = 2, parity_comp = 0;
  static qlten::special_qn::fU1U1QN make(const int32_t* v) { return qlten::special_qn::fU1U1QN(v[0], v[1]); }
};

template <typename QNT>
void qn_values(const QNT& qn, int32_t* out) {
  for (int k = 0; k < QNTraits<QNT>::ncomp; ++k) out[k] = qn.GetQNVal(k).GetVal();
}

template <typename ElemT> constexpr int dtype_of() {
  return std::is_same<ElemT, qlten::QLTEN_Complex>::value ? QLTG_C128 : QLTG_F64;
}

// ------------------------------------------------------------------ descriptors
// Plain-array view of a QLTensor's indexes and block map (arrays owned by this object).
template <typename ElemT, typename QNT>
struct Desc {
  std::vector<int32_t> dirs, nsct, qns;
  std::vector<int64_t> dims, coords;
  qltg_tensor_desc d{};

  explicit Desc(const qlten::QLTensor<ElemT, QNT>& t) {
    for (const auto& ix : t.GetIndexes()) {
      dirs.push_back(ix.GetDir() == qlten::TenIndexDirType::IN ? QLTG_IN : QLTG_OUT);
      nsct.push_back((int32_t)ix.GetQNSctNum());
      for (const auto& s : ix.GetQNScts()) {
        int32_t v[4];
        qn_values(s.GetQn(), v);
        qns.insert(qns.end(), v, v + QNTraits<QNT>::ncomp);
        dims.push_back((int64_t)s.GetDegeneracy());
      }
    }
    for (const auto& kv : t.GetBlkSparDataTen().GetBlkIdxDataBlkMap())
      for (auto c : kv.second.blk_coors) coords.push_back((int64_t)c);
    d.rank = (int32_t)t.Rank();
    d.dtype = dtype_of<ElemT>();
    d.qn_ncomp = QNTraits<QNT>::ncomp;
    d.parity_comp = QNTraits<QNT>::parity_comp;
    d.dirs = dirs.data();
    d.nsct = nsct.data();
    d.qns = qns.data();
    d.dims = dims.data();
    d.nblk = (int64_t)t.GetBlkSparDataTen().GetBlkIdxDataBlkMap().size();
    d.coords = coords.data();
  }
};

// Raw data of a QLTensor as a device pointer: the buffer itself in a GPU build of qlten,
// a staged device copy in a CPU build (written back by sync_back for outputs).
template <typename ElemT, typename QNT>
class DeviceView {
 public:
  DeviceView(qlten::QLTensor<ElemT, QNT>& t, bool copy_in) : t_(t) {
    auto& bsdt = t.GetBlkSparDataTen();
    bytes_ = bsdt.GetActualRawDataSize() * sizeof(ElemT);
#ifdef USE_GPU
    (void)copy_in;
    ptr_ = bsdt.GetActualRawDataPtr();
#else
    if (bytes_) {
      if (cudaMalloc(&ptr_, bytes_) != cudaSuccess) throw std::runtime_error("qlten_gb300: cudaMalloc failed");
      if (copy_in && cudaMemcpy(ptr_, bsdt.GetActualRawDataPtr(), bytes_, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(ptr_);
        ptr_ = nullptr;
        throw std::runtime_error("qlten_gb300: copy of a tensor to the device failed");
      }
    }
#endif
  }
  ~DeviceView() {
#ifndef USE_GPU
    if (ptr_) cudaFree(ptr_);
#endif
  }
  DeviceView(const DeviceView&) = delete;
  DeviceView& operator=(const DeviceView&) = delete;
  void* get() const { return ptr_; }
  void sync_back() {
#ifndef USE_GPU
    if (bytes_ &&
        cudaMemcpy(t_.GetBlkSparDataTen().GetActualRawDataPtr(), ptr_, bytes_, cudaMemcpyDeviceToHost) != cudaSuccess)
      throw std::runtime_error("qlten_gb300: copy of a result to the host failed");
#endif
  }

 private:
  qlten::QLTensor<ElemT, QNT>& t_;
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

class Context {
 public:
  // max_plans: contraction plans kept for reuse (oldest dropped first); autotune: time the
  // candidate GEMM schedules on a plan's first use
  explicit Context(int device = 0, size_t max_plans = 256, bool autotune = true)
      : max_plans_(max_plans), autotune_(autotune) {
    check(qltg_create(device, &ctx_));
  }
  ~Context() {
    for (auto& kv : plans_) qltg_ctrct_plan_destroy(kv.second);
    qltg_destroy(ctx_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  qltg_ctx* get() const { return ctx_; }
  bool autotune() const { return autotune_; }

  // The cached plan of this (A layout, B layout, axes), or a new one (*fresh = true) that the
  // cache now owns.
  qltg_ctrct_plan* plan_for(const qltg_tensor_desc& a, const qltg_tensor_desc& b, const std::vector<int64_t>& axa,
                            const std::vector<int64_t>& axb, bool* fresh) const {
    std::vector<int64_t> key;
    append(key, a);
    append(key, b);
    key.push_back((int64_t)axa.size());
    key.insert(key.end(), axa.begin(), axa.end());
    key.insert(key.end(), axb.begin(), axb.end());
    auto it = plans_.find(key);
    *fresh = it == plans_.end();
    if (!*fresh) return it->second;
    qltg_ctrct_plan* plan = nullptr;
    check(qltg_ctrct_plan_create(ctx_, &a, &b, axa.data(), axb.data(), (int32_t)axa.size(), &plan));
    if (max_plans_ && plans_.size() >= max_plans_) {
      auto old = plans_.find(order_.front());
      qltg_ctrct_plan_destroy(old->second);
      plans_.erase(old);
      order_.pop_front();
    }
    plans_.emplace(key, plan);
    order_.push_back(key);
    return plan;
  }
  size_t cached_plans() const { return plans_.size(); }

 private:
  static void append(std::vector<int64_t>& k, const qltg_tensor_desc& d) {
    k.push_back(d.rank);
    k.push_back(d.dtype);
    k.push_back(d.qn_ncomp);
    k.push_back(d.parity_comp);
    int64_t ts = 0;
    for (int l = 0; l < d.rank; ++l) {
      k.push_back(d.dirs[l]);
      k.push_back(d.nsct[l]);
      ts += d.nsct[l];
    }
    for (int64_t i = 0; i < ts * d.qn_ncomp; ++i) k.push_back(d.qns[i]);
    k.insert(k.end(), d.dims, d.dims + ts);
    k.push_back(d.nblk);
    k.insert(k.end(), d.coords, d.coords + d.nblk * d.rank);
  }
  qltg_ctx* ctx_ = nullptr;
  size_t max_plans_;
  bool autotune_;
  mutable std::map<std::vector<int64_t>, qltg_ctrct_plan*> plans_;
  mutable std::deque<std::vector<int64_t>> order_;
};

// ------------------------------------------------------------------ Contract
template <typename ElemT, typename QNT>
void Contract(const qlten::QLTensor<ElemT, QNT>* pa, const qlten::QLTensor<ElemT, QNT>* pb,
              const std::vector<std::vector<size_t>>& axes_set, qlten::QLTensor<ElemT, QNT>* pc,
              const Context& ctx, int mode = QLTG_MODE_FP64) {
  Desc<ElemT, QNT> da(*pa), db(*pb);
  std::vector<int64_t> axa(axes_set[0].begin(), axes_set[0].end()), axb(axes_set[1].begin(), axes_set[1].end());
  bool fresh = false;
  qltg_ctrct_plan* plan = ctx.plan_for(da.d, db.d, axa, axb, &fresh);   // owned by the context
  // result legs: saved legs of A then saved legs of B (ten_ctrct.h:372-394)
  auto saved = qlten::TenCtrctGenSavedAxesSet(pa->Rank(), pb->Rank(), axes_set);
  qlten::TenCtrctInitResTen(pa, pb, saved, pc);
  int32_t rank = 0;
  int64_t nblk = 0, size = 0;
  check(qltg_ctrct_plan_result(plan, &rank, &nblk, &size));
  std::vector<int64_t> coords((size_t)nblk * rank);
  check(qltg_ctrct_plan_result_blocks(plan, coords.data(), nullptr));
  std::vector<qlten::CoorsT> blk_coors(nblk);
  for (int64_t b = 0; b < nblk; ++b) blk_coors[b].assign(coords.begin() + b * rank, coords.begin() + (b + 1) * rank);
  if (nblk) pc->GetBlkSparDataTen().DataBlksInsert(blk_coors, true, false);
  auto& a = const_cast<qlten::QLTensor<ElemT, QNT>&>(*pa);
  auto& b = const_cast<qlten::QLTensor<ElemT, QNT>&>(*pb);
  DeviceView<ElemT, QNT> va(a, true), vb(b, true), vc(*pc, false);
  if (fresh && ctx.autotune() && size) check(qltg_ctrct_plan_tune(plan, va.get(), vb.get(), vc.get(), mode, nullptr, nullptr));
  check(qltg_ctrct_exec(plan, va.get(), vb.get(), vc.get(), mode, nullptr));
  if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: contraction failed");
  vc.sync_back();
}

// ------------------------------------------------------------------ SVD / QR
namespace detail {

// Build a QLTensor from one exported result tensor of a decomposition.
template <typename ElemT, typename QNT>
void export_result(qltg_decomp* d, int which, qlten::QLTensor<ElemT, QNT>* out) {
  int64_t info[6];
  check(qltg_decomp_tensor_info(d, which, info));
  const int rank = (int)info[0], ncomp = (int)info[1];
  const int64_t nblk = info[3], ts = info[5];
  std::vector<int32_t> dirs(rank), nsct(rank), qns(ts * ncomp);
  std::vector<int64_t> dims(ts), coords(nblk * rank), offs(nblk);
  const void* dev = nullptr;
  check(qltg_decomp_tensor_export(d, which, dirs.data(), nsct.data(), qns.data(), dims.data(), coords.data(),
                                  offs.data(), &dev));
  qlten::IndexVec<QNT> idxs;
  int64_t qp = 0, dp = 0;
  for (int l = 0; l < rank; ++l) {
    std::vector<qlten::QNSector<QNT>> scts;
    for (int s = 0; s < nsct[l]; ++s) scts.emplace_back(QNTraits<QNT>::make(&qns[(qp + s) * ncomp]), (size_t)dims[dp + s]);
    qp += nsct[l];
    dp += nsct[l];
    idxs.emplace_back(scts, dirs[l] == QLTG_IN ? qlten::TenIndexDirType::IN : qlten::TenIndexDirType::OUT);
  }
  *out = qlten::QLTensor<ElemT, QNT>(idxs);
  std::vector<qlten::CoorsT> blk_coors(nblk);
  for (int64_t b = 0; b < nblk; ++b) blk_coors[b].assign(coords.begin() + b * rank, coords.begin() + (b + 1) * rank);
  if (nblk) out->GetBlkSparDataTen().DataBlksInsert(blk_coors, true, false);
  const size_t bytes = out->GetBlkSparDataTen().GetActualRawDataSize() * sizeof(ElemT);
#ifdef USE_GPU
  const cudaMemcpyKind kind = cudaMemcpyDeviceToDevice;
#else
  const cudaMemcpyKind kind = cudaMemcpyDeviceToHost;
#endif
  if (bytes && cudaMemcpy(out->GetBlkSparDataTen().GetActualRawDataPtr(), dev, bytes, kind) != cudaSuccess)
    throw std::runtime_error("qlten_gb300: result copy failed");
}

}  // namespace detail

template <typename ElemT, typename QNT>
void SVD(const qlten::QLTensor<ElemT, QNT>* pt, size_t ldims, const QNT& lqndiv, double trunc_err, size_t Dmin,
         size_t Dmax, qlten::QLTensor<ElemT, QNT>* pu, qlten::QLTensor<qlten::QLTEN_Double, QNT>* ps,
         qlten::QLTensor<ElemT, QNT>* pvt, double* pactual_trunc_err, size_t* pD, const Context& ctx) {
  Desc<ElemT, QNT> dt(*pt);
  int32_t div[4];
  qn_values(lqndiv, div);
  auto& t = const_cast<qlten::QLTensor<ElemT, QNT>&>(*pt);
  DeviceView<ElemT, QNT> vt(t, true);
  qltg_decomp* d = nullptr;
  check(qltg_svd(ctx.get(), &dt.d, vt.get(), (int32_t)ldims, div, trunc_err, (int64_t)Dmin, (int64_t)Dmax, nullptr, &d));
  try {
    int64_t D = 0;
    check(qltg_decomp_info(d, pactual_trunc_err, &D));
    *pD = (size_t)D;
    detail::export_result(d, 0, pu);
    detail::export_result(d, 1, ps);
    detail::export_result(d, 2, pvt);
  } catch (...) {
    qltg_decomp_destroy(d);
    throw;
  }
  qltg_decomp_destroy(d);
}

template <typename ElemT, typename QNT>
void QR(const qlten::QLTensor<ElemT, QNT>* pt, size_t ldims, const QNT& lqndiv, qlten::QLTensor<ElemT, QNT>* pq,
        qlten::QLTensor<ElemT, QNT>* pr, const Context& ctx) {
  Desc<ElemT, QNT> dt(*pt);
  int32_t div[4];
  qn_values(lqndiv, div);
  auto& t = const_cast<qlten::QLTensor<ElemT, QNT>&>(*pt);
  DeviceView<ElemT, QNT> vt(t, true);
  qltg_decomp* d = nullptr;
  check(qltg_qr(ctx.get(), &dt.d, vt.get(), (int32_t)ldims, div, nullptr, &d));
  try {
    detail::export_result(d, 0, pq);
    detail::export_result(d, 1, pr);
  } catch (...) {
    qltg_decomp_destroy(d);
    throw;
  }
  qltg_decomp_destroy(d);
}

// ------------------------------------------------------------------ contiguous axes
namespace detail {

inline void scalar_pair(double v, double* o) {
  o[0] = v;
  o[1] = 0.0;
}
inline void scalar_pair(const qlten::QLTEN_Complex& v, double* o) {
  o[0] = v.real();
  o[1] = v.imag();
}

// *out = a tensor with `idxs` holding the blocks listed by a plan's result query.
template <typename ElemT, typename QNT, typename ResultFn, typename BlocksFn, typename Plan>
void init_from_plan(qlten::QLTensor<ElemT, QNT>* out, const qlten::IndexVec<QNT>& idxs, Plan* plan, ResultFn result,
                    BlocksFn blocks) {
  int32_t rank = 0;
  int64_t nblk = 0, size = 0;
  check(result(plan, &rank, &nblk, &size));
  if (rank == 0) throw std::invalid_argument("qlten_gb300: scalar results go through Contract");
  std::vector<int64_t> coords((size_t)nblk * rank);
  check(blocks(plan, coords.data(), nullptr));
  *out = qlten::QLTensor<ElemT, QNT>(idxs);
  std::vector<qlten::CoorsT> blk_coors(nblk);
  for (int64_t b = 0; b < nblk; ++b) blk_coors[b].assign(coords.begin() + b * rank, coords.begin() + (b + 1) * rank);
  if (nblk) out->GetBlkSparDataTen().DataBlksInsert(blk_coors, true, false);
}

// Result indexes of ContractContiguousAxes: A's saved legs, then B's, each in cyclic order from
// the end of its contracted range (contract_contiguous_axes.h:849-868).
template <typename ElemT, typename QNT>
qlten::IndexVec<QNT> contiguous_result_indexes(const qlten::QLTensor<ElemT, QNT>& a, const qlten::QLTensor<ElemT, QNT>& b,
                                               size_t a0, size_t b0, size_t n) {
  qlten::IndexVec<QNT> idxs;
  const size_t ra = a.Rank(), rb = b.Rank();
  for (size_t i = 0; i + n < ra; ++i) idxs.push_back(a.GetIndex((a0 + n + i) % ra));
  for (size_t i = 0; i + n < rb; ++i) idxs.push_back(b.GetIndex((b0 + n + i) % rb));
  return idxs;
}

template <typename ElemT, typename QNT>
bool accumulate(const qlten::QLTensor<ElemT, QNT>& a, const qlten::QLTensor<ElemT, QNT>& b, size_t a0, size_t b0,
                size_t n, ElemT alpha, ElemT beta, qlten::QLTensor<ElemT, QNT>& c, const Context& ctx, int mode,
                bool allow_expand) {
  Desc<ElemT, QNT> da(a), db(b);
  const bool has_c = !c.IsDefault();
  std::vector<Desc<ElemT, QNT>> dc;
  if (has_c) dc.emplace_back(c);
  qltg_accum_plan* acc = nullptr;
  int32_t expanded = 0;
  const int rc = qltg_accum_plan_create(ctx.get(), &da.d, &db.d, (int64_t)a0, (int64_t)b0, (int32_t)n,
                                        has_c ? &dc[0].d : nullptr, allow_expand ? 1 : 0, &acc, &expanded);
  if (rc == QLTG_ERR_LAYOUT && !allow_expand) return false;   // the Try form: C untouched
  check(rc);
  try {
    double al[2], be[2];
    scalar_pair(alpha, al);
    scalar_pair(beta, be);
    auto& ma = const_cast<qlten::QLTensor<ElemT, QNT>&>(a);
    auto& mb = const_cast<qlten::QLTensor<ElemT, QNT>&>(b);
    DeviceView<ElemT, QNT> va(ma, true), vb(mb, true);
    if (!has_c || expanded) {   // a new output topology
      qlten::QLTensor<ElemT, QNT> out;
      init_from_plan(&out, has_c ? c.GetIndexes() : contiguous_result_indexes(a, b, a0, b0, n), acc,
                     qltg_accum_plan_result, qltg_accum_plan_result_blocks);
      DeviceView<ElemT, QNT> vo(out, false);
      if (has_c) {
        DeviceView<ElemT, QNT> vc(c, true);
        check(qltg_accum_exec(acc, va.get(), vb.get(), vc.get(), vo.get(), al, be, mode, nullptr));
      } else {
        check(qltg_accum_exec(acc, va.get(), vb.get(), nullptr, vo.get(), al, be, mode, nullptr));
      }
      if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: accumulate failed");
      vo.sync_back();
      c = std::move(out);
    } else {                    // in place
      DeviceView<ElemT, QNT> vc(c, true);
      check(qltg_accum_exec(acc, va.get(), vb.get(), vc.get(), vc.get(), al, be, mode, nullptr));
      if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: accumulate failed");
      vc.sync_back();
    }
  } catch (...) {
    qltg_accum_plan_destroy(acc);
    throw;
  }
  qltg_accum_plan_destroy(acc);
  return true;
}

}  // namespace detail

// qlten::ContractContiguousAxes<ElemT, QNT, ASide, BSide>(A, B, a0, b0, n, C)
// (contract_contiguous_axes.h:849-868); the sides only tell which view needs no transpose.
template <typename ElemT, typename QNT>
void ContractContiguousAxes(const qlten::QLTensor<ElemT, QNT>& a, const qlten::QLTensor<ElemT, QNT>& b, size_t a0,
                            size_t b0, size_t n, qlten::QLTensor<ElemT, QNT>& c, const Context& ctx,
                            int mode = QLTG_MODE_FP64, int a_side = QLTG_SIDE_TAIL, int b_side = QLTG_SIDE_HEAD) {
  Desc<ElemT, QNT> da(a), db(b);
  qltg_ctrct_plan* plan = nullptr;
  check(qltg_ctrct_plan_create_contiguous(ctx.get(), &da.d, &db.d, (int64_t)a0, (int64_t)b0, (int32_t)n, a_side,
                                          b_side, &plan));
  try {
    detail::init_from_plan(&c, detail::contiguous_result_indexes(a, b, a0, b0, n), plan, qltg_ctrct_plan_result,
                           qltg_ctrct_plan_result_blocks);
    auto& ma = const_cast<qlten::QLTensor<ElemT, QNT>&>(a);
    auto& mb = const_cast<qlten::QLTensor<ElemT, QNT>&>(b);
    DeviceView<ElemT, QNT> va(ma, true), vb(mb, true), vc(c, false);
    check(qltg_ctrct_exec(plan, va.get(), vb.get(), vc.get(), mode, nullptr));
    if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: contraction failed");
    vc.sync_back();
  } catch (...) {
    qltg_ctrct_plan_destroy(plan);
    throw;
  }
  qltg_ctrct_plan_destroy(plan);
}

// C = beta C + alpha A.B over the union topology (ContractTailHeadContiguousAccumulate,
// contract_contiguous_axes.h:953-1000); a default C needs beta == 0.
template <typename ElemT, typename QNT>
void ContractTailHeadContiguousAccumulate(const qlten::QLTensor<ElemT, QNT>& a, const qlten::QLTensor<ElemT, QNT>& b,
                                          size_t a0, size_t b0, size_t n, ElemT alpha, ElemT beta,
                                          qlten::QLTensor<ElemT, QNT>& c, const Context& ctx,
                                          int mode = QLTG_MODE_FP64) {
  detail::accumulate(a, b, a0, b0, n, alpha, beta, c, ctx, mode, true);
}

// The no-expansion form (contract_contiguous_axes.h:1002-1040): false, C untouched, when C
// lacks blocks the product needs or has other indexes.
template <typename ElemT, typename QNT>
bool TryContractTailHeadContiguousAccumulate(const qlten::QLTensor<ElemT, QNT>& a,
                                             const qlten::QLTensor<ElemT, QNT>& b, size_t a0, size_t b0, size_t n,
                                             ElemT alpha, ElemT beta, qlten::QLTensor<ElemT, QNT>& c,
                                             const Context& ctx, int mode = QLTG_MODE_FP64) {
  return detail::accumulate(a, b, a0, b0, n, alpha, beta, c, ctx, mode, false);
}

// ------------------------------------------------------------------ LinearCombine
// *pres = sum_i coefs[i] *tens[i] + beta *pres over the union of the contributing blocks
// (LinearCombine, tensor_manipulation/ten_linear_combine.h:186-197).
template <typename ElemT, typename QNT>
void LinearCombine(const std::vector<ElemT>& coefs, const std::vector<qlten::QLTensor<ElemT, QNT>*>& tens, ElemT beta,
                   qlten::QLTensor<ElemT, QNT>* pres, const Context& ctx) {
  const size_t n = tens.size();
  if (n == 0 || coefs.size() != n) throw std::invalid_argument("qlten_gb300: one coefficient per tensor");
  std::vector<Desc<ElemT, QNT>> descs;
  descs.reserve(n + 1);
  std::vector<const qltg_tensor_desc*> dptr;
  for (auto* t : tens) {
    descs.emplace_back(*t);
    dptr.push_back(&descs.back().d);
  }
  const bool has_res = !pres->IsDefault();
  if (has_res) descs.emplace_back(*pres);
  std::vector<double> cf;
  for (const auto& x : coefs) {
    double v[2];
    detail::scalar_pair(x, v);
    cf.push_back(v[0]);
    if (dtype_of<ElemT>() == QLTG_C128) cf.push_back(v[1]);
  }
  double be[2];
  detail::scalar_pair(beta, be);
  qltg_lincomb_plan* lc = nullptr;
  check(qltg_lincomb_plan_create(ctx.get(), (int32_t)n, dptr.data(), cf.data(), has_res ? &descs[n].d : nullptr, be,
                                 0, &lc));
  try {
    qlten::QLTensor<ElemT, QNT> out;
    detail::init_from_plan(&out, tens[0]->GetIndexes(), lc, qltg_lincomb_plan_result,
                           qltg_lincomb_plan_result_blocks);
    std::vector<std::unique_ptr<DeviceView<ElemT, QNT>>> views;
    std::vector<const void*> devs;
    for (auto* t : tens) {
      views.push_back(std::make_unique<DeviceView<ElemT, QNT>>(*t, true));
      devs.push_back(views.back()->get());
    }
    DeviceView<ElemT, QNT> vo(out, false);
    if (has_res) {
      DeviceView<ElemT, QNT> vr(*pres, true);
      check(qltg_lincomb_exec(lc, devs.data(), vr.get(), vo.get(), nullptr));
      if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: combination failed");
    } else {
      check(qltg_lincomb_exec(lc, devs.data(), nullptr, vo.get(), nullptr));
      if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: combination failed");
    }
    vo.sync_back();
    *pres = std::move(out);
  } catch (...) {
    qltg_lincomb_plan_destroy(lc);
    throw;
  }
  qltg_lincomb_plan_destroy(lc);
}

}  // namespace qlten_gb300

#endif  // QLTEN_GB300_H_
