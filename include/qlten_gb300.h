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
 *   qlten::dmrg::ApplyAxisDiagonal / ProjectAxis / ApplyAxisMonomial / ApplyRank2ToAxis... /
 *   the composed ApplyRank2Then... / ApplyTwoRank2Then... forms / MoveHeadAxisToTail
 *   (tensor_manipulation/dmrg/axis_ops.h:2391-3678)
 *     -> qlten_gb300::dmrg::<same name>(<same arguments>, ctx [, mode]) (bosonic tensors)
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
#include "qlten/tensor_manipulation/dmrg/axis_ops.h"

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

// ------------------------------------------------------------------ qlten::dmrg axis operations
// The bosonic axis-local operators of qlten::dmrg (tensor_manipulation/dmrg/axis_ops.h) with
// the reference's signatures plus a Context. The work counters (AxisOpStats and friends) are
// reset and left at zero: the device path has no loop of host GEMM calls to count. The
// composed forms run as the device primitives in sequence (the reference's "Fused" forms avoid
// a CPU intermediate; here the intermediate is one device tensor).
namespace dmrg {

namespace detail {

template <typename ElemT>
void append_value(std::vector<double>& v, const ElemT& x) {
  double p[2];
  qlten_gb300::detail::scalar_pair(x, p);
  v.push_back(p[0]);
  if (dtype_of<ElemT>() == QLTG_C128) v.push_back(p[1]);
}

inline void sync_or_throw(const char* what) {
  if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error(std::string("qlten_gb300: ") + what);
}

// A tensor with `idxs` and the blocks an axis plan reports.
template <typename ElemT, typename QNT>
qlten::QLTensor<ElemT, QNT> from_axis_plan(const qlten::IndexVec<QNT>& idxs, qltg_axis_plan* plan) {
  qlten::QLTensor<ElemT, QNT> out;
  qlten_gb300::detail::init_from_plan(&out, idxs, plan, qltg_axis_plan_result, qltg_axis_plan_result_blocks);
  return out;
}

// Destroys an axis plan on every way out.
struct AxisPlan {
  qltg_axis_plan* h = nullptr;
  ~AxisPlan() {
    if (h) qltg_axis_plan_destroy(h);
  }
};

template <typename ElemT, typename QNT>
qlten::QLTensor<ElemT, QNT> rank2(const qlten::QLTensor<ElemT, QNT>& in, const qlten::QLTensor<ElemT, QNT>& op1,
                                  size_t axis1, const qlten::QLTensor<ElemT, QNT>* op2, size_t axis2,
                                  const Context& ctx, int mode) {
  Desc<ElemT, QNT> dt(in), d1(op1);
  AxisPlan plan;
  qlten::IndexVec<QNT> idxs = in.GetIndexes();
  idxs[axis1] = op1.GetIndex(1);
  if (op2) {
    Desc<ElemT, QNT> d2(*op2);
    check(qltg_axis_two_rank2_plan_create(ctx.get(), &dt.d, &d1.d, (int32_t)axis1, &d2.d, (int32_t)axis2, &plan.h));
    idxs[axis2] = op2->GetIndex(1);
  } else {
    check(qltg_axis_rank2_plan_create(ctx.get(), &dt.d, &d1.d, (int32_t)axis1, &plan.h));
  }
  auto out = from_axis_plan<ElemT, QNT>(idxs, plan.h);
  auto& mi = const_cast<qlten::QLTensor<ElemT, QNT>&>(in);
  auto& m1 = const_cast<qlten::QLTensor<ElemT, QNT>&>(op1);
  DeviceView<ElemT, QNT> vi(mi, true), v1(m1, true), vo(out, false);
  std::unique_ptr<DeviceView<ElemT, QNT>> v2;
  if (op2) v2 = std::make_unique<DeviceView<ElemT, QNT>>(const_cast<qlten::QLTensor<ElemT, QNT>&>(*op2), true);
  check(qltg_axis_plan_exec(plan.h, vi.get(), v1.get(), v2 ? v2->get() : nullptr, vo.get(), mode, nullptr));
  check(qltg_axis_plan_device_status(plan.h, nullptr));
  vo.sync_back();
  return out;
}

template <typename ElemT, typename QNT>
void sector_scalars(const qlten::QLTensor<ElemT, QNT>& in, size_t axis, const std::vector<ElemT>& values,
                    qlten::QLTensor<ElemT, QNT>& out, const Context& ctx) {
  Desc<ElemT, QNT> dt(in);
  std::vector<double> v;
  for (const auto& x : values) append_value(v, x);
  auto& mi = const_cast<qlten::QLTensor<ElemT, QNT>&>(in);
  if (&out != &in) {
    out = qlten::QLTensor<ElemT, QNT>(in.GetIndexes());
    std::vector<qlten::CoorsT> coors;
    for (const auto& kv : in.GetBlkSparDataTen().GetBlkIdxDataBlkMap()) coors.push_back(kv.second.blk_coors);
    if (!coors.empty()) out.GetBlkSparDataTen().DataBlksInsert(coors, true, false);
  }
  DeviceView<ElemT, QNT> vi(mi, true);
  if (&out == &in) {
    check(qltg_axis_sector_scalars(ctx.get(), &dt.d, (int32_t)axis, v.data(), vi.get(), vi.get(), nullptr));
    sync_or_throw("axis sector scalars failed");
    vi.sync_back();
  } else {
    DeviceView<ElemT, QNT> vo(out, false);
    check(qltg_axis_sector_scalars(ctx.get(), &dt.d, (int32_t)axis, v.data(), vi.get(), vo.get(), nullptr));
    sync_or_throw("axis sector scalars failed");
    vo.sync_back();
  }
}

}  // namespace detail

// output = beta output + alpha D(input) (axis_ops.h:2391-2466); output = input with alpha 1,
// beta 0 is ApplyAxisDiagonalInPlace.
template <typename ElemT, typename QNT>
void ApplyAxisDiagonal(const qlten::QLTensor<ElemT, QNT>& input, size_t axis,
                       const qlten::dmrg::AxisDiagonalOp<ElemT, QNT>& op, qlten::QLTensor<ElemT, QNT>& output,
                       const Context& ctx, ElemT alpha = ElemT(1), ElemT beta = ElemT(0)) {
  Desc<ElemT, QNT> dt(input);
  std::vector<double> v;
  for (const auto& sector : op.values)
    for (const auto& x : sector) detail::append_value(v, x);
  double al[2], be[2];
  qlten_gb300::detail::scalar_pair(alpha, al);
  qlten_gb300::detail::scalar_pair(beta, be);
  auto& mi = const_cast<qlten::QLTensor<ElemT, QNT>&>(input);
  if (&output == &input) {
    DeviceView<ElemT, QNT> vi(mi, true);
    check(qltg_axis_diagonal(ctx.get(), &dt.d, (int32_t)axis, v.data(), vi.get(), vi.get(), al, be, nullptr));
    detail::sync_or_throw("axis diagonal failed");
    vi.sync_back();
    return;
  }
  const bool keep = be[0] != 0.0 || be[1] != 0.0;
  if (!keep) {
    output = qlten::QLTensor<ElemT, QNT>(input.GetIndexes());
    std::vector<qlten::CoorsT> coors;
    for (const auto& kv : input.GetBlkSparDataTen().GetBlkIdxDataBlkMap()) coors.push_back(kv.second.blk_coors);
    if (!coors.empty()) output.GetBlkSparDataTen().DataBlksInsert(coors, true, false);
  }
  DeviceView<ElemT, QNT> vi(mi, true), vo(output, keep);
  check(qltg_axis_diagonal(ctx.get(), &dt.d, (int32_t)axis, v.data(), vi.get(), vo.get(), al, be, nullptr));
  detail::sync_or_throw("axis diagonal failed");
  vo.sync_back();
}

// axis_ops.h:2548-2582
template <typename ElemT, typename QNT>
void ApplyAxisDiagonalInPlace(qlten::QLTensor<ElemT, QNT>& tensor, size_t axis,
                              const qlten::dmrg::AxisDiagonalOp<ElemT, QNT>& op, const Context& ctx) {
  ApplyAxisDiagonal(tensor, axis, op, tensor, ctx);
}

// axis_ops.h:2583-2637 (either storage mode gives the same result here; kConsumeOwnedInPlace
// with output aliasing input scales in place)
template <typename ElemT, typename QNT>
void ApplyAxisDiagonalPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input, size_t axis,
                                    const qlten::dmrg::AxisDiagonalOp<ElemT, QNT>& op,
                                    qlten::QLTensor<ElemT, QNT>& output, qlten::dmrg::AxisApplyStorageMode,
                                    const Context& ctx, qlten::dmrg::AxisOpStats* stats = nullptr) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  ApplyAxisDiagonal(input, axis, op, output, ctx);
}

// axis_ops.h:2638-2675
template <typename ElemT, typename QNT>
void ScaleAxisSectorsInPlace(qlten::QLTensor<ElemT, QNT>& tensor, const qlten::dmrg::AxisSectorScalar<ElemT, QNT>& scale,
                             const Context& ctx) {
  detail::sector_scalars(tensor, scale.axis, scale.values_by_sector, tensor, ctx);
}

// axis_ops.h:2676-2744
template <typename ElemT, typename QNT>
void ApplyAxisSectorScalarsPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input,
                                         const qlten::dmrg::AxisSectorScalar<ElemT, QNT>& scale,
                                         qlten::QLTensor<ElemT, QNT>& output, qlten::dmrg::AxisApplyStorageMode,
                                         const Context& ctx, qlten::dmrg::AxisOpStats* stats = nullptr) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  detail::sector_scalars(input, scale.axis, scale.values_by_sector, output, ctx);
}

// output = beta output + alpha M(input) (axis_ops.h:2772-2860); beta != 0 needs an output with
// the result's topology.
template <typename ElemT, typename QNT>
void ApplyAxisMonomial(const qlten::QLTensor<ElemT, QNT>& input, size_t axis,
                       const qlten::dmrg::AxisMonomialOp<ElemT, QNT>& op, qlten::QLTensor<ElemT, QNT>& output,
                       const Context& ctx, ElemT alpha = ElemT(1), ElemT beta = ElemT(0)) {
  Desc<ElemT, QNT> dt(input);
  std::vector<int32_t> oq;
  std::vector<int64_t> od, ent;
  for (const auto& s : op.output_index.GetQNScts()) {
    int32_t v[4];
    qn_values(s.GetQn(), v);
    oq.insert(oq.end(), v, v + QNTraits<QNT>::ncomp);
    od.push_back((int64_t)s.GetDegeneracy());
  }
  int32_t flux[4];
  qn_values(op.flux, flux);
  std::vector<double> cf;
  for (const auto& e : op.entries) {
    ent.insert(ent.end(), {(int64_t)e.in_sector, (int64_t)e.in_offset, (int64_t)e.out_sector, (int64_t)e.out_offset});
    detail::append_value(cf, e.coef);
  }
  detail::AxisPlan plan;
  check(qltg_axis_monomial_plan_create(ctx.get(), &dt.d, (int32_t)axis, (int32_t)od.size(), oq.data(), od.data(),
                                       flux, (int64_t)op.entries.size(), ent.empty() ? nullptr : ent.data(),
                                       cf.empty() ? nullptr : cf.data(), &plan.h));
  double al[2], be[2];
  qlten_gb300::detail::scalar_pair(alpha, al);
  qlten_gb300::detail::scalar_pair(beta, be);
  const bool keep = be[0] != 0.0 || be[1] != 0.0;
  qlten::IndexVec<QNT> idxs = input.GetIndexes();
  idxs[axis] = op.output_index;
  if (!keep) output = detail::from_axis_plan<ElemT, QNT>(idxs, plan.h);
  auto& mi = const_cast<qlten::QLTensor<ElemT, QNT>&>(input);
  DeviceView<ElemT, QNT> vi(mi, true), vo(output, keep);
  check(qltg_axis_monomial_exec(plan.h, vi.get(), vo.get(), al, be, nullptr));
  detail::sync_or_throw("axis monomial failed");
  vo.sync_back();
}

// axis_ops.h:2468-2532
template <typename ElemT, typename QNT>
void ProjectAxis(const qlten::QLTensor<ElemT, QNT>& input, size_t axis, const qlten::dmrg::AxisProjector<QNT>& projector,
                 qlten::QLTensor<ElemT, QNT>& output, const Context& ctx) {
  Desc<ElemT, QNT> dt(input);
  std::vector<int64_t> counts, kept;
  std::vector<qlten::QNSector<QNT>> scts;
  const auto& in_scts = input.GetIndex(axis).GetQNScts();
  for (size_t s = 0; s < projector.kept_degeneracies.size(); ++s) {
    const auto& k = projector.kept_degeneracies[s];
    counts.push_back((int64_t)k.size());
    for (auto x : k) kept.push_back((int64_t)x);
    if (!k.empty()) scts.emplace_back(in_scts.at(s).GetQn(), k.size());
  }
  detail::AxisPlan plan;
  check(qltg_axis_project_plan_create(ctx.get(), &dt.d, (int32_t)axis, counts.data(), kept.empty() ? nullptr : kept.data(),
                                      &plan.h));
  qlten::IndexVec<QNT> idxs = input.GetIndexes();
  idxs[axis] = qlten::Index<QNT>(scts, input.GetIndex(axis).GetDir());
  output = detail::from_axis_plan<ElemT, QNT>(idxs, plan.h);
  double al[2] = {1.0, 0.0}, be[2] = {0.0, 0.0};
  auto& mi = const_cast<qlten::QLTensor<ElemT, QNT>&>(input);
  DeviceView<ElemT, QNT> vi(mi, true), vo(output, false);
  check(qltg_axis_monomial_exec(plan.h, vi.get(), vo.get(), al, be, nullptr));
  detail::sync_or_throw("axis projection failed");
  vo.sync_back();
}

// axis_ops.h:2889-2993 (rank2_op index 0 contracts with `target_axis`, index 1 takes its place)
template <typename ElemT, typename QNT>
void ApplyRank2ToAxisPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input, const qlten::QLTensor<ElemT, QNT>& rank2_op,
                                   size_t target_axis, qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                   qlten::dmrg::Rank2AxisApplyStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::Rank2AxisApplyStats{};
  out = detail::rank2(input, rank2_op, target_axis, (const qlten::QLTensor<ElemT, QNT>*)nullptr, 0, ctx, mode);
}

// axis_ops.h:2994-3126
template <typename ElemT, typename QNT>
void ApplyTwoRank2ToAxesPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input, const qlten::QLTensor<ElemT, QNT>& op1,
                                      size_t axis1, const qlten::QLTensor<ElemT, QNT>& op2, size_t axis2,
                                      qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                      qlten::dmrg::AxisOpStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  out = detail::rank2(input, op1, axis1, &op2, axis2, ctx, mode);
}

// axis_ops.h:3127-3151
template <typename ElemT, typename QNT>
void ApplyRank2ThenAxisDiagonalPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input,
                                             const qlten::QLTensor<ElemT, QNT>& rank2_op, size_t rank2_axis,
                                             size_t diagonal_axis, const qlten::dmrg::AxisDiagonalOp<ElemT, QNT>& diagonal,
                                             qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                             qlten::dmrg::AxisOpStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  out = detail::rank2(input, rank2_op, rank2_axis, (const qlten::QLTensor<ElemT, QNT>*)nullptr, 0, ctx, mode);
  ApplyAxisDiagonal(out, diagonal_axis, diagonal, out, ctx);
}

// axis_ops.h:3152-3180
template <typename ElemT, typename QNT>
void ApplyRank2ThenAxisSectorScalarsPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input,
                                                  const qlten::QLTensor<ElemT, QNT>& rank2_op, size_t rank2_axis,
                                                  const qlten::dmrg::AxisSectorScalar<ElemT, QNT>& scale,
                                                  qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                                  qlten::dmrg::AxisOpStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  out = detail::rank2(input, rank2_op, rank2_axis, (const qlten::QLTensor<ElemT, QNT>*)nullptr, 0, ctx, mode);
  detail::sector_scalars(out, scale.axis, scale.values_by_sector, out, ctx);
}

// out = beta out + alpha S(R(input)) with R on axis 0 or the last axis (axis_ops.h:3181-3283):
// an existing out keeps its blocks and gains the ones R produces; a default out needs beta 0.
template <typename ElemT, typename QNT>
void ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder(
    const qlten::QLTensor<ElemT, QNT>& input, const qlten::QLTensor<ElemT, QNT>& rank2_op, size_t rank2_axis,
    const qlten::dmrg::AxisSectorScalar<ElemT, QNT>& scale, const ElemT alpha, const ElemT beta,
    qlten::QLTensor<ElemT, QNT>& out, const Context& ctx, qlten::dmrg::AxisOpStats* stats = nullptr,
    int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  if (rank2_axis != 0 && rank2_axis + 1 != input.Rank())
    throw std::invalid_argument("qlten_gb300: rank2_axis must be axis 0 or the last axis");
  double be[2];
  qlten_gb300::detail::scalar_pair(beta, be);
  const bool has_out = !out.IsDefault();
  if (!has_out && (be[0] != 0.0 || be[1] != 0.0))
    throw std::invalid_argument("qlten_gb300: beta != 0 needs an existing output");
  qlten::QLTensor<ElemT, QNT> r =
      detail::rank2(input, rank2_op, rank2_axis, (const qlten::QLTensor<ElemT, QNT>*)nullptr, 0, ctx, mode);
  detail::sector_scalars(r, scale.axis, scale.values_by_sector, r, ctx);
  // out = alpha r + beta out over the union of both block sets, out's blocks kept
  Desc<ElemT, QNT> dr(r);
  std::vector<Desc<ElemT, QNT>> dout;
  if (has_out) dout.emplace_back(out);
  const qltg_tensor_desc* dp = &dr.d;
  std::vector<double> cf;
  detail::append_value(cf, alpha);
  qltg_lincomb_plan* lc = nullptr;
  check(qltg_lincomb_plan_create(ctx.get(), 1, &dp, cf.data(), has_out ? &dout[0].d : nullptr, be, has_out ? 1 : 0, &lc));
  try {
    qlten::QLTensor<ElemT, QNT> res;
    qlten_gb300::detail::init_from_plan(&res, r.GetIndexes(), lc, qltg_lincomb_plan_result,
                                        qltg_lincomb_plan_result_blocks);
    DeviceView<ElemT, QNT> vr(r, true), vo(res, false);
    const void* src = vr.get();
    if (has_out) {
      DeviceView<ElemT, QNT> vold(out, true);
      check(qltg_lincomb_exec(lc, &src, vold.get(), vo.get(), nullptr));
      detail::sync_or_throw("accumulate failed");
    } else {
      check(qltg_lincomb_exec(lc, &src, nullptr, vo.get(), nullptr));
      detail::sync_or_throw("accumulate failed");
    }
    vo.sync_back();
    out = std::move(res);
  } catch (...) {
    qltg_lincomb_plan_destroy(lc);
    throw;
  }
  qltg_lincomb_plan_destroy(lc);
}

// axis_ops.h:3284-3302: the accumulate form with alpha 1, beta 0, as in the reference
template <typename ElemT, typename QNT>
void ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder(
    const qlten::QLTensor<ElemT, QNT>& input, const qlten::QLTensor<ElemT, QNT>& rank2_op, size_t rank2_axis,
    const qlten::dmrg::AxisSectorScalar<ElemT, QNT>& scale, qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
    qlten::dmrg::AxisOpStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder(input, rank2_op, rank2_axis, scale, ElemT(1), ElemT(0),
                                                                 out, ctx, stats, mode);
}

// axis_ops.h:3319-3503: the rank-2 operator, then the monomial on the result
template <typename ElemT, typename QNT>
void ApplyRank2ThenAxisMonomialFusedPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input,
                                                  const qlten::QLTensor<ElemT, QNT>& rank2_op, size_t rank2_axis,
                                                  size_t monomial_axis,
                                                  const qlten::dmrg::AxisMonomialOp<ElemT, QNT>& monomial,
                                                  qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                                  qlten::dmrg::AxisOpStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  if (&input == &out || &rank2_op == &out) throw std::invalid_argument("qlten_gb300: output aliasing is not allowed");
  const qlten::QLTensor<ElemT, QNT> r =
      detail::rank2(input, rank2_op, rank2_axis, (const qlten::QLTensor<ElemT, QNT>*)nullptr, 0, ctx, mode);
  ApplyAxisMonomial(r, monomial_axis, monomial, out, ctx);
}

// axis_ops.h:3504-3532
template <typename ElemT, typename QNT>
void ApplyTwoRank2ThenAxisDiagonalPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input,
                                                const qlten::QLTensor<ElemT, QNT>& op1, size_t axis1,
                                                const qlten::QLTensor<ElemT, QNT>& op2, size_t axis2,
                                                size_t diagonal_axis,
                                                const qlten::dmrg::AxisDiagonalOp<ElemT, QNT>& diagonal,
                                                qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                                qlten::dmrg::AxisOpStats* stats = nullptr, int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  out = detail::rank2(input, op1, axis1, &op2, axis2, ctx, mode);
  ApplyAxisDiagonal(out, diagonal_axis, diagonal, out, ctx);
}

// axis_ops.h:3533-3577
template <typename ElemT, typename QNT>
void ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder(const qlten::QLTensor<ElemT, QNT>& input,
                                                     const qlten::QLTensor<ElemT, QNT>& op1, size_t axis1,
                                                     const qlten::QLTensor<ElemT, QNT>& op2, size_t axis2,
                                                     const qlten::dmrg::AxisSectorScalar<ElemT, QNT>& scale,
                                                     qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                                                     qlten::dmrg::AxisOpStats* stats = nullptr,
                                                     int mode = QLTG_MODE_FP64) {
  if (stats) *stats = qlten::dmrg::AxisOpStats{};
  out = detail::rank2(input, op1, axis1, &op2, axis2, ctx, mode);
  detail::sector_scalars(out, scale.axis, scale.values_by_sector, out, ctx);
}

// axis_ops.h:3578-3678: axis 0 moved to the end (a bosonic transpose)
template <typename ElemT, typename QNT>
void MoveHeadAxisToTail(const qlten::QLTensor<ElemT, QNT>& input, qlten::QLTensor<ElemT, QNT>& out, const Context& ctx,
                        qlten::dmrg::AxisLayoutMoveStats* stats = nullptr) {
  if (stats) *stats = qlten::dmrg::AxisLayoutMoveStats{};
  const size_t r = input.Rank();
  std::vector<int32_t> perm;
  for (size_t i = 1; i < r; ++i) perm.push_back((int32_t)i);
  perm.push_back(0);
  qlten::IndexVec<QNT> idxs;
  for (auto i : perm) idxs.push_back(input.GetIndex(i));
  out = qlten::QLTensor<ElemT, QNT>(idxs);
  std::vector<qlten::CoorsT> coors;
  for (const auto& kv : input.GetBlkSparDataTen().GetBlkIdxDataBlkMap()) {
    qlten::CoorsT c;
    for (auto i : perm) c.push_back(kv.second.blk_coors[i]);
    coors.push_back(c);
  }
  if (!coors.empty()) out.GetBlkSparDataTen().DataBlksInsert(coors, true, false);
  Desc<ElemT, QNT> dt(input);
  auto& mi = const_cast<qlten::QLTensor<ElemT, QNT>&>(input);
  DeviceView<ElemT, QNT> vi(mi, true), vo(out, false);
  check(qltg_transpose(ctx.get(), &dt.d, vi.get(), perm.data(), vo.get(), nullptr));
  detail::sync_or_throw("axis move failed");
  vo.sync_back();
}

}  // namespace dmrg

}  // namespace qlten_gb300

#endif  // QLTEN_GB300_H_
