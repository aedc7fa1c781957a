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
 *
 * With the reference built for the GPU (USE_GPU) the QLTensor raw buffers already live in
 * device memory and are passed straight through. With the CPU build they are staged
 * through device buffers (one copy in, one copy out per call).
 *
 * Supported quantum numbers: U1QN, U1U1QN, fU1QN, fU1U1QN (integer-additive components;
 * the fermionic ones take their parity from the particle-number component).
 */
#ifndef QLTEN_GB300_H_
#define QLTEN_GB300_H_

#include <cuda_runtime.h>

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
      if (copy_in) cudaMemcpy(ptr_, bsdt.GetActualRawDataPtr(), bytes_, cudaMemcpyHostToDevice);
    }
#endif
  }
  ~DeviceView() {
#ifndef USE_GPU
    if (ptr_) cudaFree(ptr_);
#endif
  }
  void* get() const { return ptr_; }
  void sync_back() {
#ifndef USE_GPU
    if (bytes_) cudaMemcpy(t_.GetBlkSparDataTen().GetActualRawDataPtr(), ptr_, bytes_, cudaMemcpyDeviceToHost);
#endif
  }

 private:
  qlten::QLTensor<ElemT, QNT>& t_;
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

class Context {
 public:
  explicit Context(int device = 0) { check(qltg_create(device, &ctx_)); }
  ~Context() { qltg_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  qltg_ctx* get() const { return ctx_; }

 private:
  qltg_ctx* ctx_ = nullptr;
};

// ------------------------------------------------------------------ Contract
template <typename ElemT, typename QNT>
void Contract(const qlten::QLTensor<ElemT, QNT>* pa, const qlten::QLTensor<ElemT, QNT>* pb,
              const std::vector<std::vector<size_t>>& axes_set, qlten::QLTensor<ElemT, QNT>* pc,
              const Context& ctx, int mode = QLTG_MODE_FP64) {
  Desc<ElemT, QNT> da(*pa), db(*pb);
  std::vector<int64_t> axa(axes_set[0].begin(), axes_set[0].end()), axb(axes_set[1].begin(), axes_set[1].end());
  qltg_ctrct_plan* plan = nullptr;
  check(qltg_ctrct_plan_create(ctx.get(), &da.d, &db.d, axa.data(), axb.data(), (int32_t)axa.size(), &plan));
  try {
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
    check(qltg_ctrct_exec(plan, va.get(), vb.get(), vc.get(), mode, nullptr));
    if (cudaStreamSynchronize(nullptr) != cudaSuccess) throw std::runtime_error("qlten_gb300: contraction failed");
    vc.sync_back();
  } catch (...) {
    qltg_ctrct_plan_destroy(plan);
    throw;
  }
  qltg_ctrct_plan_destroy(plan);
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

}  // namespace qlten_gb300

#endif  // QLTEN_GB300_H_
