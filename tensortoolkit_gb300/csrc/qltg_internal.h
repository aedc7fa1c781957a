// Internal definitions shared by the translation units of libqltg.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/qltg.h"

namespace qltg {

constexpr int kMaxRank = 8;

// ------------------------------------------------------------------ errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define QLTG_CHECK(cond, code, msg)                                  \
  do {                                                               \
    if (!(cond)) throw ::qltg::Error((code), (msg));                 \
  } while (0)

#define QLTG_CUDA(call)                                                                     \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      (void)cudaGetLastError();                                                             \
      throw ::qltg::Error(e_ == cudaErrorMemoryAllocation ? QLTG_ERR_OOM : QLTG_ERR_CUDA,   \
                          std::string(#call) + ": " + cudaGetErrorString(e_));              \
    }                                                                                       \
  } while (0)

// Run `body` and translate exceptions into a status code plus the thread-local message.
template <typename F>
int guarded(F&& body) {
  try {
    body();
    return QLTG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return QLTG_ERR_OOM;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return QLTG_ERR_INVALID;
  }
}

// ------------------------------------------------------------------ device memory
class DevBuf {
 public:
  DevBuf() = default;
  explicit DevBuf(size_t bytes) { alloc(bytes); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { release(); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
    return *this;
  }
  void alloc(size_t bytes) {
    release();
    if (bytes) QLTG_CUDA(cudaMalloc(&p_, bytes));
    n_ = bytes;
  }
  void release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
  }
  template <typename T> T* as() const { return static_cast<T*>(p_); }
  void* get() const { return p_; }
  size_t bytes() const { return n_; }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

// Streaming multiprocessors of the current device (grid sizing for kernels launched without
// a context at hand).
inline int current_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

template <typename T>
DevBuf upload(const std::vector<T>& v, cudaStream_t s) {
  DevBuf b(v.size() * sizeof(T));
  if (!v.empty()) QLTG_CUDA(cudaMemcpyAsync(b.get(), v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return b;
}

// ------------------------------------------------------------------ tensor metadata
// Validated host copy of a qltg_tensor_desc.
struct Meta {
  int rank = 0;
  int dtype = QLTG_F64;
  int ncomp = 1;
  int parity_comp = -1;
  std::vector<int32_t> dirs;
  std::vector<std::vector<int32_t>> qns;   // per leg, nsct * ncomp
  std::vector<std::vector<int64_t>> dims;  // per leg
  std::vector<int64_t> coords;             // nblk * rank
  std::vector<int64_t> offsets;            // nblk
  int64_t nblk = 0;
  int64_t size = 0;

  int64_t nsct(int l) const { return (int64_t)dims[l].size(); }
  int64_t dim(int64_t b, int l) const { return dims[l][coords[b * rank + l]]; }
  int64_t blk_size(int64_t b) const {
    int64_t s = 1;
    for (int l = 0; l < rank; ++l) s *= dim(b, l);
    return s;
  }
  bool parity(int l, int64_t sct) const {
    return parity_comp >= 0 && (qns[l][sct * ncomp + parity_comp] % 2) != 0;
  }
  size_t elem_bytes() const { return dtype == QLTG_C128 ? 16 : 8; }
  uint64_t blk_idx(const int64_t* c) const {
    uint64_t idx = 0;
    for (int l = 0; l < rank; ++l) idx = idx * (uint64_t)dims[l].size() + (uint64_t)c[l];
    return idx;
  }
  void refresh_offsets();
  // Fill a caller-visible descriptor that points into this object.
  void export_arrays(int32_t* dirs, int32_t* nsct, int32_t* qns, int64_t* dims, int64_t* coords,
                     int64_t* offsets) const;
};

Meta meta_from_desc(const qltg_tensor_desc* d);
bool same_leg(const Meta& a, int la, const Meta& b, int lb);        // identical space
bool inverse_leg(const Meta& a, int la, const Meta& b, int lb);     // same sectors, opposite dir
bool same_indexes(const Meta& x, const Meta& y);                    // element type and every leg

}  // namespace qltg

struct qltg_ctx {
  int device = 0;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
};
