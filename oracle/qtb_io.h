// Minimal named-array container ("QTB1") used to move test vectors between the C++
// reference driver, the C++ CPU restatement and Python. Test infrastructure only.
//
// File = "QTB1" then records until EOF:
//   u32 name_len, name bytes, u8 dtype (0 f64, 1 i64, 2 i32, 3 u8), u32 ndim,
//   u64 shape[ndim], raw little-endian data.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace qtb {

class Writer {
 public:
  explicit Writer(const std::string& path) {
    f_ = std::fopen(path.c_str(), "wb");
    if (!f_) throw std::runtime_error("qtb: cannot open " + path);
    std::fwrite("QTB1", 1, 4, f_);
  }
  ~Writer() { if (f_) std::fclose(f_); }
  void put(const std::string& name, uint8_t dtype, const std::vector<uint64_t>& shape,
           const void* data, size_t elem_bytes) {
    uint32_t nl = (uint32_t)name.size();
    std::fwrite(&nl, 4, 1, f_);
    std::fwrite(name.data(), 1, nl, f_);
    std::fwrite(&dtype, 1, 1, f_);
    uint32_t nd = (uint32_t)shape.size();
    std::fwrite(&nd, 4, 1, f_);
    size_t n = 1;
    for (auto s : shape) { std::fwrite(&s, 8, 1, f_); n *= s; }
    if (n) std::fwrite(data, elem_bytes, n, f_);
  }
  void f64(const std::string& name, const std::vector<double>& v) {
    put(name, 0, {v.size()}, v.data(), 8);
  }
  void i64(const std::string& name, const std::vector<int64_t>& v) {
    put(name, 1, {v.size()}, v.data(), 8);
  }
  void i32(const std::string& name, const std::vector<int32_t>& v) {
    put(name, 2, {v.size()}, v.data(), 4);
  }
  void scalar_f64(const std::string& name, double x) { put(name, 0, {1}, &x, 8); }
  void scalar_i64(const std::string& name, int64_t x) { put(name, 1, {1}, &x, 8); }

 private:
  FILE* f_ = nullptr;
};

}  // namespace qtb
