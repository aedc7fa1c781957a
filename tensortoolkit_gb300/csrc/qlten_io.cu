// .qlten stream I/O: the reference's QLTensor serialisation, read into device memory through
// a pinned staging buffer and written from device or host memory.
//
// Format (text numbers, one per line, then the raw buffer):
//   rank
//   per index (qltensor/index.h:170-188):
//     sector count
//     per sector (qltensor/qnsct.h:106-115): the quantum number (U1QN: value, hash;
//       U1U1QN / fU1U1QN: two values, hash; special_qn/u1qn.h:126-133, u1u1qn.h), the
//       degeneracy, the sector hash
//     direction (IN = -1, OUT = 1), dimension, index hash
//   block count, then every block's coordinates, blocks in ascending block index
//     (qltensor/blk_spar_data_ten/blk_spar_data_ten.h:791-830)
//   one line break, the raw buffer (FP64 or interleaved complex128), a line break
//     (raw_data_operations.h:583-640). A scalar stores no blocks and one value.
// Hashes (checked on read, reproduced on write, so files round-trip with the reference):
//   U1QN: rotate-left-31 of the value as size_t (special_qn/u1qn.h:139-153)
//   U1U1QN / fU1U1QN: h = (v0 + 2^30) + (v1 + 2^30) 2^31, rotate-left-10 (u1u1qn.h)
//   sector: QN hash ^ degeneracy (qnsct.h:138)
//   index: xxHash-style fold of the sector hashes (framework/vec_hash.h:25-36) ^ direction
//     as size_t (index.h:225-228)
#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>

#include "qltg_internal.h"

namespace qltg {
namespace {

constexpr uint64_t kP1 = 11400714785074694791ULL, kP2 = 14029467366897019727ULL, kP5 = 2870177450012600261ULL;
inline uint64_t rotl(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

uint64_t qn_hash(const int32_t* q, int ncomp) {
  if (ncomp == 1) return rotl((uint64_t)(int64_t)q[0], 31);
  const uint64_t s = 1ull << 30;
  const uint64_t h = ((uint64_t)(int64_t)q[0] + s) + ((uint64_t)(int64_t)q[1] + s) * (2 * s);
  return rotl(h, 10);
}

uint64_t index_hash(const std::vector<uint64_t>& sct, int dir_ref) {
  uint64_t h = kP5;
  for (uint64_t x : sct) {
    h += x * kP2;
    h = rotl(h, 31);
    h *= kP1;
  }
  h += (uint64_t)sct.size() ^ kP5;
  return h ^ (uint64_t)(int64_t)dir_ref;
}

int ref_dir(int32_t d) { return d == QLTG_IN ? -1 : 1; }

template <typename T>
T read_num(std::istream& is, const char* what) {
  T v;
  is >> v;
  QLTG_CHECK(!is.fail(), QLTG_ERR_INVALID, std::string(".qlten: cannot read ") + what);
  return v;
}

}  // namespace
}  // namespace qltg

struct qltg_qlten_file {
  qltg::Meta m;
  std::string path;
  std::streamoff data_pos = 0;   // first byte of the raw buffer
};

using namespace qltg;

extern "C" {

int qltg_qlten_open(const char* path, int32_t qn_ncomp, int32_t parity_comp, int32_t elem_type,
                    qltg_qlten_file** file) {
  return guarded([&] {
    QLTG_CHECK(path && file, QLTG_ERR_INVALID, "null path or file out-pointer");
    QLTG_CHECK(qn_ncomp == 1 || qn_ncomp == 2, QLTG_ERR_UNSUPPORTED,
               ".qlten: quantum numbers with 1 (U1QN) or 2 (U1U1QN, fU1U1QN) components");
    QLTG_CHECK(parity_comp >= -1 && parity_comp < qn_ncomp, QLTG_ERR_INVALID, "parity_comp out of range");
    QLTG_CHECK(elem_type == QLTG_F64 || elem_type == QLTG_C128, QLTG_ERR_INVALID, "unknown element type");
    std::ifstream is(path, std::ios::binary);
    QLTG_CHECK(is.good(), QLTG_ERR_INVALID, std::string(".qlten: cannot open ") + path);
    auto f = std::make_unique<qltg_qlten_file>();
    f->path = path;
    Meta& m = f->m;
    m.dtype = elem_type;
    m.ncomp = qn_ncomp;
    m.parity_comp = parity_comp;
    m.rank = (int)read_num<int64_t>(is, "rank");
    QLTG_CHECK(m.rank >= 0 && m.rank <= kMaxRank, QLTG_ERR_UNSUPPORTED, ".qlten: rank outside 0..8");
    for (int l = 0; l < m.rank; ++l) {
      const int64_t ns = read_num<int64_t>(is, "sector count");
      QLTG_CHECK(ns >= 1 && ns < (1 << 24), QLTG_ERR_INVALID, ".qlten: bad sector count");
      std::vector<int32_t> qns;
      std::vector<int64_t> dims;
      std::vector<uint64_t> sh;
      int64_t dim_sum = 0;
      for (int64_t k = 0; k < ns; ++k) {
        int32_t q[2];
        for (int c = 0; c < qn_ncomp; ++c) q[c] = (int32_t)read_num<int64_t>(is, "quantum number");
        const uint64_t h = read_num<uint64_t>(is, "quantum number hash");
        QLTG_CHECK(h == qn_hash(q, qn_ncomp), QLTG_ERR_INVALID,
                   ".qlten: quantum number hash mismatch (wrong quantum number type?)");
        const int64_t dg = read_num<int64_t>(is, "degeneracy");
        QLTG_CHECK(dg >= 1, QLTG_ERR_INVALID, ".qlten: bad degeneracy");
        const uint64_t hs = read_num<uint64_t>(is, "sector hash");
        QLTG_CHECK(hs == (h ^ (uint64_t)dg), QLTG_ERR_INVALID, ".qlten: sector hash mismatch");
        qns.insert(qns.end(), q, q + qn_ncomp);
        dims.push_back(dg);
        sh.push_back(hs);
        dim_sum += dg;
      }
      const int dir = (int)read_num<int64_t>(is, "direction");
      QLTG_CHECK(dir == -1 || dir == 1, QLTG_ERR_INVALID, ".qlten: index direction must be IN or OUT");
      const int64_t dim = read_num<int64_t>(is, "dimension");
      QLTG_CHECK(dim == dim_sum, QLTG_ERR_INVALID, ".qlten: index dimension mismatch");
      const uint64_t hi = read_num<uint64_t>(is, "index hash");
      QLTG_CHECK(hi == index_hash(sh, dir), QLTG_ERR_INVALID, ".qlten: index hash mismatch");
      m.dirs.push_back(dir == -1 ? QLTG_IN : QLTG_OUT);
      m.qns.push_back(std::move(qns));
      m.dims.push_back(std::move(dims));
    }
    const int64_t nb = read_num<int64_t>(is, "block count");
    QLTG_CHECK(nb >= 0, QLTG_ERR_INVALID, ".qlten: bad block count");
    m.coords.resize((size_t)nb * m.rank);
    for (int64_t b = 0; b < nb; ++b)
      for (int l = 0; l < m.rank; ++l) {
        const int64_t c = read_num<int64_t>(is, "block coordinate");
        QLTG_CHECK(c >= 0 && c < m.nsct(l), QLTG_ERR_INVALID, ".qlten: block coordinate out of range");
        m.coords[(size_t)b * m.rank + l] = c;
      }
    for (int64_t b = 1; b < nb; ++b)
      QLTG_CHECK(m.blk_idx(&m.coords[(b - 1) * m.rank]) < m.blk_idx(&m.coords[b * m.rank]), QLTG_ERR_INVALID,
                 ".qlten: blocks not in ascending block index order");
    if (m.rank == 0) {
      QLTG_CHECK(nb == 0, QLTG_ERR_INVALID, ".qlten: a scalar stores no blocks");
      m.nblk = 1;                 // one value
      m.refresh_offsets();
    } else {
      m.nblk = nb;
      m.refresh_offsets();
    }
    is.seekg(1, std::ios::cur);   // the line break before the raw buffer
    f->data_pos = is.tellg();
    is.seekg(0, std::ios::end);
    const std::streamoff end = is.tellg();
    QLTG_CHECK(end - f->data_pos >= (std::streamoff)(m.size * m.elem_bytes()), QLTG_ERR_INVALID,
               ".qlten: file shorter than its raw buffer");
    *file = f.release();
  });
}

int qltg_qlten_info(const qltg_qlten_file* f, int32_t* rank, int64_t* total_sectors, int64_t* nblk, int64_t* size) {
  return guarded([&] {
    QLTG_CHECK(f, QLTG_ERR_INVALID, "null file");
    int64_t ts = 0;
    for (int l = 0; l < f->m.rank; ++l) ts += f->m.nsct(l);
    if (rank) *rank = f->m.rank;
    if (total_sectors) *total_sectors = ts;
    if (nblk) *nblk = f->m.rank ? f->m.nblk : 1;
    if (size) *size = f->m.size;
  });
}

int qltg_qlten_meta(const qltg_qlten_file* f, int32_t* dirs, int32_t* nsct, int32_t* qns, int64_t* dims,
                    int64_t* coords) {
  return guarded([&] {
    QLTG_CHECK(f, QLTG_ERR_INVALID, "null file");
    f->m.export_arrays(dirs, nsct, qns, dims, coords, nullptr);
  });
}

int qltg_qlten_read_data(qltg_qlten_file* f, void* dst, int32_t dst_is_device, void* stream) {
  return guarded([&] {
    QLTG_CHECK(f && dst, QLTG_ERR_INVALID, "null file or destination");
    const size_t bytes = (size_t)f->m.size * f->m.elem_bytes();
    if (!bytes) return;
    std::ifstream is(f->path, std::ios::binary);
    QLTG_CHECK(is.good(), QLTG_ERR_INVALID, ".qlten: cannot reopen " + f->path);
    is.seekg(f->data_pos);
    if (!dst_is_device) {
      is.read(static_cast<char*>(dst), (std::streamsize)bytes);
      QLTG_CHECK((size_t)is.gcount() == bytes, QLTG_ERR_INVALID, ".qlten: short raw buffer");
      return;
    }
    // device-direct: file -> pinned staging -> HBM (asynchronous copy, then released)
    void* pinned = nullptr;
    QLTG_CUDA(cudaMallocHost(&pinned, bytes));
    std::unique_ptr<void, void (*)(void*)> guard(pinned, [](void* p) { cudaFreeHost(p); });
    is.read(static_cast<char*>(pinned), (std::streamsize)bytes);
    QLTG_CHECK((size_t)is.gcount() == bytes, QLTG_ERR_INVALID, ".qlten: short raw buffer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    QLTG_CUDA(cudaMemcpyAsync(dst, pinned, bytes, cudaMemcpyHostToDevice, s));
    QLTG_CUDA(cudaStreamSynchronize(s));
  });
}

int qltg_qlten_close(qltg_qlten_file* f) {
  delete f;
  return QLTG_OK;
}

int qltg_qlten_write(const char* path, const qltg_tensor_desc* t, const void* data, int32_t data_is_device,
                     void* stream) {
  return guarded([&] {
    QLTG_CHECK(path, QLTG_ERR_INVALID, "null path");
    const Meta m = meta_from_desc(t);
    QLTG_CHECK(m.ncomp == 1 || m.ncomp == 2, QLTG_ERR_UNSUPPORTED,
               ".qlten: quantum numbers with 1 (U1QN) or 2 (U1U1QN, fU1U1QN) components");
    const int64_t nvals = m.rank ? m.size : 1;   // a scalar always stores one value
    const size_t bytes = (size_t)nvals * m.elem_bytes();
    std::vector<char> host(bytes, 0);
    if (m.rank == 0 && m.size == 0) {
      // empty scalar: the reference writes a default-constructed value
    } else if (bytes) {
      QLTG_CHECK(data, QLTG_ERR_INVALID, "null raw buffer");
      if (data_is_device) {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        QLTG_CUDA(cudaMemcpyAsync(host.data(), data, bytes, cudaMemcpyDeviceToHost, s));
        QLTG_CUDA(cudaStreamSynchronize(s));
      } else {
        std::memcpy(host.data(), data, bytes);
      }
    }
    std::ostringstream os;
    os << m.rank << "\n";
    for (int l = 0; l < m.rank; ++l) {
      os << m.nsct(l) << "\n";
      std::vector<uint64_t> sh;
      for (int64_t k = 0; k < m.nsct(l); ++k) {
        const int32_t* q = &m.qns[l][k * m.ncomp];
        const uint64_t h = qn_hash(q, m.ncomp);
        for (int c = 0; c < m.ncomp; ++c) os << q[c] << "\n";
        os << h << "\n";
        const uint64_t hs = h ^ (uint64_t)m.dims[l][k];
        os << m.dims[l][k] << "\n" << hs << "\n";
        sh.push_back(hs);
      }
      int64_t dim = 0;
      for (auto d : m.dims[l]) dim += d;
      const int dir = ref_dir(m.dirs[l]);
      os << dir << "\n" << dim << "\n" << index_hash(sh, dir) << "\n";
    }
    os << (m.rank ? m.nblk : 0) << "\n";
    for (int64_t b = 0; m.rank && b < m.nblk; ++b)
      for (int l = 0; l < m.rank; ++l) os << m.coords[(size_t)b * m.rank + l] << "\n";
    std::ofstream of(path, std::ios::binary | std::ios::trunc);
    QLTG_CHECK(of.good(), QLTG_ERR_INVALID, std::string(".qlten: cannot create ") + path);
    const std::string head = os.str();
    of.write(head.data(), (std::streamsize)head.size());
    of.write(host.data(), (std::streamsize)host.size());
    of << "\n";
    QLTG_CHECK(of.good(), QLTG_ERR_INVALID, std::string(".qlten: write failed: ") + path);
  });
}

}  // extern "C"
