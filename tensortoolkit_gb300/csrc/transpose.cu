// Batched block permutation: one launch permutes every block of a tensor.
//
// Replaces the reference's per-block hp_numeric::TensorTranspose (HPTT plan + execute on
// the CPU, a cuTENSOR plan / permute / destroy per block on the GPU;
// framework/hp_numeric/ten_trans.h:56-114, :245-349) and the ±1 block sign of
// BlockSparseDataTensor::Transpose (global_operations.h:393-441).
//
// Per block, unit dims are squeezed and destination-adjacent dims that are also adjacent
// in the source are merged. If the innermost destination dim is also innermost in the
// source, the block is a set of contiguous runs copied with 16-byte vector accesses;
// otherwise 32 x 32 tiles over (source-innermost dim p, destination-innermost dim q) are
// staged through shared memory so both the read (along p) and the write (along q) are
// coalesced. The sign multiply is exact (+-1).
#include <algorithm>
#include <mutex>
#include <string>

#include "ctrct.h"

namespace qltg {
namespace {

constexpr int kTile = 32;
constexpr int kRunChunk = 1024;   // elements per copy-mode work item

template <typename T>
__device__ __forceinline__ T mul_sign(T x, double s);
template <>
__device__ __forceinline__ double mul_sign<double>(double x, double s) { return x * s; }
template <>
__device__ __forceinline__ double2 mul_sign<double2>(double2 x, double s) { return make_double2(x.x * s, x.y * s); }

template <typename T>
__global__ void __launch_bounds__(256) k_permute(const PermDesc* __restrict__ descs, int nd, int64_t ntiles,
                                                 const T* __restrict__ src, T* __restrict__ dst) {
  __shared__ T tile[kTile][kTile + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    // locate the block owning global tile t
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (descs[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    const PermDesc& d = descs[lo];
    int64_t local = t - d.tile_begin;
    const int r = d.rank;
    const int q = r - 1;
    const double sign = d.sign;
    if (r == 0) {   // single element
      if (threadIdx.x == 0) dst[d.dst_off] = mul_sign(src[d.src_off], sign);
      continue;
    }
    // destination strides
    int64_t dstride[kMaxRank];
    dstride[r - 1] = 1;
    for (int i = r - 2; i >= 0; --i) dstride[i] = dstride[i + 1] * d.dims[i + 1];
    if (d.p < 0) {
      // gather mode (small inner dims): 1024 consecutive destination elements per work item,
      // each thread decodes its source offset; writes coalesced, reads in short runs
      // block sizes are below 2^31 (checked on the host): 32-bit index arithmetic
      const uint32_t total = (uint32_t)d.nouter;   // block size for this mode
      const uint32_t e0 = (uint32_t)local * kRunChunk;
      const uint32_t e1 = min(e0 + (uint32_t)kRunChunk, total);
      for (uint32_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        uint32_t rem = e;
        int64_t soff = 0;
        for (int i = r - 1; i >= 0; --i) {
          const uint32_t di = (uint32_t)d.dims[i];
          const uint32_t q = rem / di;
          soff += (int64_t)(rem - q * di) * d.sstride[i];
          rem = q;
        }
        dst[d.dst_off + e] = mul_sign(src[d.src_off + soff], sign);
      }
      continue;
    }
    if (d.p == q) {
      // copy mode: innermost run of length dims[q] contiguous on both sides
      const uint32_t chunks_per_run = ((uint32_t)d.dims[q] + kRunChunk - 1) / kRunChunk;
      const uint32_t run = (uint32_t)local / chunks_per_run;
      const int64_t c0 = (int64_t)((uint32_t)local - run * chunks_per_run) * kRunChunk;
      uint32_t rem = run;
      int64_t soff = 0, doff = 0;
      for (int i = r - 2; i >= 0; --i) {
        const uint32_t di = (uint32_t)d.dims[i];
        const uint32_t qq = rem / di;
        const uint32_t x = rem - qq * di;
        rem = qq;
        soff += (int64_t)x * d.sstride[i];
        doff += (int64_t)x * dstride[i];
      }
      const T* s = src + d.src_off + soff;
      T* o = dst + d.dst_off + doff;
      const int64_t n = min((int64_t)kRunChunk, (int64_t)d.dims[q] - c0);
      if (sizeof(T) == 8 && ((((uintptr_t)(s + c0)) | ((uintptr_t)(o + c0))) & 15) == 0) {
        const int64_t n2 = n >> 1;
        const double2* s2 = reinterpret_cast<const double2*>(s + c0);
        double2* o2 = reinterpret_cast<double2*>(o + c0);
        for (int64_t e = threadIdx.x; e < n2; e += blockDim.x) {
          double2 v = __ldg(s2 + e);
          v.x *= sign; v.y *= sign;
          o2[e] = v;
        }
        if ((n & 1) && threadIdx.x == 0) o[c0 + n - 1] = mul_sign(s[c0 + n - 1], sign);
      } else {
        for (int64_t e = threadIdx.x; e < n; e += blockDim.x) o[c0 + e] = mul_sign(s[c0 + e], sign);
      }
      continue;
    }
    // tile mode over (p, q)
    const uint32_t per_outer = (uint32_t)d.tiles_p * (uint32_t)d.tiles_q;
    const uint32_t outer = (uint32_t)local / per_outer;
    const uint32_t tt = (uint32_t)local - outer * per_outer;
    const uint32_t tq = tt / (uint32_t)d.tiles_q;
    const int64_t p0 = (int64_t)tq * kTile, q0 = (int64_t)(tt - tq * (uint32_t)d.tiles_q) * kTile;
    uint32_t rem = outer;
    int64_t soff = 0, doff = 0;
    for (int i = r - 1; i >= 0; --i) {
      if (i == d.p || i == q) continue;
      const uint32_t di = (uint32_t)d.dims[i];
      const uint32_t qq = rem / di;
      const uint32_t x = rem - qq * di;
      rem = qq;
      soff += (int64_t)x * d.sstride[i];
      doff += (int64_t)x * dstride[i];
    }
    const T* s = src + d.src_off + soff;
    T* o = dst + d.dst_off + doff;
    const int64_t np_ = d.dims[d.p], nq = d.dims[q];
    // read: threads along p (stride 1 in the source)
    for (int j = ty; j < kTile; j += 8) {
      const int64_t pi = p0 + tx, qi = q0 + j;
      if (pi < np_ && qi < nq) tile[j][tx] = __ldg(s + pi + qi * d.sstride[q]);
    }
    __syncthreads();
    // write: threads along q (stride 1 in the destination)
    for (int j = ty; j < kTile; j += 8) {
      const int64_t qi = q0 + tx, pi = p0 + j;
      if (pi < np_ && qi < nq) o[qi + pi * dstride[d.p]] = mul_sign(tile[tx][j], sign);
    }
    __syncthreads();
  }
}

}  // namespace

void TransposeList::describe(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
                             const std::vector<int64_t>* dst_offsets) {
  host.clear();
  ntiles = 0;
  const int r = t.rank;
  for (int64_t b = 0; b < t.nblk; ++b) {
    PermDesc d{};
    d.src_off = t.offsets[b];
    d.dst_off = dst_offsets ? (*dst_offsets)[b] : t.offsets[b];
    d.sign = signs.empty() ? 1.0 : signs[b];
    int64_t sstr[kMaxRank];
    sstr[r - 1] = 1;
    for (int i = r - 2; i >= 0; --i) sstr[i] = sstr[i + 1] * t.dim(b, i + 1);
    // destination-order dims / strides, unit dims dropped
    int64_t dd[kMaxRank], ds[kMaxRank];
    int n = 0;
    for (int i = 0; i < r; ++i) {
      const int64_t dim = t.dim(b, order[i]);
      if (dim == 1) continue;
      dd[n] = dim;
      ds[n] = sstr[order[i]];
      ++n;
    }
    // merge destination neighbours that are source neighbours in the same order
    int m = 0;
    for (int i = 0; i < n; ++i) {
      if (m > 0 && ds[m - 1] == ds[i] * dd[i]) {
        dd[m - 1] *= dd[i];
        ds[m - 1] = ds[i];
      } else {
        dd[m] = dd[i];
        ds[m] = ds[i];
        ++m;
      }
    }
    d.rank = m;
    d.p = -1;
    for (int i = 0; i < m; ++i) {
      QLTG_CHECK(dd[i] < ((int64_t)1 << 31), QLTG_ERR_UNSUPPORTED, "block dimension above 2^31");
      d.dims[i] = (int32_t)dd[i];
      d.sstride[i] = ds[i];
      if (ds[i] == 1) d.p = i;
    }
    QLTG_CHECK(t.blk_size(b) < ((int64_t)1 << 31), QLTG_ERR_UNSUPPORTED, "block with 2^31 or more elements");
    int64_t tiles;
    if (m == 0) {
      d.p = 0;
      tiles = 1;
    } else if (d.p == m - 1) {
      const int64_t runs = t.blk_size(b) / dd[m - 1];
      tiles = runs * ((dd[m - 1] + kRunChunk - 1) / kRunChunk);
    } else if (d.p < 0 || dd[d.p] < 16 || dd[m - 1] < 16) {
      // inner dims too short for 32 x 32 tiles: destination-ordered gather
      d.p = -1;
      d.nouter = t.blk_size(b);
      tiles = (d.nouter + kRunChunk - 1) / kRunChunk;
    } else {
      d.tiles_p = (int32_t)((dd[d.p] + kTile - 1) / kTile);
      d.tiles_q = (int32_t)((dd[m - 1] + kTile - 1) / kTile);
      d.nouter = t.blk_size(b) / (dd[d.p] * dd[m - 1]);
      tiles = d.nouter * d.tiles_p * d.tiles_q;
    }
    d.tile_begin = ntiles;
    ntiles += tiles;
    host.push_back(d);
  }
  nblocks = (int64_t)host.size();
}

void TransposeList::build(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
                          const std::vector<int64_t>* dst_offsets, cudaStream_t s) {
  describe(t, order, signs, dst_offsets);
  dev = upload(host, s);
}

void TransposeList::launch(const void* src, void* dst, int elem_bytes, cudaStream_t s) const {
  if (ntiles == 0) return;
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, 152 * 8);
  if (elem_bytes == 8)
    k_permute<double><<<grid, 256, 0, s>>>(dev.as<PermDesc>(), (int)nblocks, ntiles, static_cast<const double*>(src),
                                           static_cast<double*>(dst));
  else
    k_permute<double2><<<grid, 256, 0, s>>>(dev.as<PermDesc>(), (int)nblocks, ntiles,
                                            static_cast<const double2*>(src), static_cast<double2*>(dst));
  QLTG_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Allocation-free variant (qltg_transpose_noalloc). Some callers cannot allocate device
// memory while they run - a DMRG sweep driven from inside another library's CUDA-graph
// capture or memory-pool budget, or a host thread that must not take the allocator's
// locks - so the per-call permutation work list lives in this fixed device table instead
// of a fresh cudaMalloc. Every GPU that loads the library holds the table (about 600 KB)
// until the process exits. All calls share it and it keeps the last call's descriptors, so
// calls that overlap on the GPU (on different streams or devices' queues at once) race;
// each call waits for its own kernel before returning.
namespace {

__device__ __align__(256) PermDesc g_noalloc_perm[kNoAllocPermBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
PermDesc* g_noalloc_addr[kMaxDevices] = {};

// Device address of the table for `device`, looked up once per device with that device
// current (host code may not use the symbol itself as a device pointer).
PermDesc* noalloc_table(int device) {
  QLTG_CHECK(device >= 0 && device < kMaxDevices, QLTG_ERR_UNSUPPORTED, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    QLTG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_perm));
    g_noalloc_addr[device] = static_cast<PermDesc*>(p);
  }
  return g_noalloc_addr[device];
}

}  // namespace

void launch_permute_noalloc(int device, const TransposeList& tl, const void* src, void* dst, int elem_bytes,
                            cudaStream_t s) {
  QLTG_CHECK(tl.nblocks <= kNoAllocPermBlocks, QLTG_ERR_INVALID,
             "qltg_transpose_noalloc: tensor has " + std::to_string(tl.nblocks) + " blocks, the fixed table holds " +
                 std::to_string(kNoAllocPermBlocks));
  PermDesc* table = noalloc_table(device);
  if (tl.ntiles == 0) return;
  QLTG_CUDA(cudaMemcpyAsync(table, tl.host.data(), tl.host.size() * sizeof(PermDesc), cudaMemcpyHostToDevice, s));
  const unsigned grid = (unsigned)std::min<int64_t>(tl.ntiles, 152 * 8);
  if (elem_bytes == 8)
    k_permute<double><<<grid, 256, 0, s>>>(table, (int)tl.nblocks, tl.ntiles, static_cast<const double*>(src),
                                           static_cast<double*>(dst));
  else
    k_permute<double2><<<grid, 256, 0, s>>>(table, (int)tl.nblocks, tl.ntiles, static_cast<const double2*>(src),
                                            static_cast<double2*>(dst));
  QLTG_CUDA(cudaGetLastError());
  // the descriptors were copied from this call's host memory and the table is shared:
  // finish before returning
  QLTG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace qltg
