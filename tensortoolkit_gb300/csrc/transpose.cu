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
// otherwise tiles over (source-innermost dim p, destination-innermost dim q) are staged
// through shared memory so both the read (along p) and the write (along q) are coalesced.
// Tiles are 32 x 32, or Tp x Tq (x Tu of one batched outer dim) up to 32 KB of data when one
// of the two dims is short (an inner dim of 4 elements gets 4 x 256 tiles, whose reads and
// writes are still long contiguous runs). A CTA reads its next tile into a second shared
// buffer (cp.async, no staging registers) while it writes the current one out, so a tile's
// worth of loads is always in flight. Only blocks whose two inner dims are both short fall
// back to a destination-ordered gather. The +-1 block sign is applied by flipping the sign
// bit (no floating-point multiply). Each CTA takes a contiguous range of work items, so it
// looks up its first block once and then walks forward.
#include <algorithm>
#include <mutex>
#include <string>

#include "ctrct.h"

namespace qltg {
namespace {

constexpr int kTile = 32;
constexpr int kTileMax = 4096;    // elements per batched tile (Tp * Tq * Tu), 8-byte elements
constexpr int kRunChunk = 4096;   // elements per copy-mode / gather-mode work item
constexpr int kPermThreads = 256;
constexpr int kLoadBatch = 8;     // copy-mode loads issued per thread before storing

// Tile budget in elements: the same 32 KB of data per tile for real and complex elements.
__host__ __device__ constexpr int tile_budget(int elem_bytes) { return elem_bytes == 16 ? kTileMax / 2 : kTileMax; }
// One tile buffer in elements: Tu planes of Tq rows of Tp + 1 (Tp >= 2): at most 1.5x the tile.
__host__ __device__ constexpr int tile_buf_elems(int elem_bytes) { return tile_budget(elem_bytes) * 3 / 2; }

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src));
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ double flip(double x, uint64_t m) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)m);
}
__device__ __forceinline__ double2 flip(double2 x, uint64_t m) { return make_double2(flip(x.x, m), flip(x.y, m)); }

// A tile-mode work item, decoded: a Tp x Tq x Tu tile over (p, q, u) (u: one outer dim batched
// so a tile holds up to the budget even when the inner dims are short).
template <typename T>
struct TileJob {
  const T* s;
  T* o;
  uint32_t sq, su, dp, du;
  int np, nq, ulim, ip0, iq0;
  int tp, tq, tu, lp, lq, lu, n;
  bool u_next;
  uint64_t sg;
};

__host__ __device__ inline bool is_tile_item(const PermDesc& d) { return d.rank > 0 && d.p >= 0 && d.p != d.rank - 1; }

template <typename T>
__device__ __forceinline__ TileJob<T> tile_job(const PermDesc& d, int64_t local, const T* src, T* dst) {
  TileJob<T> j;
  const int r = d.rank, q = r - 1;
  j.tp = d.tp;
  j.tq = d.tq;
  j.tu = d.tu;
  const uint32_t per_outer = (uint32_t)d.tiles_p * (uint32_t)d.tiles_q * (uint32_t)d.tiles_u;
  const uint32_t outer = (uint32_t)local / per_outer;
  uint32_t tt = (uint32_t)local - outer * per_outer;
  const uint32_t tui = tt / ((uint32_t)d.tiles_p * (uint32_t)d.tiles_q);
  tt -= tui * ((uint32_t)d.tiles_p * (uint32_t)d.tiles_q);
  const uint32_t tpi = tt / (uint32_t)d.tiles_q;
  j.ip0 = (int)(tpi * (uint32_t)j.tp);
  j.iq0 = (int)((tt - tpi * (uint32_t)d.tiles_q) * (uint32_t)j.tq);
  const int u0 = (int)(tui * (uint32_t)j.tu);
  uint32_t rem = outer, soff = 0, doff = 0, dstr = 1, dp = 0, du = 0;
  for (int i = r - 1; i >= 0; --i) {
    const uint32_t di = (uint32_t)d.dims[i];
    if (i == d.p) dp = dstr;
    if (i == d.u) du = dstr;
    if (i != d.p && i != q && i != d.u) {
      const uint32_t qq = rem / di;
      const uint32_t x = rem - qq * di;
      rem = qq;
      soff += x * (uint32_t)d.sstride[i];
      doff += x * dstr;
    }
    dstr *= di;
  }
  const int nu = d.u >= 0 ? d.dims[d.u] : 1;
  j.su = d.u >= 0 ? (uint32_t)d.sstride[d.u] : 0u;
  j.dp = dp;
  j.du = du;
  j.s = src + d.src_off + soff + (uint32_t)u0 * j.su;
  j.o = dst + d.dst_off + doff + (uint32_t)u0 * du;
  j.np = d.dims[d.p];
  j.nq = d.dims[q];
  j.sq = (uint32_t)d.sstride[q];
  j.lp = __ffs(j.tp) - 1;   // tile extents are powers of two
  j.lq = __ffs(j.tq) - 1;
  j.lu = __ffs(j.tu) - 1;
  j.n = j.tp * j.tq * j.tu;
  j.ulim = nu - u0;
  // write order: q fastest (stride 1 in the destination), then whichever of u and p has the
  // smaller destination stride (a short q dim with u next to it in the destination)
  j.u_next = d.u >= 0 && du < dp;
  j.sg = d.sign_mask;
  return j;
}

// read into a tile buffer: p fastest (stride 1 in the source), straight into shared memory
// (cp.async), so a whole tile is in flight per CTA without staging registers. With Tp <= the
// CTA size a thread keeps one column pi and walks the (q, u) rows of the tile, so the index
// arithmetic per element is a few integer operations.
template <typename T>
__device__ __forceinline__ void tile_loads(const TileJob<T>& j, T* buf) {
  const int row = j.tp + 1, plane = j.tq * row;
  if (j.tp <= kPermThreads) {
    const int pi = threadIdx.x & (j.tp - 1);
    if (j.ip0 + pi >= j.np) return;
    const T* sb = j.s + (uint32_t)(j.ip0 + pi);
    const int rstep = kPermThreads >> j.lp, nrows = j.tq * j.tu;
    for (int ri = threadIdx.x >> j.lp; ri < nrows; ri += rstep) {
      const int qi = ri & (j.tq - 1), ui = ri >> j.lq;
      if (j.iq0 + qi < j.nq && ui < j.ulim)
        cp_async_elem(buf + (ui * plane + qi * row + pi), sb + ((uint32_t)(j.iq0 + qi) * j.sq + (uint32_t)ui * j.su));
    }
    return;
  }
  for (int e = threadIdx.x; e < j.n; e += kPermThreads) {
    const int pi = e & (j.tp - 1), qi = (e >> j.lp) & (j.tq - 1), ui = e >> (j.lp + j.lq);
    if (j.ip0 + pi < j.np && j.iq0 + qi < j.nq && ui < j.ulim)
      cp_async_elem(buf + (ui * plane + qi * row + pi),
                    j.s + ((uint32_t)(j.ip0 + pi) + (uint32_t)(j.iq0 + qi) * j.sq + (uint32_t)ui * j.su));
  }
}

// write out of a tile buffer in the write order (q fastest, then u or p); with Tq <= the CTA
// size a thread keeps one q and walks the (p, u) columns
template <typename T>
__device__ __forceinline__ void tile_stores(const TileJob<T>& j, const T* buf) {
  const int row = j.tp + 1, plane = j.tq * row;
  if (j.tq <= kPermThreads) {
    const int qi = threadIdx.x & (j.tq - 1);
    if (j.iq0 + qi >= j.nq) return;
    T* ob = j.o + (uint32_t)(j.iq0 + qi);
    const int cstep = kPermThreads >> j.lq, ncols = j.tp * j.tu;
    for (int ci = threadIdx.x >> j.lq; ci < ncols; ci += cstep) {
      const int pi = j.u_next ? ci >> j.lu : ci & (j.tp - 1);
      const int ui = j.u_next ? ci & (j.tu - 1) : ci >> j.lp;
      if (j.ip0 + pi < j.np && ui < j.ulim)
        ob[(uint32_t)(j.ip0 + pi) * j.dp + (uint32_t)ui * j.du] = flip(buf[ui * plane + qi * row + pi], j.sg);
    }
    return;
  }
  for (int e = threadIdx.x; e < j.n; e += kPermThreads) {
    const int qi = e & (j.tq - 1);
    const int pi = j.u_next ? (e >> (j.lq + j.lu)) & (j.tp - 1) : (e >> j.lq) & (j.tp - 1);
    const int ui = j.u_next ? (e >> j.lq) & (j.tu - 1) : e >> (j.lp + j.lq);
    if (j.ip0 + pi < j.np && j.iq0 + qi < j.nq && ui < j.ulim)
      j.o[(uint32_t)(j.iq0 + qi) + (uint32_t)(j.ip0 + pi) * j.dp + (uint32_t)ui * j.du] =
          flip(buf[ui * plane + qi * row + pi], j.sg);
  }
}

template <typename T>
__global__ void __launch_bounds__(kPermThreads) k_permute(const PermDesc* __restrict__ descs, int nd, int64_t ntiles,
                                                          const T* __restrict__ src, T* __restrict__ dst) {
  // two tile buffers: Tu planes of Tq rows of Tp + 1 (Tp a power of two, so the row stride
  // is odd); tile t + 1 is read into one while tile t is written out of the other
  extern __shared__ __align__(16) uint8_t perm_smem[];
  T* const bufs = reinterpret_cast<T*>(perm_smem);
  constexpr int kBuf = tile_buf_elems((int)sizeof(T));
  const int64_t per = (ntiles + gridDim.x - 1) / gridDim.x;
  const int64_t t_begin = (int64_t)blockIdx.x * per, t_end = min(ntiles, t_begin + per);
  if (t_begin >= t_end) return;
  // the block owning the first work item; later items walk forward from it
  int lo = 0, hi = nd - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (descs[mid].tile_begin <= t_begin) lo = mid; else hi = mid - 1;
  }
  // the current block's descriptor, staged in shared memory when the walk reaches a new block
  __shared__ PermDesc sdesc;
  int cur = -1;
  int b = 0;              // the buffer of the current tile item
  bool pending = false;   // its loads were issued by the previous item
  // first work item of the next block, read from global memory only when the walk moves on
  constexpr int64_t kNone = 0x7FFFFFFFFFFFFFFFll;
  int64_t next_begin = lo + 1 < nd ? descs[lo + 1].tile_begin : kNone;
  for (int64_t t = t_begin; t < t_end; ++t) {
    while (t >= next_begin) {
      ++lo;
      next_begin = lo + 1 < nd ? descs[lo + 1].tile_begin : kNone;
    }
    if (lo != cur) {   // uniform across the CTA: every thread walks the same items
      __syncthreads();
      if (threadIdx.x == 0) sdesc = descs[lo];
      __syncthreads();
      cur = lo;
    }
    const PermDesc& d = sdesc;
    const int64_t local = t - d.tile_begin;
    const int r = d.rank;
    const int q = r - 1;
    const uint64_t sg = d.sign_mask;
    if (r == 0) {   // single element
      if (threadIdx.x == 0) dst[d.dst_off] = flip(src[d.src_off], sg);
      continue;
    }
    // Offsets inside a block are below 2^31 (checked on the host), so the index arithmetic
    // below is 32-bit; destination strides are running products (no per-thread stride array,
    // which kept the kernel at 128 registers).
    if (d.p < 0) {
      // gather mode (both inner dims short): 1024 consecutive destination elements per work
      // item, each thread decodes its source offset; block sizes are below 2^31 (checked on
      // the host), so the index arithmetic is 32-bit
      const uint32_t total = (uint32_t)d.nouter;
      const uint32_t e0 = (uint32_t)local * kRunChunk;
      const uint32_t e1 = min(e0 + (uint32_t)kRunChunk, total);
      for (uint32_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        uint32_t rem = e, soff = 0;
        for (int i = r - 1; i >= 0; --i) {
          const uint32_t di = (uint32_t)d.dims[i];
          const uint32_t qq = rem / di;
          soff += (rem - qq * di) * (uint32_t)d.sstride[i];
          rem = qq;
        }
        dst[d.dst_off + e] = flip(src[d.src_off + soff], sg);
      }
      continue;
    }
    if (d.p == q && d.tq > 1) {
      // copy mode with short runs: a work item is d.tq consecutive runs (of dims[q] elements,
      // contiguous on both sides). The runs' offsets are decoded once, one thread per run,
      // into shared memory (the tile buffers are idle: only tile items prefetch into them);
      // then the item's elements are copied as one flat range, kLoadBatch loads in flight
      // per thread before the stores.
      const uint32_t len = (uint32_t)d.dims[q];
      const uint32_t nruns = (uint32_t)(d.nouter);
      const uint32_t r0 = (uint32_t)local * (uint32_t)d.tq;
      const uint32_t nr = min(nruns, r0 + (uint32_t)d.tq) - r0;
      uint32_t* run_s = reinterpret_cast<uint32_t*>(perm_smem);
      uint32_t* run_d = run_s + nr;
      for (uint32_t j = threadIdx.x; j < nr; j += kPermThreads) {
        uint32_t rem = r0 + j, soff = 0, doff = 0, dstr = len;
        for (int i = r - 2; i >= 0; --i) {
          const uint32_t di = (uint32_t)d.dims[i];
          const uint32_t qq = rem / di;
          const uint32_t x = rem - qq * di;
          rem = qq;
          soff += x * (uint32_t)d.sstride[i];
          doff += x * dstr;
          dstr *= di;
        }
        run_s[j] = soff;
        run_d[j] = doff;
      }
      __syncthreads();
      const uint32_t total = nr * len;
      const float rlen = 1.0f / (float)len;
      const T* s = src + d.src_off;
      T* o = dst + d.dst_off;
      for (uint32_t e0 = threadIdx.x; e0 < total; e0 += kPermThreads * kLoadBatch) {
        T v[kLoadBatch];
        uint32_t at[kLoadBatch];
#pragma unroll
        for (int i = 0; i < kLoadBatch; ++i) {
          const uint32_t e = e0 + (uint32_t)i * kPermThreads;
          if (e < total) {
            // run = e / len: the float quotient, corrected to the exact one
            uint32_t run = (uint32_t)((float)e * rlen);
            if (run * len > e) --run;
            else if ((run + 1) * len <= e) ++run;
            const uint32_t off = e - run * len;
            v[i] = __ldg(s + run_s[run] + off);
            at[i] = run_d[run] + off;
          }
        }
#pragma unroll
        for (int i = 0; i < kLoadBatch; ++i) {
          const uint32_t e = e0 + (uint32_t)i * kPermThreads;
          if (e < total) o[at[i]] = flip(v[i], sg);
        }
      }
      __syncthreads();   // the run tables are rewritten by the next item
      continue;
    }
    if (d.p == q) {
      // copy mode: innermost run of length dims[q] contiguous on both sides
      const uint32_t chunks_per_run = ((uint32_t)d.dims[q] + kRunChunk - 1) / kRunChunk;
      const uint32_t run = (uint32_t)local / chunks_per_run;
      const int64_t c0 = (int64_t)((uint32_t)local - run * chunks_per_run) * kRunChunk;
      uint32_t rem = run, soff = 0, doff = 0, dstr = (uint32_t)d.dims[q];
      for (int i = r - 2; i >= 0; --i) {
        const uint32_t di = (uint32_t)d.dims[i];
        const uint32_t qq = rem / di;
        const uint32_t x = rem - qq * di;
        rem = qq;
        soff += x * (uint32_t)d.sstride[i];
        doff += x * dstr;
        dstr *= di;
      }
      const T* s = src + d.src_off + soff;
      T* o = dst + d.dst_off + doff;
      const int64_t n = min((int64_t)kRunChunk, (int64_t)d.dims[q] - c0);
      if (sizeof(T) == 8 && ((((uintptr_t)(s + c0)) | ((uintptr_t)(o + c0))) & 15) == 0) {
        // 16-byte vectors, kLoadBatch loads in flight per thread before the stores
        const int64_t n2 = n >> 1;
        const double2* s2 = reinterpret_cast<const double2*>(s + c0);
        double2* o2 = reinterpret_cast<double2*>(o + c0);
        for (int64_t e0 = threadIdx.x; e0 < n2; e0 += (int64_t)blockDim.x * kLoadBatch) {
          double2 v[kLoadBatch];
#pragma unroll
          for (int i = 0; i < kLoadBatch; ++i) {
            const int64_t e = e0 + (int64_t)i * blockDim.x;
            if (e < n2) v[i] = __ldg(s2 + e);
          }
#pragma unroll
          for (int i = 0; i < kLoadBatch; ++i) {
            const int64_t e = e0 + (int64_t)i * blockDim.x;
            if (e < n2) o2[e] = flip(v[i], sg);
          }
        }
        if ((n & 1) && threadIdx.x == 0) o[c0 + n - 1] = flip(s[c0 + n - 1], sg);
      } else {
        for (int64_t e0 = threadIdx.x; e0 < n; e0 += (int64_t)blockDim.x * kLoadBatch) {
          T v[kLoadBatch];
#pragma unroll
          for (int i = 0; i < kLoadBatch; ++i) {
            const int64_t e = e0 + (int64_t)i * blockDim.x;
            if (e < n) v[i] = __ldg(s + c0 + e);
          }
#pragma unroll
          for (int i = 0; i < kLoadBatch; ++i) {
            const int64_t e = e0 + (int64_t)i * blockDim.x;
            if (e < n) o[c0 + e] = flip(v[i], sg);
          }
        }
      }
      continue;
    }
    // tile mode
    T* cb = bufs + b * kBuf;
    const TileJob<T> j = tile_job<T>(d, local, src, dst);
    if (!pending) tile_loads(j, cb);
    cp_async_wait_all();
    __syncthreads();
    // the next item's tile goes into the other buffer while this one is written out
    pending = false;
    if (t + 1 < t_end) {
      int ln = lo;
      if (t + 1 >= next_begin) {
        ++ln;
        while (ln + 1 < nd && descs[ln + 1].tile_begin <= t + 1) ++ln;
      }
      const PermDesc& dn = ln == lo ? sdesc : descs[ln];
      if (is_tile_item(dn)) {
        tile_loads(tile_job<T>(dn, t + 1 - dn.tile_begin, src, dst), bufs + (b ^ 1) * kBuf);
        pending = true;
      }
    }
    tile_stores(j, cb);
    __syncthreads();
    b ^= 1;
  }
  cp_async_wait_all();
}

// dynamic shared memory of k_permute (also set as the kernel's maximum, per device)
size_t perm_smem_bytes(int elem_bytes) { return (size_t)2 * tile_buf_elems(elem_bytes) * elem_bytes; }

// once per device (the attribute belongs to the current device's copy of the kernel)
void perm_set_smem_attr() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  QLTG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (dev >= 0 && dev < 64 && done[dev]) return;
  QLTG_CUDA(cudaFuncSetAttribute(k_permute<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)perm_smem_bytes(8)));
  QLTG_CUDA(cudaFuncSetAttribute(k_permute<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)perm_smem_bytes(16)));
  if (dev >= 0 && dev < 64) done[dev] = true;
}

int pow2_at_least(int64_t x, int cap) {
  int v = 1;
  while (v < x && v < cap) v <<= 1;
  return v;
}

}  // namespace

void TransposeList::describe(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
                             const std::vector<int64_t>* dst_offsets, bool skip_identity,
                             const std::vector<uint8_t>* skip) {
  host.clear();
  identity.assign(t.nblk, 0);
  ntiles = 0;
  const int r = t.rank;
  const int budget = tile_budget((int)t.elem_bytes());   // elements per tile (32 KB of data)
  for (int64_t b = 0; b < t.nblk; ++b) {
    PermDesc d{};
    d.src_off = t.offsets[b];
    d.dst_off = dst_offsets ? (*dst_offsets)[b] : t.offsets[b];
    d.sign_mask = (!signs.empty() && signs[b] < 0) ? 0x8000000000000000ull : 0ull;
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
    // at most one non-unit dim left after merging: the block's data is laid out the same way
    identity[b] = m <= 1 && d.sign_mask == 0 && d.src_off == d.dst_off;
    int64_t tiles;
    if ((identity[b] && skip_identity) || (skip && (*skip)[b])) {
      tiles = 0;
    } else if (m == 0) {
      d.p = 0;
      tiles = 1;
    } else if (d.p == m - 1) {
      const int64_t runs = t.blk_size(b) / dd[m - 1];
      if (dd[m - 1] * 2 <= kRunChunk) {
        // short runs: several per work item (tq = runs per item)
        d.tq = (int32_t)std::max<int64_t>(2, kRunChunk / dd[m - 1]);
        d.nouter = runs;
        tiles = (runs + d.tq - 1) / d.tq;
      } else {
        d.tq = 1;
        tiles = runs * ((dd[m - 1] + kRunChunk - 1) / kRunChunk);
      }
    } else {
      // tile extents: 32 x 32, or stretched along the longer dim when the other is short
      int tp = -1, tq = -1;
      if (d.p >= 0) {
        const int a = pow2_at_least(dd[d.p], budget), c = pow2_at_least(dd[m - 1], budget);
        if (a >= kTile && c >= kTile) {
          tp = tq = kTile;
        } else if (a < kTile) {
          tp = a;
          tq = std::min(c, budget / a);
        } else {
          tq = c;
          tp = std::min(a, budget / c);
        }
      }
      if (tp < 0 || tp * tq < 64) {
        // both inner dims short: destination-ordered gather
        d.p = -1;
        d.nouter = t.blk_size(b);
        tiles = (d.nouter + kRunChunk - 1) / kRunChunk;
      } else {
        d.tp = tp;
        d.tq = tq;
        d.tiles_p = (int32_t)((dd[d.p] + tp - 1) / tp);
        d.tiles_q = (int32_t)((dd[m - 1] + tq - 1) / tq);
        // batch the largest remaining dim when the (p, q) tile holds few valid elements
        d.u = -1;
        d.tu = 1;
        const int64_t valid = std::min<int64_t>(dd[d.p], tp) * std::min<int64_t>(dd[m - 1], tq);
        int64_t best = 1;
        for (int i = 0; i < m - 1; ++i)
          if (i != d.p && dd[i] > best) { best = dd[i]; d.u = i; }
        if (d.u >= 0 && valid < budget / 2) {
          int tu = 1;
          while (tu * 2 <= budget / (tp * tq) && tu * 2 * valid <= budget && tu < dd[d.u]) tu *= 2;
          d.tu = tu;
        } else {
          d.u = -1;
        }
        d.tiles_u = (int32_t)(d.u >= 0 ? (dd[d.u] + d.tu - 1) / d.tu : 1);
        d.nouter = t.blk_size(b) / (dd[d.p] * dd[m - 1] * (d.u >= 0 ? dd[d.u] : 1));
        tiles = d.nouter * d.tiles_p * d.tiles_q * d.tiles_u;
      }
    }
    d.tile_begin = ntiles;
    ntiles += tiles;
    host.push_back(d);
  }
  nblocks = (int64_t)host.size();
}

void TransposeList::build(const Meta& t, const std::vector<int>& order, const std::vector<double>& signs,
                          const std::vector<int64_t>* dst_offsets, cudaStream_t s, bool skip_identity,
                          const std::vector<uint8_t>* skip) {
  describe(t, order, signs, dst_offsets, skip_identity, skip);
  dev = upload(host, s);
}

void TransposeList::launch(const void* src, void* dst, int elem_bytes, cudaStream_t s) const {
  if (ntiles == 0) return;
  perm_set_smem_attr();
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, (int64_t)current_sm_count() * 8);
  if (elem_bytes == 8)
    k_permute<double><<<grid, kPermThreads, perm_smem_bytes(8), s>>>(dev.as<PermDesc>(), (int)nblocks, ntiles, static_cast<const double*>(src),
                                           static_cast<double*>(dst));
  else
    k_permute<double2><<<grid, kPermThreads, perm_smem_bytes(16), s>>>(dev.as<PermDesc>(), (int)nblocks, ntiles,
                                            static_cast<const double2*>(src), static_cast<double2*>(dst));
  QLTG_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Allocation-free variant (qltg_transpose_noalloc). Some callers cannot allocate device
// memory while they run - a DMRG sweep whose device memory was handed up front to another
// framework's pool (a cudaMalloc then fails or evicts that pool's cache), or a loop that
// cannot pay for the device-wide synchronisation of cudaMalloc / cudaFree - so the per-call
// permutation work list lives in this fixed device table instead of a fresh cudaMalloc.
// Every GPU that loads the library holds the table (about 600 KB) until the process exits.
// All calls share it and it keeps the last call's descriptors, so calls that overlap on the
// GPU (on different streams at once) race; each call waits for its own kernel before
// returning. The table's device address is looked up once per device and kept for the life
// of the process: the library must not outlive a cudaDeviceReset.
namespace {

__device__ __align__(256) PermDesc g_noalloc_perm[kNoAllocPermBlocks];

// Device address of the table on the current device, looked up on every call (host code
// may not use the symbol itself as a device pointer; the lookup allocates nothing, and not
// caching it keeps the address right after a device reset or a reload of the module).
PermDesc* noalloc_table(int device) {
  int cur = -1;
  QLTG_CUDA(cudaGetDevice(&cur));
  QLTG_CHECK(cur == device, QLTG_ERR_INVALID, "the no-allocation permute runs on the current device");
  void* p = nullptr;
  QLTG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_perm));
  return static_cast<PermDesc*>(p);
}

}  // namespace

void launch_permute_noalloc(int device, const TransposeList& tl, const void* src, void* dst, int elem_bytes,
                            cudaStream_t s) {
  QLTG_CHECK(tl.nblocks <= kNoAllocPermBlocks, QLTG_ERR_INVALID,
             "qltg_transpose_noalloc: tensor has " + std::to_string(tl.nblocks) + " blocks, the fixed table holds " +
                 std::to_string(kNoAllocPermBlocks));
  PermDesc* table = noalloc_table(device);
  perm_set_smem_attr();
  if (tl.ntiles == 0) return;
  QLTG_CUDA(cudaMemcpyAsync(table, tl.host.data(), tl.host.size() * sizeof(PermDesc), cudaMemcpyHostToDevice, s));
  const unsigned grid = (unsigned)std::min<int64_t>(tl.ntiles, (int64_t)current_sm_count() * 8);
  if (elem_bytes == 8)
    k_permute<double><<<grid, kPermThreads, perm_smem_bytes(8), s>>>(table, (int)tl.nblocks, tl.ntiles, static_cast<const double*>(src),
                                           static_cast<double*>(dst));
  else
    k_permute<double2><<<grid, kPermThreads, perm_smem_bytes(16), s>>>(table, (int)tl.nblocks, tl.ntiles, static_cast<const double2*>(src),
                                            static_cast<double2*>(dst));
  QLTG_CUDA(cudaGetLastError());
  // the descriptors were copied from this call's host memory and the table is shared:
  // finish before returning
  QLTG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace qltg
