// Contraction planning: sector pairing on the device.
//
// The reference builds the task list on the host with an O(nA * nB) double loop comparing
// VecPartHasher values of the contracted block coordinates
// (qltensor/blk_spar_data_ten/data_blk_operations.h:411-578, framework/vec_hash.h:39-51).
// Here each block gets an exact integer key (the mixed-radix value of its contracted
// coordinates, so no hash collisions), B blocks are radix-sorted by key, every A block
// finds its matching B range by binary search, pairs are emitted in the reference's
// generation order (A blocks outer, B blocks inner, both ascending), and a stable sort
// by output block index groups the tasks per output block; the first task of each group
// is the reference's beta = 0 task. Output block offsets come from a device scan.
#include <cub/cub.cuh>

#include <algorithm>
#include <numeric>

#include "ctrct.h"

namespace qltg {
namespace {

struct PairParams {
  int ra, rb, rc, nax, nsa, nsb;
  int axa[kMaxRank], axb[kMaxRank], sa[kMaxRank], sb[kMaxRank];
  int64_t key_w[kMaxRank];       // mixed-radix weights of the contracted coordinates
  int64_t c_w[kMaxRank];         // block-index weights of C's legs
  int a_leg_off[kMaxRank], b_leg_off[kMaxRank];   // per-leg offsets into flattened sector arrays
  int fermionic;
  // the contracted pairs in the caller's order, for the exchange sign (the pairing and the
  // operand transposes may use another order of the same pairs)
  int sgn_axa[kMaxRank], sgn_axb[kMaxRank];
  int a_ctrct_in[kMaxRank];      // A's i-th contracted leg (caller's order) is IN
};

__global__ void k_keys_a(const int32_t* __restrict__ coords, int64_t n, const int64_t* __restrict__ dims,
                         PairParams P, uint64_t* __restrict__ key, int64_t* __restrict__ m_out,
                         int64_t* __restrict__ k_out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t* c = coords + i * P.ra;
  uint64_t kk = 0;
  int64_t kd = 1, md = 1;
  for (int t = 0; t < P.nax; ++t) {
    kk += (uint64_t)c[P.axa[t]] * (uint64_t)P.key_w[t];
    kd *= dims[P.a_leg_off[P.axa[t]] + c[P.axa[t]]];
  }
  for (int t = 0; t < P.nsa; ++t) md *= dims[P.a_leg_off[P.sa[t]] + c[P.sa[t]]];
  key[i] = kk;
  m_out[i] = md;
  k_out[i] = kd;
}

__global__ void k_keys_b(const int32_t* __restrict__ coords, int64_t n, const int64_t* __restrict__ dims,
                         PairParams P, uint64_t* __restrict__ key, int64_t* __restrict__ n_out,
                         int32_t* __restrict__ iota) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int32_t* c = coords + j * P.rb;
  uint64_t kk = 0;
  int64_t nd = 1;
  for (int t = 0; t < P.nax; ++t) kk += (uint64_t)c[P.axb[t]] * (uint64_t)P.key_w[t];
  for (int t = 0; t < P.nsb; ++t) nd *= dims[P.b_leg_off[P.sb[t]] + c[P.sb[t]]];
  key[j] = kk;
  n_out[j] = nd;
  iota[j] = (int32_t)j;
}

__global__ void k_match(const uint64_t* __restrict__ key_a, int64_t na, const uint64_t* __restrict__ key_b_sorted,
                        int64_t nb, int64_t* __restrict__ lo_out, int64_t* __restrict__ cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= na) return;
  const uint64_t k = key_a[i];
  int64_t lo = 0, hi = nb;
  while (lo < hi) { int64_t mid = (lo + hi) >> 1; if (key_b_sorted[mid] < k) lo = mid + 1; else hi = mid; }
  int64_t l = lo;
  hi = nb;
  while (lo < hi) { int64_t mid = (lo + hi) >> 1; if (key_b_sorted[mid] <= k) lo = mid + 1; else hi = mid; }
  lo_out[i] = l;
  cnt[i] = lo - l;
}

// Sign of reordering a block's saved legs from ascending leg order to `order` (n legs):
// -1 per pair of odd legs that trade places. +1 for the ascending order of Contract; for the
// cyclic order of ContractContiguousAxes it is the residue sign of the reference's rotated
// matrix view (qltensor/blk_spar_data_ten/data_blk_operations.h:580-611).
__host__ __device__ inline int saved_order_sign(const uint8_t* par, const int* order, int n) {
  int c = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) c += (order[i] > order[j]) & par[order[i]] & par[order[j]];
  return (c & 1) ? -1 : 1;
}

// Fermionic exchange sign of one pair, the reference's FermionExchangeSignForCtrct
// (data_blk_operations.h:351-401): bring each contracted B leg next to its A partner,
// counting odd legs passed over, plus one exchange per odd IN-direction A leg.
__host__ __device__ inline int exchange_sign(const uint8_t* pa, int ra, const uint8_t* pb, int rb, const int* axa,
                                             const int* axb, int nax, const int* a_in) {
  uint8_t par[2 * kMaxRank];
  int ax[2 * kMaxRank];
  for (int i = 0; i < ra; ++i) par[i] = pa[i];
  for (int i = 0; i < rb; ++i) par[ra + i] = pb[i];
  for (int i = 0; i < nax; ++i) { ax[2 * i] = axa[i]; ax[2 * i + 1] = axb[i] + ra; }
  int ex = 0;
  for (int i = 0; i < nax; ++i) {
    const int x1 = ax[2 * i], x2 = ax[2 * i + 1];
    const int p1 = par[x1], p2 = par[x2];
    if (p2)
      for (int j = x1 + 1; j < x2; ++j) ex += par[j];
    const uint8_t moved = par[x2];
    for (int j = x2; j > x1 + 1; --j) par[j] = par[j - 1];
    par[x1 + 1] = moved;
    for (int j = 0; j < 2 * nax; ++j)
      if (ax[j] > x1 && ax[j] < x2) ax[j]++;
    ax[2 * i + 1] = x1 + 1;
    ex += (p1 && a_in[i]) ? 1 : 0;
  }
  return (ex & 1) ? -1 : 1;
}

__global__ void k_emit(const int32_t* __restrict__ ca, const int32_t* __restrict__ cb, int64_t na,
                       const int64_t* __restrict__ lo, const int64_t* __restrict__ off,
                       const int64_t* __restrict__ cnt, const int32_t* __restrict__ b_sorted_idx,
                       const uint8_t* __restrict__ par_a, const uint8_t* __restrict__ par_b, PairParams P,
                       int32_t* __restrict__ pa, int32_t* __restrict__ pb, uint64_t* __restrict__ cidx,
                       int32_t* __restrict__ psign, int32_t* __restrict__ iota) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= na) return;
  const int32_t* c1 = ca + i * P.ra;
  uint8_t pa_l[kMaxRank], pb_l[kMaxRank];
  uint64_t cbase = 0;
  for (int t = 0; t < P.nsa; ++t) cbase += (uint64_t)c1[P.sa[t]] * (uint64_t)P.c_w[t];
  if (P.fermionic)
    for (int l = 0; l < P.ra; ++l) pa_l[l] = par_a[P.a_leg_off[l] + c1[l]];
  for (int64_t t = 0; t < cnt[i]; ++t) {
    const int64_t p = off[i] + t;
    const int32_t j = b_sorted_idx[lo[i] + t];
    const int32_t* c2 = cb + (int64_t)j * P.rb;
    uint64_t ci = cbase;
    for (int u = 0; u < P.nsb; ++u) ci += (uint64_t)c2[P.sb[u]] * (uint64_t)P.c_w[P.nsa + u];
    int sign = 1;
    if (P.fermionic) {
      for (int l = 0; l < P.rb; ++l) pb_l[l] = par_b[P.b_leg_off[l] + c2[l]];
      sign = exchange_sign(pa_l, P.ra, pb_l, P.rb, P.sgn_axa, P.sgn_axb, P.nax, P.a_ctrct_in) *
             saved_order_sign(pa_l, P.sa, P.nsa) * saved_order_sign(pb_l, P.sb, P.nsb);
    }
    pa[p] = (int32_t)i;
    pb[p] = j;
    cidx[p] = ci;
    psign[p] = sign;
    iota[p] = (int32_t)p;
  }
}

__global__ void k_heads(const uint64_t* __restrict__ cidx_sorted, int64_t n, int32_t* __restrict__ head) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  head[q] = (q == 0 || cidx_sorted[q] != cidx_sorted[q - 1]) ? 1 : 0;
}

__global__ void k_cblocks(const int32_t* __restrict__ head, const int32_t* __restrict__ cb_incl, int64_t n,
                          const uint64_t* __restrict__ cidx_sorted, const int32_t* __restrict__ perm,
                          const int32_t* __restrict__ pa, const int32_t* __restrict__ pb,
                          const int64_t* __restrict__ m_a, const int64_t* __restrict__ n_b,
                          uint64_t* __restrict__ c_idx, int32_t* __restrict__ c_first, int64_t* __restrict__ c_size) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n || !head[q]) return;
  const int32_t cbk = cb_incl[q] - 1;
  const int32_t p = perm[q];
  c_idx[cbk] = cidx_sorted[q];
  c_first[cbk] = (int32_t)q;
  c_size[cbk] = m_a[pa[p]] * n_b[pb[p]];
}

inline unsigned grid_for(int64_t n, int bs = 256) { return (unsigned)std::max<int64_t>(1, (n + bs - 1) / bs); }

int bits_for(uint64_t maxval) {
  int b = 1;
  while (b < 64 && (maxval >> b) != 0) ++b;
  return b;
}

std::vector<int64_t> saved_axes(int rank, const std::vector<int64_t>& ctrct) {
  std::vector<int64_t> s;
  for (int i = 0; i < rank; ++i)
    if (std::find(ctrct.begin(), ctrct.end(), (int64_t)i) == ctrct.end()) s.push_back(i);
  return s;
}

bool is_identity(const std::vector<int64_t>& first, const std::vector<int64_t>& second) {
  for (size_t i = 0; i < first.size(); ++i) if (first[i] != (int64_t)i) return false;
  for (size_t i = 0; i < second.size(); ++i) if (second[i] != (int64_t)(i + first.size())) return false;
  return true;
}

template <typename T>
std::vector<T> download(const DevBuf& b, int64_t n, cudaStream_t s) {
  std::vector<T> v(n);
  if (n) QLTG_CUDA(cudaMemcpyAsync(v.data(), b.get(), n * sizeof(T), cudaMemcpyDeviceToHost, s));
  return v;
}

}  // namespace

int host_exchange_sign(const bool* pa, int ra, const bool* pb, int rb, const int64_t* axa, const int64_t* axb,
                       int nax, const int32_t* a_ctrct_dirs) {
  uint8_t a[kMaxRank], b[kMaxRank];
  int xa[kMaxRank], xb[kMaxRank], in[kMaxRank];
  for (int i = 0; i < ra; ++i) a[i] = pa[i];
  for (int i = 0; i < rb; ++i) b[i] = pb[i];
  for (int i = 0; i < nax; ++i) { xa[i] = (int)axa[i]; xb[i] = (int)axb[i]; in[i] = a_ctrct_dirs[i] == QLTG_IN; }
  return exchange_sign(a, ra, b, rb, xa, xb, nax, in);
}

void plan_contraction(CtrctPlan& p, cudaStream_t s) {
  const Meta& A = p.a;
  const Meta& B = p.b;
  const int nax = (int)p.axa.size();
  QLTG_CHECK(p.axb.size() == p.axa.size(), QLTG_ERR_INVALID, "axes_a and axes_b differ in length");
  QLTG_CHECK(A.dtype == B.dtype, QLTG_ERR_INVALID, "A and B element types differ");
  QLTG_CHECK(A.ncomp == B.ncomp && A.parity_comp == B.parity_comp, QLTG_ERR_INVALID,
             "A and B quantum number types differ");
  QLTG_CHECK(A.rank >= 1 && B.rank >= 1, QLTG_ERR_INVALID, "contraction of a scalar tensor");
  for (int t = 0; t < nax; ++t) {
    QLTG_CHECK(p.axa[t] >= 0 && p.axa[t] < A.rank && p.axb[t] >= 0 && p.axb[t] < B.rank, QLTG_ERR_INVALID,
               "contraction axis out of range");
    for (int u = 0; u < t; ++u)
      QLTG_CHECK(p.axa[u] != p.axa[t] && p.axb[u] != p.axb[t], QLTG_ERR_INVALID, "repeated contraction axis");
    QLTG_CHECK(inverse_leg(A, (int)p.axa[t], B, (int)p.axb[t]), QLTG_ERR_INVALID,
               "contracted legs are not inverse indexes (A[a_i] must equal InverseIndex(B[b_i]))");
  }
  p.sa = saved_axes(A.rank, p.axa);
  p.sb = saved_axes(B.rank, p.axb);
  auto reorder = [](std::vector<int64_t>& saved, const std::vector<int64_t>& order) {
    if (order.empty()) return;
    std::vector<int64_t> x = order, y = saved;
    std::sort(x.begin(), x.end());
    QLTG_CHECK(x == y, QLTG_ERR_INVALID, "saved-leg order is not a permutation of the saved legs");
    saved = order;
  };
  reorder(p.sa, p.sa_order);
  reorder(p.sb, p.sb_order);
  const int rc = (int)(p.sa.size() + p.sb.size());
  QLTG_CHECK(rc <= kMaxRank, QLTG_ERR_UNSUPPORTED, "result rank above 8");

  // The order of the contracted pairs (a_i, b_i) is internal to the contraction: any
  // consistent reordering of the pairs gives the same C (the k index of every block pair
  // is only permuted, in A and B alike; the operand transposes carry no signs). Pick, among
  // the given order and the orders sorted by A's or by B's leg numbers, the one whose operand
  // transposes move the fewest bytes (blocks whose layout a transpose leaves unchanged move
  // none). The fermionic exchange sign of a block pair depends on the order the caller gave,
  // so it is computed from that order (sgn_axa / sgn_axb below), whatever order is used here.
  const std::vector<int64_t> given_axa = p.axa, given_axb = p.axb;
  if (nax >= 2) {
    auto order_of = [&](const std::vector<int64_t>& axa, const std::vector<int64_t>& axb, std::vector<int>& oa,
                        std::vector<int>& ob) {
      oa.assign(p.sa.begin(), p.sa.end());
      oa.insert(oa.end(), axa.begin(), axa.end());
      ob.assign(axb.begin(), axb.end());
      ob.insert(ob.end(), p.sb.begin(), p.sb.end());
    };
    auto moved_bytes = [&](const std::vector<int64_t>& axa, const std::vector<int64_t>& axb) {
      std::vector<int> oa, ob;
      order_of(axa, axb, oa, ob);
      int64_t bytes = 0;
      TransposeList ta, tb;
      ta.describe(A, oa, {}, nullptr);
      tb.describe(B, ob, {}, nullptr);
      for (int64_t b = 0; b < A.nblk; ++b) if (!ta.identity[b]) bytes += A.blk_size(b);
      for (int64_t b = 0; b < B.nblk; ++b) if (!tb.identity[b]) bytes += B.blk_size(b);
      return bytes;
    };
    std::vector<int> idx(nax);
    std::vector<int64_t> best_a = p.axa, best_b = p.axb;
    int64_t best = moved_bytes(p.axa, p.axb);
    for (int by_b = 0; by_b < 2; ++by_b) {
      for (int t = 0; t < nax; ++t) idx[t] = t;
      const auto& key = by_b ? p.axb : p.axa;
      std::sort(idx.begin(), idx.end(), [&](int x, int y) { return key[x] < key[y]; });
      std::vector<int64_t> xa(nax), xb(nax);
      for (int t = 0; t < nax; ++t) { xa[t] = p.axa[idx[t]]; xb[t] = p.axb[idx[t]]; }
      const int64_t m = moved_bytes(xa, xb);
      if (m < best) { best = m; best_a = xa; best_b = xb; }
    }
    p.axa = best_a;
    p.axb = best_b;
  }

  // transpose orders: A -> (saved, contracted), B -> (contracted, saved)
  p.a_order.assign(p.sa.begin(), p.sa.end());
  p.a_order.insert(p.a_order.end(), p.axa.begin(), p.axa.end());
  p.b_order.assign(p.axb.begin(), p.axb.end());
  p.b_order.insert(p.b_order.end(), p.sb.begin(), p.sb.end());
  p.a_trans = !is_identity(p.sa, p.axa);
  p.b_trans = !is_identity(p.axb, p.sb);

  // result metadata (legs)
  Meta& C = p.c;
  C = Meta();
  C.rank = rc;
  C.dtype = A.dtype;
  C.ncomp = A.ncomp;
  C.parity_comp = A.parity_comp;
  for (auto l : p.sa) { C.dirs.push_back(A.dirs[l]); C.qns.push_back(A.qns[l]); C.dims.push_back(A.dims[l]); }
  for (auto l : p.sb) { C.dirs.push_back(B.dirs[l]); C.qns.push_back(B.qns[l]); C.dims.push_back(B.dims[l]); }

  PairParams P{};
  P.ra = A.rank; P.rb = B.rank; P.rc = rc; P.nax = nax;
  P.nsa = (int)p.sa.size(); P.nsb = (int)p.sb.size();
  for (int t = 0; t < nax; ++t) {
    P.axa[t] = (int)p.axa[t];
    P.axb[t] = (int)p.axb[t];
    P.sgn_axa[t] = (int)given_axa[t];
    P.sgn_axb[t] = (int)given_axb[t];
    P.a_ctrct_in[t] = A.dirs[given_axa[t]] == QLTG_IN;
  }
  for (int t = 0; t < P.nsa; ++t) P.sa[t] = (int)p.sa[t];
  for (int t = 0; t < P.nsb; ++t) P.sb[t] = (int)p.sb[t];
  // key weights over the contracted legs (sector counts of A's contracted legs)
  {
    long double range = 1;
    uint64_t w = 1;
    for (int t = nax - 1; t >= 0; --t) { P.key_w[t] = (int64_t)w; w *= (uint64_t)A.nsct((int)p.axa[t]); range *= A.nsct((int)p.axa[t]); }
    QLTG_CHECK(range < 9.0e18L, QLTG_ERR_UNSUPPORTED, "contracted sector space exceeds 63 bits");
    long double crange = 1;
    uint64_t cw = 1;
    for (int l = rc - 1; l >= 0; --l) { P.c_w[l] = (int64_t)cw; cw *= (uint64_t)C.nsct(l); crange *= C.nsct(l); }
    QLTG_CHECK(crange < 9.0e18L, QLTG_ERR_UNSUPPORTED, "result block index exceeds 63 bits");
  }
  P.fermionic = A.parity_comp >= 0;
  std::vector<int64_t> dims_a, dims_b;
  std::vector<uint8_t> par_a, par_b;
  for (int l = 0; l < A.rank; ++l) {
    P.a_leg_off[l] = (int)dims_a.size();
    for (int64_t s2 = 0; s2 < A.nsct(l); ++s2) { dims_a.push_back(A.dims[l][s2]); par_a.push_back(A.parity(l, s2)); }
  }
  for (int l = 0; l < B.rank; ++l) {
    P.b_leg_off[l] = (int)dims_b.size();
    for (int64_t s2 = 0; s2 < B.nsct(l); ++s2) { dims_b.push_back(B.dims[l][s2]); par_b.push_back(B.parity(l, s2)); }
  }
  std::vector<int32_t> ca(A.coords.begin(), A.coords.end()), cb(B.coords.begin(), B.coords.end());

  const int64_t na = A.nblk, nb = B.nblk;
  p.tasks_gen.clear();
  p.flops = 0;
  p.bytes = (double)(A.size + B.size) * A.elem_bytes();
  if (na == 0 || nb == 0) {
    C.nblk = 0;
    C.refresh_offsets();
    return;
  }

  DevBuf d_ca = upload(ca, s), d_cb = upload(cb, s);
  DevBuf d_da = upload(dims_a, s), d_db = upload(dims_b, s);
  DevBuf d_pa = upload(par_a, s), d_pb = upload(par_b, s);
  DevBuf d_keya(na * 8), d_ma(na * 8), d_ka(na * 8);
  DevBuf d_keyb(nb * 8), d_keyb_s(nb * 8), d_nb(nb * 8), d_iotab(nb * 4), d_iotab_s(nb * 4);
  k_keys_a<<<grid_for(na), 256, 0, s>>>(d_ca.as<int32_t>(), na, d_da.as<int64_t>(), P, d_keya.as<uint64_t>(),
                                        d_ma.as<int64_t>(), d_ka.as<int64_t>());
  k_keys_b<<<grid_for(nb), 256, 0, s>>>(d_cb.as<int32_t>(), nb, d_db.as<int64_t>(), P, d_keyb.as<uint64_t>(),
                                        d_nb.as<int64_t>(), d_iotab.as<int32_t>());
  QLTG_CUDA(cudaGetLastError());
  uint64_t kmax = 1;
  for (int t = 0; t < nax; ++t) kmax *= (uint64_t)A.nsct((int)p.axa[t]);
  const int kbits = bits_for(kmax);
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_keyb.as<uint64_t>(), d_keyb_s.as<uint64_t>(),
                                  d_iotab.as<int32_t>(), d_iotab_s.as<int32_t>(), (int)nb, 0, kbits, s);
  DevBuf d_tmp(std::max<size_t>(tmp_bytes, 16));
  QLTG_CUDA(cub::DeviceRadixSort::SortPairs(d_tmp.get(), tmp_bytes, d_keyb.as<uint64_t>(), d_keyb_s.as<uint64_t>(),
                                            d_iotab.as<int32_t>(), d_iotab_s.as<int32_t>(), (int)nb, 0, kbits, s));
  DevBuf d_lo(na * 8), d_cnt(na * 8), d_off(na * 8);
  k_match<<<grid_for(na), 256, 0, s>>>(d_keya.as<uint64_t>(), na, d_keyb_s.as<uint64_t>(), nb, d_lo.as<int64_t>(),
                                       d_cnt.as<int64_t>());
  QLTG_CUDA(cudaGetLastError());
  tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, d_cnt.as<int64_t>(), d_off.as<int64_t>(), (int)na, s);
  if (tmp_bytes > d_tmp.bytes()) d_tmp.alloc(tmp_bytes);
  QLTG_CUDA(cub::DeviceScan::ExclusiveSum(d_tmp.get(), tmp_bytes, d_cnt.as<int64_t>(), d_off.as<int64_t>(), (int)na, s));
  int64_t last_off = 0, last_cnt = 0;
  QLTG_CUDA(cudaMemcpyAsync(&last_off, d_off.as<int64_t>() + na - 1, 8, cudaMemcpyDeviceToHost, s));
  QLTG_CUDA(cudaMemcpyAsync(&last_cnt, d_cnt.as<int64_t>() + na - 1, 8, cudaMemcpyDeviceToHost, s));
  QLTG_CUDA(cudaStreamSynchronize(s));
  const int64_t np = last_off + last_cnt;
  QLTG_CHECK(np < (int64_t)1 << 31, QLTG_ERR_UNSUPPORTED, "more than 2^31 block pairs");
  if (np == 0) {
    C.nblk = 0;
    C.refresh_offsets();
    return;
  }
  DevBuf d_ppa(np * 4), d_ppb(np * 4), d_cidx(np * 8), d_cidx_s(np * 8), d_sign(np * 4), d_iota(np * 4), d_perm(np * 4);
  k_emit<<<grid_for(na, 128), 128, 0, s>>>(d_ca.as<int32_t>(), d_cb.as<int32_t>(), na, d_lo.as<int64_t>(),
                                           d_off.as<int64_t>(), d_cnt.as<int64_t>(), d_iotab_s.as<int32_t>(),
                                           d_pa.as<uint8_t>(), d_pb.as<uint8_t>(), P, d_ppa.as<int32_t>(),
                                           d_ppb.as<int32_t>(), d_cidx.as<uint64_t>(), d_sign.as<int32_t>(),
                                           d_iota.as<int32_t>());
  QLTG_CUDA(cudaGetLastError());
  uint64_t cmax = 1;
  for (int l = 0; l < rc; ++l) cmax *= (uint64_t)C.nsct(l);
  const int cbits = bits_for(cmax);
  tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_cidx.as<uint64_t>(), d_cidx_s.as<uint64_t>(),
                                  d_iota.as<int32_t>(), d_perm.as<int32_t>(), (int)np, 0, cbits, s);
  if (tmp_bytes > d_tmp.bytes()) d_tmp.alloc(tmp_bytes);
  QLTG_CUDA(cub::DeviceRadixSort::SortPairs(d_tmp.get(), tmp_bytes, d_cidx.as<uint64_t>(), d_cidx_s.as<uint64_t>(),
                                            d_iota.as<int32_t>(), d_perm.as<int32_t>(), (int)np, 0, cbits, s));
  DevBuf d_head(np * 4), d_cbi(np * 4);
  k_heads<<<grid_for(np), 256, 0, s>>>(d_cidx_s.as<uint64_t>(), np, d_head.as<int32_t>());
  QLTG_CUDA(cudaGetLastError());
  tmp_bytes = 0;
  cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, d_head.as<int32_t>(), d_cbi.as<int32_t>(), (int)np, s);
  if (tmp_bytes > d_tmp.bytes()) d_tmp.alloc(tmp_bytes);
  QLTG_CUDA(cub::DeviceScan::InclusiveSum(d_tmp.get(), tmp_bytes, d_head.as<int32_t>(), d_cbi.as<int32_t>(), (int)np, s));
  int32_t ncb = 0;
  QLTG_CUDA(cudaMemcpyAsync(&ncb, d_cbi.as<int32_t>() + np - 1, 4, cudaMemcpyDeviceToHost, s));
  QLTG_CUDA(cudaStreamSynchronize(s));
  DevBuf d_cidxu(ncb * 8), d_cfirst(ncb * 4), d_csize(ncb * 8), d_coff(ncb * 8);
  k_cblocks<<<grid_for(np), 256, 0, s>>>(d_head.as<int32_t>(), d_cbi.as<int32_t>(), np, d_cidx_s.as<uint64_t>(),
                                         d_perm.as<int32_t>(), d_ppa.as<int32_t>(), d_ppb.as<int32_t>(),
                                         d_ma.as<int64_t>(), d_nb.as<int64_t>(), d_cidxu.as<uint64_t>(),
                                         d_cfirst.as<int32_t>(), d_csize.as<int64_t>());
  QLTG_CUDA(cudaGetLastError());
  tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, d_csize.as<int64_t>(), d_coff.as<int64_t>(), ncb, s);
  if (tmp_bytes > d_tmp.bytes()) d_tmp.alloc(tmp_bytes);
  QLTG_CUDA(cub::DeviceScan::ExclusiveSum(d_tmp.get(), tmp_bytes, d_csize.as<int64_t>(), d_coff.as<int64_t>(), ncb, s));

  auto h_cidxu = download<uint64_t>(d_cidxu, ncb, s);
  auto h_cfirst = download<int32_t>(d_cfirst, ncb, s);
  auto h_coff = download<int64_t>(d_coff, ncb, s);
  auto h_perm = download<int32_t>(d_perm, np, s);
  auto h_ppa = download<int32_t>(d_ppa, np, s);
  auto h_ppb = download<int32_t>(d_ppb, np, s);
  auto h_sign = download<int32_t>(d_sign, np, s);
  auto h_cidx = download<uint64_t>(d_cidx, np, s);
  auto h_ma = download<int64_t>(d_ma, na, s);
  auto h_ka = download<int64_t>(d_ka, na, s);
  auto h_nb = download<int64_t>(d_nb, nb, s);
  QLTG_CUDA(cudaStreamSynchronize(s));

  // Result blocks (ascending block index) and offsets.
  C.nblk = ncb;
  C.coords.assign((size_t)ncb * rc, 0);
  for (int32_t q = 0; q < ncb; ++q) {
    uint64_t rem = h_cidxu[q];
    for (int l = rc - 1; l >= 0; --l) { C.coords[(size_t)q * rc + l] = (int64_t)(rem % (uint64_t)C.nsct(l)); rem /= (uint64_t)C.nsct(l); }
  }
  C.refresh_offsets();
  for (int32_t q = 0; q < ncb; ++q)
    QLTG_CHECK(C.offsets[q] == h_coff[q], QLTG_ERR_INVALID, "internal: device and host result offsets differ");
  p.bytes += (double)C.size * C.elem_bytes();

  // Generation-order task export and the grouped GEMM schedule.
  std::vector<int32_t> beta(np, 1), cblk_of(np, 0);
  {
    int32_t cbk = -1;
    for (int64_t q = 0; q < np; ++q) {
      if (cbk + 1 < ncb && h_cfirst[cbk + 1] == q) { ++cbk; beta[h_perm[q]] = 0; }
      cblk_of[h_perm[q]] = cbk;
    }
  }
  p.tasks_gen.resize((size_t)np * 8);
  const double fl_mul = A.dtype == QLTG_C128 ? 8.0 : 2.0;
  for (int64_t t = 0; t < np; ++t) {
    const int32_t i = h_ppa[t], j = h_ppb[t];
    int64_t* r = &p.tasks_gen[(size_t)t * 8];
    r[0] = (int64_t)A.blk_idx(&A.coords[(size_t)i * A.rank]);
    r[1] = (int64_t)B.blk_idx(&B.coords[(size_t)j * B.rank]);
    r[2] = (int64_t)h_cidx[t];
    r[3] = h_ma[i]; r[4] = h_ka[i]; r[5] = h_nb[j];
    r[6] = h_sign[t]; r[7] = beta[t];
    p.flops += fl_mul * (double)h_ma[i] * (double)h_ka[i] * (double)h_nb[j];
  }

  GemmSchedule& g = p.sched;
  g.cblk.resize(ncb);
  g.task.resize(np);
  for (int64_t q = 0; q < np; ++q) {
    const int32_t t = h_perm[q];
    const int32_t i = h_ppa[t], j = h_ppb[t];
    g.task[q] = GemmTask{A.offsets[i], B.offsets[j], (int32_t)h_ka[i], h_sign[t], (int32_t)h_ka[i], 1};
  }
  for (int32_t q = 0; q < ncb; ++q) {
    const int32_t t = h_perm[h_cfirst[q]];
    const int32_t t1 = (q + 1 < ncb) ? h_cfirst[q + 1] : (int32_t)np;
    g.cblk[q] = GemmCBlk{C.offsets[q], (int32_t)h_ma[h_ppa[t]], (int32_t)h_nb[h_ppb[t]], h_cfirst[q], t1};
  }
}

}  // namespace qltg
