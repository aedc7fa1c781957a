// C entry points over synth.h: build a named synthetic workload and export its tensors
// as plain arrays. Used by the Python tests and bench.py to create inputs; it is not
// part of the contraction/decomposition path.
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "synth.h"

namespace {
struct Workload {
  std::vector<qltg_synth::Tensor> tensors;
};
std::string g_synth_err;
}  // namespace

extern "C" {

const char* qltg_synth_last_error(void) { return g_synth_err.c_str(); }

// kinds (params):
//   "cfg1" (seed)                        -> A, B
//   "matvec_u1" (qmax, sigma, D, seed)   -> lenv, psi, mpo1, mpo2, renv  (random operands)
//   "matvec_u1h" (qmax, sigma, D, seed)  -> same, real-symmetric effective Hamiltonian
//   "matvec_u1hc" (qmax, sigma, D, seed) -> same, complex128, complex-Hermitian H_eff
//   "matvec_f" (half, D, seed)           -> same, fermionic U(1)xU(1) complex128
//   "svd_u1" (qmax, sigma, D, seed)      -> T  (psi with a controlled block spectrum)
//   "svd_stress" (nb, lo, hi, seed)      -> T  (rank-2 block-diagonal, sizes lo..hi)
void* qltg_synth_create(const char* kind, const double* p, int np) {
  try {
    namespace sy = qltg_synth;
    auto w = std::make_unique<Workload>();
    std::string k(kind);
    auto need = [&](int n) { if (np < n) throw std::runtime_error("qltg_synth_create: too few parameters"); };
    if (k == "cfg1") {
      need(1);
      auto pr = sy::config1((uint64_t)p[0]);
      w->tensors = {pr.a, pr.b};
    } else if (k == "matvec_u1" || k == "matvec_u1h" || k == "matvec_u1hc" || k == "matvec_f") {
      sy::Matvec m;
      if (k == "matvec_u1") { need(4); m = sy::heisenberg_u1_random((int)p[0], p[1], (int64_t)p[2], (uint64_t)p[3]); }
      else if (k == "matvec_u1h") { need(4); m = sy::heisenberg_u1_hermitian((int)p[0], p[1], (int64_t)p[2], (uint64_t)p[3]); }
      else if (k == "matvec_u1hc") {
        need(4);
        m = sy::heisenberg_u1_hermitian_complex((int)p[0], p[1], (int64_t)p[2], (uint64_t)p[3]);
      }
      else { need(3); m = sy::hubbard_u1u1((int)p[0], (int64_t)p[1], (uint64_t)p[2]); }
      w->tensors = {m.lenv, m.psi, m.mpo1, m.mpo2, m.renv};
    } else if (k == "svd_u1") {
      need(4);
      w->tensors = {sy::svd_psi((int)p[0], p[1], (int64_t)p[2], (uint64_t)p[3])};
    } else if (k == "svd_stress") {
      need(4);
      w->tensors = {sy::svd_stress((int)p[0], (int64_t)p[1], (int64_t)p[2], (uint64_t)p[3])};
    } else {
      throw std::runtime_error("qltg_synth_create: unknown kind " + k);
    }
    return w.release();
  } catch (const std::exception& e) {
    g_synth_err = e.what();
    return nullptr;
  }
}

int qltg_synth_count(void* h) { return (int)static_cast<Workload*>(h)->tensors.size(); }

// info: rank, ncomp, parity_comp, is_complex, nblk, size, total sectors
void qltg_synth_info(void* h, int i, int64_t* info) {
  const auto& t = static_cast<Workload*>(h)->tensors.at(i);
  int64_t ts = 0;
  for (auto& l : t.legs) ts += l.nsct();
  info[0] = t.rank(); info[1] = t.ncomp(); info[2] = t.legs.empty() ? -1 : t.legs[0].parity_comp;
  info[3] = t.is_complex; info[4] = t.nblk(); info[5] = t.size; info[6] = ts;
}

void qltg_synth_export(void* h, int i, int32_t* dirs, int32_t* nsct, int32_t* qns, int64_t* dims,
                       int64_t* coords, int64_t* offsets, double* data) {
  const auto& t = static_cast<Workload*>(h)->tensors.at(i);
  int64_t qp = 0, dp = 0;
  for (int l = 0; l < t.rank(); ++l) {
    dirs[l] = t.legs[l].dir;
    nsct[l] = (int32_t)t.legs[l].nsct();
    for (auto q : t.legs[l].qns) qns[qp++] = q;
    for (auto d : t.legs[l].dims) dims[dp++] = d;
  }
  std::memcpy(coords, t.coords.data(), t.coords.size() * sizeof(int64_t));
  std::memcpy(offsets, t.offsets.data(), t.offsets.size() * sizeof(int64_t));
  std::memcpy(data, t.data.data(), t.data.size() * sizeof(double));
}

void qltg_synth_free(void* h) { delete static_cast<Workload*>(h); }

}  // extern "C"
