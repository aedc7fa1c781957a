// Explicit instantiations of the qlten drop-in adapter (include/qlten_gb300.h) against the
// reference headers: proves the adapter compiles with the reference's own QLTensor types.
#include "qlten/qlten.h"
#include "qlten_gb300.h"
using namespace qlten;
using qlten::special_qn::U1QN;
using qlten::special_qn::fU1U1QN;
template void qlten_gb300::Contract<double, U1QN>(const QLTensor<double, U1QN>*, const QLTensor<double, U1QN>*, const std::vector<std::vector<size_t>>&, QLTensor<double, U1QN>*, const qlten_gb300::Context&, int);
template void qlten_gb300::Contract<QLTEN_Complex, fU1U1QN>(const QLTensor<QLTEN_Complex, fU1U1QN>*, const QLTensor<QLTEN_Complex, fU1U1QN>*, const std::vector<std::vector<size_t>>&, QLTensor<QLTEN_Complex, fU1U1QN>*, const qlten_gb300::Context&, int);
template void qlten_gb300::SVD<double, U1QN>(const QLTensor<double, U1QN>*, size_t, const U1QN&, double, size_t, size_t, QLTensor<double, U1QN>*, QLTensor<double, U1QN>*, QLTensor<double, U1QN>*, double*, size_t*, const qlten_gb300::Context&);
template void qlten_gb300::QR<QLTEN_Complex, fU1U1QN>(const QLTensor<QLTEN_Complex, fU1U1QN>*, size_t, const fU1U1QN&, QLTensor<QLTEN_Complex, fU1U1QN>*, QLTensor<QLTEN_Complex, fU1U1QN>*, const qlten_gb300::Context&);
template void qlten_gb300::ContractContiguousAxes<double, U1QN>(const QLTensor<double, U1QN>&, const QLTensor<double, U1QN>&, size_t, size_t, size_t, QLTensor<double, U1QN>&, const qlten_gb300::Context&, int, int, int);
template void qlten_gb300::ContractTailHeadContiguousAccumulate<QLTEN_Complex, fU1U1QN>(const QLTensor<QLTEN_Complex, fU1U1QN>&, const QLTensor<QLTEN_Complex, fU1U1QN>&, size_t, size_t, size_t, QLTEN_Complex, QLTEN_Complex, QLTensor<QLTEN_Complex, fU1U1QN>&, const qlten_gb300::Context&, int);
template bool qlten_gb300::TryContractTailHeadContiguousAccumulate<double, U1QN>(const QLTensor<double, U1QN>&, const QLTensor<double, U1QN>&, size_t, size_t, size_t, double, double, QLTensor<double, U1QN>&, const qlten_gb300::Context&, int);
template void qlten_gb300::LinearCombine<double, U1QN>(const std::vector<double>&, const std::vector<QLTensor<double, U1QN>*>&, double, QLTensor<double, U1QN>*, const qlten_gb300::Context&);
template void qlten_gb300::LinearCombine<QLTEN_Complex, fU1U1QN>(const std::vector<QLTEN_Complex>&, const std::vector<QLTensor<QLTEN_Complex, fU1U1QN>*>&, QLTEN_Complex, QLTensor<QLTEN_Complex, fU1U1QN>*, const qlten_gb300::Context&);
int main() { return 0; }
