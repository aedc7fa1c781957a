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
using DT = QLTensor<double, U1QN>;
using CT = QLTensor<QLTEN_Complex, U1QN>;
template void qlten_gb300::dmrg::ApplyAxisDiagonal<double, U1QN>(const DT&, size_t, const qlten::dmrg::AxisDiagonalOp<double, U1QN>&, DT&, const qlten_gb300::Context&, double, double);
template void qlten_gb300::dmrg::ApplyAxisDiagonalInPlace<QLTEN_Complex, U1QN>(CT&, size_t, const qlten::dmrg::AxisDiagonalOp<QLTEN_Complex, U1QN>&, const qlten_gb300::Context&);
template void qlten_gb300::dmrg::ApplyAxisDiagonalPreserveOrder<double, U1QN>(const DT&, size_t, const qlten::dmrg::AxisDiagonalOp<double, U1QN>&, DT&, qlten::dmrg::AxisApplyStorageMode, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*);
template void qlten_gb300::dmrg::ScaleAxisSectorsInPlace<double, U1QN>(DT&, const qlten::dmrg::AxisSectorScalar<double, U1QN>&, const qlten_gb300::Context&);
template void qlten_gb300::dmrg::ApplyAxisSectorScalarsPreserveOrder<QLTEN_Complex, U1QN>(const CT&, const qlten::dmrg::AxisSectorScalar<QLTEN_Complex, U1QN>&, CT&, qlten::dmrg::AxisApplyStorageMode, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*);
template void qlten_gb300::dmrg::ApplyAxisMonomial<double, U1QN>(const DT&, size_t, const qlten::dmrg::AxisMonomialOp<double, U1QN>&, DT&, const qlten_gb300::Context&, double, double);
template void qlten_gb300::dmrg::ProjectAxis<QLTEN_Complex, U1QN>(const CT&, size_t, const qlten::dmrg::AxisProjector<U1QN>&, CT&, const qlten_gb300::Context&);
template void qlten_gb300::dmrg::ApplyRank2ToAxisPreserveOrder<double, U1QN>(const DT&, const DT&, size_t, DT&, const qlten_gb300::Context&, qlten::dmrg::Rank2AxisApplyStats*, int);
template void qlten_gb300::dmrg::ApplyTwoRank2ToAxesPreserveOrder<QLTEN_Complex, U1QN>(const CT&, const CT&, size_t, const CT&, size_t, CT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyRank2ThenAxisDiagonalPreserveOrder<double, U1QN>(const DT&, const DT&, size_t, size_t, const qlten::dmrg::AxisDiagonalOp<double, U1QN>&, DT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyRank2ThenAxisSectorScalarsPreserveOrder<double, U1QN>(const DT&, const DT&, size_t, const qlten::dmrg::AxisSectorScalar<double, U1QN>&, DT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder<QLTEN_Complex, U1QN>(const CT&, const CT&, size_t, const qlten::dmrg::AxisSectorScalar<QLTEN_Complex, U1QN>&, const QLTEN_Complex, const QLTEN_Complex, CT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder<double, U1QN>(const DT&, const DT&, size_t, const qlten::dmrg::AxisSectorScalar<double, U1QN>&, DT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyRank2ThenAxisMonomialFusedPreserveOrder<double, U1QN>(const DT&, const DT&, size_t, size_t, const qlten::dmrg::AxisMonomialOp<double, U1QN>&, DT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyTwoRank2ThenAxisDiagonalPreserveOrder<double, U1QN>(const DT&, const DT&, size_t, const DT&, size_t, size_t, const qlten::dmrg::AxisDiagonalOp<double, U1QN>&, DT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder<QLTEN_Complex, U1QN>(const CT&, const CT&, size_t, const CT&, size_t, const qlten::dmrg::AxisSectorScalar<QLTEN_Complex, U1QN>&, CT&, const qlten_gb300::Context&, qlten::dmrg::AxisOpStats*, int);
template void qlten_gb300::dmrg::MoveHeadAxisToTail<double, U1QN>(const DT&, DT&, const qlten_gb300::Context&, qlten::dmrg::AxisLayoutMoveStats*);
int main() { return 0; }
