"""GB300-native block-sparse hot path of TensorToolkit (qlten): Contract, SVD, QR and the
two-site H*psi matvec, computed by hand-written sm_103a CUDA kernels in libqltg.so behind
the C ABI declared in include/qltg.h.

Submodules:
  tensor     host-side block-sparse metadata (BSTensor, Leg)
  capi       ctypes declarations of the C ABI
  api        Contract / Transpose / SVD / QR / Matvec / Lanczos over device-resident tensors
  workloads  deterministic synthetic workloads with the reference's shapes
"""
from .tensor import BSTensor, Leg, IN, OUT  # noqa: F401

_API = {"Contract", "ContractionPlan", "ContractContiguousAxes", "ContiguousContractionPlan",
        "ContractTailHeadContiguous", "ContractTailHeadContiguousAccumulate",
        "TryContractTailHeadContiguousAccumulate", "AccumulatePlan", "read_qlten", "write_qlten", "ApplyAxisDiagonal",
        "ApplyAxisDiagonalInPlace", "ApplyAxisSectorScalars", "AxisRank2Plan", "ApplyRank2ToAxisPreserveOrder",
        "ApplyTwoRank2ToAxesPreserveOrder", "ApplyAxisMonomial", "AxisMonomialPlan", "AxisProjectPlan", "ProjectAxis",
        "LinearCombinePlan", "LinearCombine", "AddScaledAssign", "ApplyAxisDiagonalPreserveOrder",
        "ScaleAxisSectorsInPlace", "ApplyAxisSectorScalarsPreserveOrder", "ApplyRank2ThenAxisDiagonalPreserveOrder",
        "ApplyRank2ThenAxisSectorScalarsPreserveOrder",
        "ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder",
        "ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder", "ApplyRank2ThenAxisMonomialFusedPreserveOrder",
        "ApplyTwoRank2ThenAxisDiagonalPreserveOrder", "ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder",
        "MoveHeadAxisToTail", "Transpose", "SVD", "QR", "Matvec", "Lanczos", "DTensor", "Context", "context"}


def __getattr__(name):
    if name in _API:
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
