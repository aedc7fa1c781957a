"""User-facing Python API over the C ABI, with the reference's names and semantics.

`Contract`, `SVD`, `QR` and `Transpose` take and return `DTensor`s: block-sparse tensors
whose metadata lives on the host (`BSTensor`) and whose raw buffer lives in HBM (a torch
CUDA tensor used only as device storage). Every computation runs in libqltg.so; nothing
here falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import capi
from .capi import check, lib
from .tensor import BSTensor, Leg

MODES = {"fp64": capi.QLTG_MODE_FP64, "split": capi.QLTG_MODE_SPLIT}


def _mode(m) -> int:
    return MODES[m] if isinstance(m, str) else int(m)


class Context:
    """A qltg context bound to one CUDA device."""

    def __init__(self, device: int = 0):
        self.device = device
        h = C.c_void_p()
        check(lib().qltg_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().qltg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ctx = {}


def context(device: int = 0) -> Context:
    if device not in _ctx:
        _ctx[device] = Context(device)
    return _ctx[device]


def stream_ptr(device: int = 0) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class _Desc:
    """A TensorDesc plus the numpy arrays it points into."""

    def __init__(self, t: BSTensor):
        self.dirs, self.nsct, self.qns, self.dims = t.meta_arrays()
        self.coords = np.ascontiguousarray(t.coords.reshape(-1), dtype=np.int64)
        p = lambda a: a.ctypes.data if a.size else None
        self.s = capi.TensorDesc(t.rank, capi.QLTG_C128 if t.is_complex else capi.QLTG_F64, t.ncomp,
                                 t.parity_comp, p(self.dirs), p(self.nsct), p(self.qns), p(self.dims),
                                 t.nblk if t.rank else (1 if t.size else 0), p(self.coords))

    @property
    def ref(self):
        return C.byref(self.s)


class DTensor:
    """Block-sparse tensor with its raw buffer resident on a CUDA device."""

    def __init__(self, meta: BSTensor, buf: torch.Tensor):
        n = meta.size * (2 if meta.is_complex else 1)
        if buf.dtype != torch.float64 or buf.numel() < n or not buf.is_cuda:
            raise ValueError("raw buffer must be a CUDA float64 tensor of the layout's size")
        self.meta = meta
        self.buf = buf

    @staticmethod
    def empty(meta: BSTensor, device: int = 0) -> "DTensor":
        n = meta.size * (2 if meta.is_complex else 1)
        return DTensor(meta, torch.empty(max(n, 1), dtype=torch.float64, device=f"cuda:{device}"))

    @staticmethod
    def from_host(t: BSTensor, device: int = 0) -> "DTensor":
        meta = BSTensor(t.legs, t.coords, t.dtype, None, offsets=t.offsets, size=t.size)
        d = DTensor.empty(meta, device)
        if t.size:
            d.buf[: t.size * (2 if t.is_complex else 1)].copy_(torch.from_numpy(t.raw_f64()))
        return d

    def to_host(self) -> BSTensor:
        n = self.meta.size * (2 if self.meta.is_complex else 1)
        raw = self.buf[:n].cpu().numpy()
        data = raw.view(np.complex128) if self.meta.is_complex else raw
        return BSTensor(self.meta.legs, self.meta.coords, self.meta.dtype, data.copy(),
                        offsets=self.meta.offsets, size=self.meta.size)

    @property
    def ptr(self) -> int:
        return self.buf.data_ptr()

    @property
    def device(self) -> int:
        return self.buf.device.index


class ContractionPlan:
    """Planned C = A . B (device sector pairing once, execute many times)."""

    def __init__(self, a: BSTensor, b: BSTensor, axes: Sequence[Sequence[int]], device: int = 0):
        self.ctx = context(device)
        self.device = device
        self.axes = (tuple(int(x) for x in axes[0]), tuple(int(x) for x in axes[1]))
        da, db = _Desc(a), _Desc(b)
        axa = np.asarray(self.axes[0], np.int64)
        axb = np.asarray(self.axes[1], np.int64)
        h = C.c_void_p()
        check(lib().qltg_ctrct_plan_create(self.ctx.h, da.ref, db.ref, axa.ctypes.data, axb.ctypes.data,
                                           len(axa), C.byref(h)))
        self.h = h
        rank, nblk, size = C.c_int32(), C.c_int64(), C.c_int64()
        check(lib().qltg_ctrct_plan_result(h, C.byref(rank), C.byref(nblk), C.byref(size)))
        coords = np.zeros(max(nblk.value * rank.value, 1), np.int64)
        offs = np.zeros(max(nblk.value, 1), np.int64)
        check(lib().qltg_ctrct_plan_result_blocks(h, coords.ctypes.data, offs.ctypes.data))
        sa = [i for i in range(a.rank) if i not in self.axes[0]]
        sb = [i for i in range(b.rank) if i not in self.axes[1]]
        legs = [a.legs[i] for i in sa] + [b.legs[i] for i in sb]
        if rank.value:
            self.result = BSTensor(legs, coords[: nblk.value * rank.value].reshape(nblk.value, rank.value),
                                   a.dtype, None, offsets=offs[: nblk.value])
        else:
            self.result = BSTensor([], np.zeros((nblk.value, 0), np.int64), a.dtype, None, size=size.value)

    def tasks(self) -> np.ndarray:
        n = C.c_int64()
        check(lib().qltg_ctrct_plan_tasks(self.h, C.byref(n), None))
        out = np.zeros((n.value, 8), np.int64)
        if n.value:
            check(lib().qltg_ctrct_plan_tasks(self.h, C.byref(n), out.ctypes.data))
        return out

    def stats(self) -> Tuple[float, float]:
        f, b = C.c_double(), C.c_double()
        check(lib().qltg_ctrct_plan_stats(self.h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def execute(self, a: DTensor, b: DTensor, out: Optional[DTensor] = None, mode="fp64") -> DTensor:
        if out is None:
            out = DTensor.empty(self.result, self.device)
        check(lib().qltg_ctrct_exec(self.h, C.c_void_p(a.ptr), C.c_void_p(b.ptr), C.c_void_p(out.ptr),
                                    _mode(mode), stream_ptr(self.device)))
        return out

    def device_status(self) -> None:
        check(lib().qltg_ctrct_plan_device_status(self.h, stream_ptr(self.device)))

    def set_schedule(self, f64_tile_rows: int = 0, split_stack: int = -1) -> None:
        """FP64 tile rows (32 or 64; 0 keeps) and split-precision row stacking (1 / 0; -1 keeps)."""
        check(lib().qltg_ctrct_plan_set_schedule(self.h, int(f64_tile_rows), int(split_stack),
                                                 stream_ptr(self.device)))

    def schedule(self) -> dict:
        """The current schedule, whether the tuner chose it per mode, and the GEMM-stage times
        (ms) it measured for the chosen and the slowest candidate."""
        rows, stack = C.c_int32(), C.c_int32()
        tuned = np.zeros(2, np.int32)
        ms = np.zeros(4, np.float32)
        check(lib().qltg_ctrct_plan_get_schedule(self.h, C.byref(rows), C.byref(stack), tuned.ctypes.data,
                                                 ms.ctypes.data))
        return {"f64_tile_rows": rows.value, "split_stack": bool(stack.value),
                "tuned": {"fp64": bool(tuned[0]), "split": bool(tuned[1])},
                "tuned_ms": {"fp64": [float(ms[0]), float(ms[1])], "split": [float(ms[2]), float(ms[3])]}}

    def split_stats(self) -> Tuple[int, float]:
        """(128 x 32 x 32 tile stages per split GEMM launch, useful share of them)."""
        n, f = C.c_int64(), C.c_double()
        check(lib().qltg_ctrct_plan_split_stats(self.h, C.byref(n), C.byref(f)))
        return n.value, f.value

    def tune(self, a: "DTensor", b: "DTensor", out: Optional["DTensor"] = None, mode="fp64") -> bool:
        """Autotune the GEMM schedule of `mode` on these operands (out is overwritten); returns
        True when the choice came from the per-signature cache."""
        if out is None:
            out = DTensor.empty(self.result, self.device)
        cached = C.c_int32()
        check(lib().qltg_ctrct_plan_tune(self.h, C.c_void_p(a.ptr), C.c_void_p(b.ptr), C.c_void_p(out.ptr),
                                         _mode(mode), stream_ptr(self.device), C.byref(cached)))
        return bool(cached.value)

    def __del__(self):
        try:
            if self.h:
                lib().qltg_ctrct_plan_destroy(self.h)
        except Exception:
            pass


def Contract(a: DTensor, b: DTensor, axes: Sequence[Sequence[int]], mode="fp64") -> DTensor:
    """C = A . B, the reference's qlten::Contract (tensor_manipulation/ten_ctrct.h:276-290).

    The result's legs are the saved legs of A followed by the saved legs of B."""
    plan = ContractionPlan(a.meta, b.meta, axes, a.device)
    return plan.execute(a, b, mode=mode)


_SIDES = {"head": capi.QLTG_SIDE_HEAD, "tail": capi.QLTG_SIDE_TAIL}


def _contiguous_axes(ra: int, rb: int, a_start: int, b_start: int, n: int):
    """Contracted axes and cyclic saved orders of ContractContiguousAxes."""
    axa = [(a_start + i) % ra for i in range(n)]
    axb = [(b_start + i) % rb for i in range(n)]
    sa = [(a_start + n + i) % ra for i in range(ra - n)]
    sb = [(b_start + n + i) % rb for i in range(rb - n)]
    return axa, axb, sa, sb


def _result_meta(h, result_fn, blocks_fn, legs, dtype) -> BSTensor:
    rank, nblk, size = C.c_int32(), C.c_int64(), C.c_int64()
    check(result_fn(h, C.byref(rank), C.byref(nblk), C.byref(size)))
    coords = np.zeros(max(nblk.value * rank.value, 1), np.int64)
    offs = np.zeros(max(nblk.value, 1), np.int64)
    check(blocks_fn(h, coords.ctypes.data, offs.ctypes.data))
    if rank.value:
        return BSTensor(legs, coords[: nblk.value * rank.value].reshape(nblk.value, rank.value), dtype, None,
                        offsets=offs[: nblk.value])
    return BSTensor([], np.zeros((nblk.value, 0), np.int64), dtype, None, size=size.value)


class ContiguousContractionPlan(ContractionPlan):
    """Planned ContractContiguousAxes<ASide, BSide>(A, B, a_start, b_start, n, C)
    (reference tensor_manipulation/contract_contiguous_axes.h:849-868): A's axes
    (a_start + i) mod rank against B's (b_start + i) mod rank; C's legs are A's saved legs
    then B's, each cyclic from the end of its contracted range. The sides are the
    reference's layout hints ("head" / "tail"); the result does not depend on them."""

    def __init__(self, a: BSTensor, b: BSTensor, a_start: int, b_start: int, n: int, a_side: str = "tail",
                 b_side: str = "head", device: int = 0):
        self.ctx = context(device)
        self.device = device
        axa, axb, sa, sb = _contiguous_axes(a.rank, b.rank, int(a_start), int(b_start), int(n))
        self.axes = (tuple(axa), tuple(axb))
        da, db = _Desc(a), _Desc(b)
        h = C.c_void_p()
        check(lib().qltg_ctrct_plan_create_contiguous(self.ctx.h, da.ref, db.ref, int(a_start), int(b_start), int(n),
                                                      _SIDES[a_side], _SIDES[b_side], C.byref(h)))
        self.h = h
        legs = [a.legs[i] for i in sa] + [b.legs[i] for i in sb]
        self.result = _result_meta(h, lib().qltg_ctrct_plan_result, lib().qltg_ctrct_plan_result_blocks, legs,
                                   a.dtype)


def ContractContiguousAxes(a: DTensor, b: DTensor, a_start: int, b_start: int, n: int, a_side: str = "tail",
                           b_side: str = "head", mode="fp64") -> DTensor:
    """The reference's ContractContiguousAxes (contract_contiguous_axes.h:849-868)."""
    plan = ContiguousContractionPlan(a.meta, b.meta, a_start, b_start, n, a_side, b_side, a.device)
    return plan.execute(a, b, mode=mode)


def ContractTailHeadContiguous(a: DTensor, b: DTensor, a_start: int, b_start: int, n: int, mode="fp64") -> DTensor:
    """The reference's ContractTailHeadContiguous (contract_contiguous_axes.h:914-928)."""
    return ContractContiguousAxes(a, b, a_start, b_start, n, "tail", "head", mode)


class AccumulatePlan:
    """Planned C = beta C + alpha A.B (tail/head contiguous contraction) over the union of C's
    blocks and the contraction's, the reference's ContractTailHeadContiguousAccumulate
    (allow_expand) / TryContractTailHeadContiguousAccumulate (contract_contiguous_axes.h:
    953-1040). Raises ContractAccumulateLayoutMismatch when C's indexes differ from the
    result's, or it lacks result blocks and allow_expand is False."""

    def __init__(self, a: BSTensor, b: BSTensor, a_start: int, b_start: int, n: int, c: Optional[BSTensor],
                 allow_expand: bool = True, device: int = 0):
        self.h = None
        self.ctx = context(device)
        self.device = device
        self.has_c = c is not None
        _, _, sa, sb = _contiguous_axes(a.rank, b.rank, int(a_start), int(b_start), int(n))
        da, db = _Desc(a), _Desc(b)
        dc = _Desc(c) if c is not None else None
        h = C.c_void_p()
        exp = C.c_int32()
        check(lib().qltg_accum_plan_create(self.ctx.h, da.ref, db.ref, int(a_start), int(b_start), int(n),
                                           dc.ref if dc is not None else None, int(bool(allow_expand)), C.byref(h),
                                           C.byref(exp)))
        self.h = h
        self.expanded = bool(exp.value)
        legs = [a.legs[i] for i in sa] + [b.legs[i] for i in sb]
        self.result = _result_meta(h, lib().qltg_accum_plan_result, lib().qltg_accum_plan_result_blocks, legs,
                                   a.dtype)

    def execute(self, a: DTensor, b: DTensor, c: Optional[DTensor], alpha, beta, out: Optional[DTensor] = None,
                mode="fp64") -> DTensor:
        """out = beta c + alpha a.b. Without `out` the result goes over c's buffer when the
        topology did not grow, else into a new tensor."""
        if out is None:
            out = c if (c is not None and not self.expanded) else DTensor.empty(self.result, self.device)
        al = np.array([complex(alpha).real, complex(alpha).imag])
        be = np.array([complex(beta).real, complex(beta).imag])
        check(lib().qltg_accum_exec(self.h, C.c_void_p(a.ptr), C.c_void_p(b.ptr),
                                    C.c_void_p(c.ptr) if c is not None else None, C.c_void_p(out.ptr),
                                    al.ctypes.data, be.ctypes.data, _mode(mode), stream_ptr(self.device)))
        if out is c:
            out.meta = self.result
        return out

    def device_status(self) -> None:
        check(lib().qltg_accum_plan_device_status(self.h, stream_ptr(self.device)))

    def __del__(self):
        try:
            if self.h:
                lib().qltg_accum_plan_destroy(self.h)
        except Exception:
            pass


def ContractTailHeadContiguousAccumulate(a: DTensor, b: DTensor, a_start: int, b_start: int, n: int, alpha, beta,
                                         c: Optional[DTensor] = None, mode="fp64") -> DTensor:
    """c = beta c + alpha A.B; returns the updated tensor (c itself unless its topology grew).
    c None is the reference's default output (beta must be 0)."""
    plan = AccumulatePlan(a.meta, b.meta, a_start, b_start, n, c.meta if c is not None else None, True, a.device)
    return plan.execute(a, b, c, alpha, beta, mode=mode)


def TryContractTailHeadContiguousAccumulate(a: DTensor, b: DTensor, a_start: int, b_start: int, n: int, alpha,
                                            beta, c: Optional[DTensor] = None,
                                            mode="fp64") -> Tuple[bool, Optional[DTensor]]:
    """(True, updated c) when c already holds every result block (or is default with
    beta == 0); (False, c unchanged) when the layout does not fit."""
    try:
        plan = AccumulatePlan(a.meta, b.meta, a_start, b_start, n, c.meta if c is not None else None, False,
                              a.device)
    except capi.ContractAccumulateLayoutMismatch:
        return False, c
    return True, plan.execute(a, b, c, alpha, beta, mode=mode)


# ------------------------------------------------------------------ dmrg axis primitives
def _ab(x) -> np.ndarray:
    return np.array([complex(x).real, complex(x).imag])


def _axis_values(vals, is_complex: bool) -> np.ndarray:
    v = np.asarray(vals)
    return np.ascontiguousarray(v.astype(np.complex128) if is_complex else v.astype(np.float64)).view(np.float64)


def ApplyAxisDiagonal(t: DTensor, axis: int, values, alpha=1.0, beta=0.0, out: Optional[DTensor] = None) -> DTensor:
    """out = beta out + alpha D(t): qlten::dmrg::ApplyAxisDiagonal (reference
    tensor_manipulation/dmrg/axis_ops.h:2370-2547). `values`: one per degeneracy of `axis`,
    sectors in index order (AxisDiagonalOp::values flattened). `out` None: a new tensor
    (beta must then be 0); `out is t`: ApplyAxisDiagonalInPlace."""
    if out is None:
        if complex(beta) != 0:
            raise ValueError("beta != 0 needs an existing output")
        out = DTensor.empty(t.meta, t.device)
    d = _Desc(t.meta)
    v = _axis_values(values, t.meta.is_complex)
    al, be = _ab(alpha), _ab(beta)   # kept alive across the call
    check(lib().qltg_axis_diagonal(context(t.device).h, d.ref, int(axis), v.ctypes.data, C.c_void_p(t.ptr),
                                   C.c_void_p(out.ptr), al.ctypes.data, be.ctypes.data, stream_ptr(t.device)))
    return out


def ApplyAxisDiagonalInPlace(t: DTensor, axis: int, values) -> DTensor:
    """qlten::dmrg::ApplyAxisDiagonalInPlace (axis_ops.h:2549-2582)."""
    return ApplyAxisDiagonal(t, axis, values, 1.0, 0.0, out=t)


def ApplyAxisSectorScalars(t: DTensor, axis: int, values_by_sector, out: Optional[DTensor] = None) -> DTensor:
    """qlten::dmrg::ApplyAxisSectorScalarsPreserveOrder (axis_ops.h:2655-2744): every block
    times the value of its sector on `axis` (out None: a new tensor; out is t: in place)."""
    if out is None:
        out = DTensor.empty(t.meta, t.device)
    d = _Desc(t.meta)
    v = _axis_values(values_by_sector, t.meta.is_complex)
    check(lib().qltg_axis_sector_scalars(context(t.device).h, d.ref, int(axis), v.ctypes.data, C.c_void_p(t.ptr),
                                         C.c_void_p(out.ptr), stream_ptr(t.device)))
    return out


class AxisRank2Plan:
    """Planned ApplyRank2ToAxisPreserveOrder (axis_ops.h:2862-2993) or, with a second
    operator, ApplyTwoRank2ToAxesPreserveOrder (:2995-3126)."""

    def __init__(self, t: BSTensor, op1: BSTensor, axis1: int, op2: Optional[BSTensor] = None,
                 axis2: Optional[int] = None, device: int = 0):
        self.h = None
        self.ctx = context(device)
        self.device = device
        dt, d1 = _Desc(t), _Desc(op1)
        h = C.c_void_p()
        legs = list(t.legs)
        legs[axis1] = op1.legs[1]
        if op2 is None:
            check(lib().qltg_axis_rank2_plan_create(self.ctx.h, dt.ref, d1.ref, int(axis1), C.byref(h)))
        else:
            d2 = _Desc(op2)
            check(lib().qltg_axis_two_rank2_plan_create(self.ctx.h, dt.ref, d1.ref, int(axis1), d2.ref, int(axis2),
                                                        C.byref(h)))
            legs[axis2] = op2.legs[1]
        self.h = h
        self.two = op2 is not None
        self.result = _result_meta(h, lib().qltg_axis_plan_result, lib().qltg_axis_plan_result_blocks, legs, t.dtype)

    def execute(self, t: DTensor, op1: DTensor, op2: Optional[DTensor] = None, out: Optional[DTensor] = None,
                mode="fp64") -> DTensor:
        if out is None:
            out = DTensor.empty(self.result, self.device)
        check(lib().qltg_axis_plan_exec(self.h, C.c_void_p(t.ptr), C.c_void_p(op1.ptr),
                                        C.c_void_p(op2.ptr) if op2 is not None else None, C.c_void_p(out.ptr),
                                        _mode(mode), stream_ptr(self.device)))
        return out

    def device_status(self) -> None:
        check(lib().qltg_axis_plan_device_status(self.h, stream_ptr(self.device)))

    def __del__(self):
        try:
            if self.h:
                lib().qltg_axis_plan_destroy(self.h)
        except Exception:
            pass


class AxisMonomialPlan:
    """Planned qlten::dmrg::ApplyAxisMonomial (axis_ops.h:2746-2860): `entries` rows
    (in_sector, in_offset, out_sector, out_offset) with `coefs`; `out_leg` replaces `axis`;
    output qn = input qn + flux for every entry."""

    def __init__(self, t: BSTensor, axis: int, out_leg: Leg, flux: Sequence[int], entries, coefs,
                 device: int = 0):
        self.h = None
        self.ctx = context(device)
        self.device = device
        dt = _Desc(t)
        ent = np.ascontiguousarray(np.asarray(entries, np.int64).reshape(-1, 4))
        cf = _axis_values(coefs, t.is_complex)
        oq = np.ascontiguousarray(out_leg.qns.reshape(-1), np.int32)
        od = np.ascontiguousarray(out_leg.dims, np.int64)
        fl = np.ascontiguousarray(np.asarray(flux, np.int32).reshape(-1))
        h = C.c_void_p()
        check(lib().qltg_axis_monomial_plan_create(self.ctx.h, dt.ref, int(axis), int(out_leg.nsct), oq.ctypes.data,
                                                   od.ctypes.data, fl.ctypes.data, len(ent),
                                                   ent.ctypes.data if len(ent) else None,
                                                   cf.ctypes.data if len(ent) else None, C.byref(h)))
        self.h = h
        legs = list(t.legs)
        legs[axis] = Leg(t.legs[axis].dir, out_leg.qns, out_leg.dims, t.legs[axis].parity_comp)
        self.result = _result_meta(h, lib().qltg_axis_plan_result, lib().qltg_axis_plan_result_blocks, legs, t.dtype)

    def execute(self, t: DTensor, alpha=1.0, beta=0.0, out: Optional[DTensor] = None) -> DTensor:
        if out is None:
            if complex(beta) != 0:
                raise ValueError("beta != 0 needs an existing output")
            out = DTensor.empty(self.result, self.device)
        al, be = _ab(alpha), _ab(beta)
        check(lib().qltg_axis_monomial_exec(self.h, C.c_void_p(t.ptr), C.c_void_p(out.ptr), al.ctypes.data,
                                            be.ctypes.data, stream_ptr(self.device)))
        return out

    def __del__(self):
        try:
            if self.h:
                lib().qltg_axis_plan_destroy(self.h)
        except Exception:
            pass


def ApplyAxisMonomial(t: DTensor, axis: int, out_leg: Leg, flux, entries, coefs, alpha=1.0, beta=0.0,
                      out: Optional[DTensor] = None) -> DTensor:
    """qlten::dmrg::ApplyAxisMonomial (axis_ops.h:2746-2860)."""
    return AxisMonomialPlan(t.meta, axis, out_leg, flux, entries, coefs, t.device).execute(t, alpha, beta, out)


def ApplyRank2ToAxisPreserveOrder(t: DTensor, op: DTensor, axis: int, mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyRank2ToAxisPreserveOrder (axis_ops.h:2862-2993)."""
    return AxisRank2Plan(t.meta, op.meta, axis, device=t.device).execute(t, op, mode=mode)


def ApplyTwoRank2ToAxesPreserveOrder(t: DTensor, op1: DTensor, axis1: int, op2: DTensor, axis2: int,
                                     mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyTwoRank2ToAxesPreserveOrder (axis_ops.h:2995-3126)."""
    plan = AxisRank2Plan(t.meta, op1.meta, axis1, op2.meta, axis2, device=t.device)
    return plan.execute(t, op1, op2, mode=mode)


class AxisProjectPlan(AxisMonomialPlan):
    """Planned qlten::dmrg::ProjectAxis (axis_ops.h:2469-2532): `kept[s]` lists the input
    degeneracy offsets of sector s kept (in output order); sectors keeping none leave the
    output index."""

    def __init__(self, t: BSTensor, axis: int, kept: Sequence[Sequence[int]], device: int = 0):
        self.h = None
        leg = t.legs[axis]
        if len(kept) != leg.nsct:
            raise ValueError("one kept list per sector of the axis")
        self.ctx = context(device)
        self.device = device
        counts = np.asarray([len(k) for k in kept], np.int64)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(k, np.int64) for k in kept] + [np.zeros(0, np.int64)]))
        dt = _Desc(t)
        h = C.c_void_p()
        check(lib().qltg_axis_project_plan_create(self.ctx.h, dt.ref, int(axis), counts.ctypes.data,
                                                  flat.ctypes.data if flat.size else None, C.byref(h)))
        self.h = h
        keep = counts > 0
        legs = list(t.legs)
        legs[axis] = Leg(leg.dir, leg.qns[keep], counts[keep], leg.parity_comp)
        self.result = _result_meta(h, lib().qltg_axis_plan_result, lib().qltg_axis_plan_result_blocks, legs, t.dtype)

    def execute(self, t: DTensor, out: Optional[DTensor] = None) -> DTensor:
        return super().execute(t, 1.0, 0.0, out)


def ProjectAxis(t: DTensor, axis: int, kept: Sequence[Sequence[int]]) -> DTensor:
    """qlten::dmrg::ProjectAxis (axis_ops.h:2469-2532)."""
    return AxisProjectPlan(t.meta, axis, kept, t.device).execute(t)


class LinearCombinePlan:
    """Planned LinearCombine (tensor_manipulation/ten_linear_combine.h:33-197):
    out = sum_i coefs[i] T_i + beta res over the union of the contributing tensors' blocks
    (res joins when beta != 0, or always with keep_res)."""

    def __init__(self, coefs, metas: Sequence[BSTensor], beta=0.0, res: Optional[BSTensor] = None,
                 keep_res: bool = False, device: int = 0):
        self.h = None
        self.device = device
        self.n = len(metas)
        cplx = metas[0].is_complex
        if len(coefs) != len(metas):
            raise ValueError("one coefficient per tensor")
        if not cplx and (np.iscomplexobj(np.asarray(coefs)) and np.any(np.imag(coefs) != 0)
                         or np.imag(complex(beta)) != 0):
            raise ValueError("complex coefficients for real tensors")
        cf = _axis_values(np.real_if_close(np.asarray(coefs)) if not cplx else np.asarray(coefs), cplx)
        be = _axis_values(np.asarray([beta if cplx else complex(beta).real]), cplx)
        self._descs = [_Desc(m) for m in metas]
        arr = (C.POINTER(capi.TensorDesc) * self.n)(*[C.pointer(d.s) for d in self._descs])
        rd = _Desc(res) if res is not None else None
        h = C.c_void_p()
        check(lib().qltg_lincomb_plan_create(context(device).h, self.n, C.cast(arr, C.c_void_p), cf.ctypes.data,
                                             rd.ref if rd is not None else None, be.ctypes.data, int(keep_res),
                                             C.byref(h)))
        self.h = h
        self.result = _result_meta(h, lib().qltg_lincomb_plan_result, lib().qltg_lincomb_plan_result_blocks,
                                   metas[0].legs, metas[0].dtype)

    def execute(self, tens: Sequence[DTensor], res: Optional[DTensor] = None,
                out: Optional[DTensor] = None) -> DTensor:
        if out is None:
            out = DTensor.empty(self.result, self.device)
        ptrs = (C.c_void_p * self.n)(*[C.c_void_p(t.ptr) for t in tens])
        check(lib().qltg_lincomb_exec(self.h, C.cast(ptrs, C.c_void_p), C.c_void_p(res.ptr) if res is not None else None,
                                      C.c_void_p(out.ptr), stream_ptr(self.device)))
        return out

    def __del__(self):
        try:
            if self.h:
                lib().qltg_lincomb_plan_destroy(self.h)
        except Exception:
            pass


def LinearCombine(coefs, tens: Sequence[DTensor], beta=0.0, res: Optional[DTensor] = None,
                  keep_res: bool = False) -> DTensor:
    """LinearCombine (ten_linear_combine.h:186-197). Written into res's buffer when the result
    has res's topology (res then is the returned tensor), else into a new tensor."""
    plan = LinearCombinePlan(coefs, [t.meta for t in tens], beta, res.meta if res is not None else None, keep_res,
                             tens[0].device)
    same = res is not None and np.array_equal(plan.result.coords, res.meta.coords)
    out = plan.execute(tens, res, res if same else None)
    if same:
        res.meta = plan.result
    return out


def AddScaledAssign(y: DTensor, alpha, x: DTensor) -> DTensor:
    """y += alpha x (ten_linear_combine.h:211-221): in place unless x has blocks y lacks."""
    return LinearCombine([alpha], [x], 1.0, y)


def ApplyAxisDiagonalPreserveOrder(t: DTensor, axis: int, values, in_place: bool = False) -> DTensor:
    """qlten::dmrg::ApplyAxisDiagonalPreserveOrder (axis_ops.h:2584-2637): out of place, or
    in place (the reference's consume-owned storage mode)."""
    return ApplyAxisDiagonalInPlace(t, axis, values) if in_place else ApplyAxisDiagonal(t, axis, values)


def ScaleAxisSectorsInPlace(t: DTensor, axis: int, values_by_sector) -> DTensor:
    """qlten::dmrg::ScaleAxisSectorsInPlace (axis_ops.h:2639-2675)."""
    return ApplyAxisSectorScalars(t, axis, values_by_sector, out=t)


def ApplyAxisSectorScalarsPreserveOrder(t: DTensor, axis: int, values_by_sector, in_place: bool = False) -> DTensor:
    """qlten::dmrg::ApplyAxisSectorScalarsPreserveOrder (axis_ops.h:2677-2744)."""
    return ApplyAxisSectorScalars(t, axis, values_by_sector, out=t if in_place else None)


def ApplyRank2ThenAxisDiagonalPreserveOrder(t: DTensor, op: DTensor, rank2_axis: int, diagonal_axis: int, values,
                                            mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyRank2ThenAxisDiagonalPreserveOrder (axis_ops.h:3128-3151)."""
    return ApplyAxisDiagonalInPlace(ApplyRank2ToAxisPreserveOrder(t, op, rank2_axis, mode), diagonal_axis, values)


def ApplyRank2ThenAxisSectorScalarsPreserveOrder(t: DTensor, op: DTensor, rank2_axis: int, scale_axis: int,
                                                 values_by_sector, mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyRank2ThenAxisSectorScalarsPreserveOrder (axis_ops.h:3153-3180)."""
    return ScaleAxisSectorsInPlace(ApplyRank2ToAxisPreserveOrder(t, op, rank2_axis, mode), scale_axis,
                                   values_by_sector)


def ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder(t: DTensor, op: DTensor, rank2_axis: int,
                                                                   scale_axis: int, values_by_sector, alpha, beta,
                                                                   out: Optional[DTensor] = None,
                                                                   mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder
    (axis_ops.h:3182-3283): out = beta out + alpha S(R(t)), R on axis 0 or the last axis, S the
    sector scalars. An existing out keeps its blocks and gains the ones R produces; a missing
    out needs beta == 0. Returns out (updated in place when no block was added) or the
    expanded result."""
    if rank2_axis not in (0, t.meta.rank - 1):
        raise ValueError("rank2_axis must be axis 0 or the last axis")
    if out is None and complex(beta) != 0:
        raise ValueError("beta != 0 needs an existing output")
    r = ApplyRank2ThenAxisSectorScalarsPreserveOrder(t, op, rank2_axis, scale_axis, values_by_sector, mode)
    if out is None:
        return r if complex(alpha) == 1 else LinearCombine([alpha], [r])
    return LinearCombine([alpha], [r], beta, out, keep_res=True)


def ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder(t: DTensor, op: DTensor, rank2_axis: int,
                                                              scale_axis: int, values_by_sector,
                                                              mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyBoundaryRank2ThenAxisSectorScalarsFusedPreserveOrder (axis_ops.h:3285-3318)."""
    return ApplyBoundaryRank2ThenAxisSectorScalarsAccumulatePreserveOrder(t, op, rank2_axis, scale_axis,
                                                                          values_by_sector, 1.0, 0.0, None, mode)


def ApplyRank2ThenAxisMonomialFusedPreserveOrder(t: DTensor, op: DTensor, rank2_axis: int, monomial_axis: int,
                                                 out_leg: Leg, flux, entries, coefs, mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyRank2ThenAxisMonomialFusedPreserveOrder (axis_ops.h:3320-3503)."""
    r = ApplyRank2ToAxisPreserveOrder(t, op, rank2_axis, mode)
    return ApplyAxisMonomial(r, monomial_axis, out_leg, flux, entries, coefs)


def ApplyTwoRank2ThenAxisDiagonalPreserveOrder(t: DTensor, op1: DTensor, axis1: int, op2: DTensor, axis2: int,
                                               diagonal_axis: int, values, mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyTwoRank2ThenAxisDiagonalPreserveOrder (axis_ops.h:3505-3532)."""
    r = ApplyTwoRank2ToAxesPreserveOrder(t, op1, axis1, op2, axis2, mode)
    return ApplyAxisDiagonalInPlace(r, diagonal_axis, values)


def ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder(t: DTensor, op1: DTensor, axis1: int, op2: DTensor, axis2: int,
                                                    scale_axis: int, values_by_sector, mode="fp64") -> DTensor:
    """qlten::dmrg::ApplyTwoRank2ThenAxisSectorScalarsPreserveOrder (axis_ops.h:3534-3561)."""
    r = ApplyTwoRank2ToAxesPreserveOrder(t, op1, axis1, op2, axis2, mode)
    return ScaleAxisSectorsInPlace(r, scale_axis, values_by_sector)


def MoveHeadAxisToTail(t: DTensor) -> DTensor:
    """qlten::dmrg::MoveHeadAxisToTail (axis_ops.h:3563-3678): axis 0 becomes the last axis
    (bosonic); a rank-1 tensor is copied."""
    if t.meta.rank == 0:
        raise ValueError("input rank must be positive")
    if t.meta.fermionic:
        raise ValueError("MoveHeadAxisToTail is bosonic-only")
    return Transpose(t, list(range(1, t.meta.rank)) + [0])


def selftest_bounded_wait(limit_cycles: int = 1 << 21, device: int = 0) -> None:
    """Run the device-side bounded-wait self-test (qltg_selftest_bounded_wait): raises
    QltgError with code QLTG_ERR_TIMEOUT when the wait gave up as designed."""
    check(lib().qltg_selftest_bounded_wait(context(device).h, int(limit_cycles), stream_ptr(device)))


def read_qlten(path: str, qn: str = "U1QN", dtype: str = "f64", device: int = 0) -> DTensor:
    """Read a .qlten file (the reference's QLTensor stream format) straight into device
    memory: header parsed in libqltg.so, raw buffer through a pinned staging buffer."""
    from .qlten_io import QltenFile
    f = QltenFile(path, qn, dtype)
    try:
        meta = BSTensor(f.meta.legs, f.meta.coords, f.meta.dtype, None, offsets=f.meta.offsets, size=f.meta.size)
        out = DTensor.empty(meta, device)
        check(lib().qltg_qlten_read_data(f.h, C.c_void_p(out.ptr), 1, stream_ptr(device)))
        return out
    finally:
        f.close()


def write_qlten(path: str, t: DTensor) -> None:
    """Write a device tensor as a .qlten file the reference reads with operator>>."""
    d = _Desc(t.meta)
    check(lib().qltg_qlten_write(path.encode(), d.ref, C.c_void_p(t.ptr), 1, stream_ptr(t.device)))


def _transposed_meta(m: BSTensor, perm: Sequence[int]) -> BSTensor:
    legs = [m.legs[i] for i in perm]
    coords = m.coords[:, perm]
    idx = np.zeros(m.nblk, np.int64)
    for l, leg in enumerate(legs):
        idx = idx * leg.nsct + coords[:, l]
    order = np.argsort(idx, kind="stable")
    return BSTensor(legs, coords[order], m.dtype, None)


class TransposePlan:
    """A reusable Transpose for one tensor layout and permutation: the block work list is
    built once; `execute` is one asynchronous kernel launch."""

    def __init__(self, meta: BSTensor, perm: Sequence[int], device: int = 0):
        self.perm = [int(x) for x in perm]
        self.device = device
        self.meta = meta
        self.result = _transposed_meta(meta, self.perm)
        d = _Desc(meta)
        p = np.asarray(self.perm, np.int32)
        h = C.c_void_p()
        check(lib().qltg_transpose_plan_create(context(device).h, d.ref, p.ctypes.data, stream_ptr(device),
                                               C.byref(h)))
        self.h = h

    def execute(self, t: DTensor, out: Optional[DTensor] = None) -> DTensor:
        if out is None:
            out = DTensor.empty(self.result, self.device)
        check(lib().qltg_transpose_plan_exec(self.h, C.c_void_p(t.ptr), C.c_void_p(out.ptr),
                                             stream_ptr(self.device)))
        return out

    def __del__(self):
        try:
            if self.h:
                lib().qltg_transpose_plan_destroy(self.h)
        except Exception:
            pass


def Transpose(t: DTensor, perm: Sequence[int]) -> DTensor:
    """QLTensor::Transpose with fermionic block signs (qltensor/qltensor_impl.h:448-464)."""
    perm = [int(x) for x in perm]
    m = t.meta
    meta = _transposed_meta(m, perm)
    out = DTensor.empty(meta, t.device)
    d = _Desc(m)
    p = np.asarray(perm, np.int32)
    check(lib().qltg_transpose(context(t.device).h, d.ref, C.c_void_p(t.ptr), p.ctypes.data,
                               C.c_void_p(out.ptr), stream_ptr(t.device)))
    return out


class Matvec:
    """The two-site effective Hamiltonian H_eff = lenv . mpo1 . mpo2 . renv as one CUDA graph."""

    def __init__(self, lenv: DTensor, psi_meta: BSTensor, mpo1: DTensor, mpo2: DTensor, renv: DTensor,
                 mode="fp64"):
        self.device = lenv.device
        self.ctx = context(self.device)
        self._keep = (lenv, mpo1, mpo2, renv)
        ds = [_Desc(x) for x in (lenv.meta, psi_meta, mpo1.meta, mpo2.meta, renv.meta)]
        h = C.c_void_p()
        check(lib().qltg_matvec_create(self.ctx.h, ds[0].ref, C.c_void_p(lenv.ptr), ds[1].ref, ds[2].ref,
                                       C.c_void_p(mpo1.ptr), ds[3].ref, C.c_void_p(mpo2.ptr), ds[4].ref,
                                       C.c_void_p(renv.ptr), _mode(mode), stream_ptr(self.device), C.byref(h)))
        self.h = h
        nblk, size = C.c_int64(), C.c_int64()
        check(lib().qltg_matvec_result(h, C.byref(nblk), C.byref(size)))
        coords = np.zeros(max(nblk.value * 4, 1), np.int64)
        offs = np.zeros(max(nblk.value, 1), np.int64)
        check(lib().qltg_matvec_result_blocks(h, coords.ctypes.data, offs.ctypes.data))
        legs = [lenv.meta.legs[2], mpo1.meta.legs[2], mpo2.meta.legs[2], renv.meta.legs[2]]
        self.result = BSTensor(legs, coords[: nblk.value * 4].reshape(-1, 4), psi_meta.dtype, None,
                               offsets=offs[: nblk.value])

    def stats(self) -> Tuple[float, int]:
        f, n = C.c_double(), C.c_int64()
        check(lib().qltg_matvec_stats(self.h, C.byref(f), C.byref(n)))
        return f.value, n.value

    def mpo_form(self) -> dict:
        """Whether the two MPO steps run fused (t1 . W12), whether they can, and the MPO part's
        time in both forms as measured at creation (ms)."""
        fused, fusable = C.c_int32(), C.c_int32()
        ms = np.zeros(2, np.float32)
        check(lib().qltg_matvec_mpo_form(self.h, C.byref(fused), C.byref(fusable), ms.ctypes.data))
        return {"fused": bool(fused.value), "fusable": bool(fusable.value),
                "ms_two_steps": round(float(ms[0]), 4), "ms_fused": round(float(ms[1]), 4)}

    def set_mpo_form(self, fused: bool) -> None:
        check(lib().qltg_matvec_set_mpo_form(self.h, 1 if fused else 0, stream_ptr(self.device)))

    def schedules(self) -> List[dict]:
        """Per contraction step, the GEMM schedule the tuner chose at creation."""
        out = []
        for step in range(4):
            rows, stack, st = C.c_int32(), C.c_int32(), C.c_int64()
            tuned = np.zeros(2, np.int32)
            ms = np.zeros(4, np.float32)
            uf = C.c_double()
            check(lib().qltg_matvec_schedule(self.h, step, C.byref(rows), C.byref(stack), tuned.ctypes.data,
                                             ms.ctypes.data, C.byref(st), C.byref(uf)))
            out.append({"f64_tile_rows": rows.value, "split_stack": bool(stack.value),
                        "tuned": {"fp64": bool(tuned[0]), "split": bool(tuned[1])},
                        "tuned_ms": {"fp64": [round(float(ms[0]), 4), round(float(ms[1]), 4)],
                                     "split": [round(float(ms[2]), 4), round(float(ms[3]), 4)]},
                        "split_tile_stages": st.value, "split_useful_frac": round(uf.value, 4)})
        return out

    def apply(self, psi: DTensor, out: Optional[DTensor] = None) -> DTensor:
        if out is None:
            out = DTensor.empty(self.result, self.device)
        check(lib().qltg_matvec_apply(self.h, C.c_void_p(psi.ptr), C.c_void_p(out.ptr),
                                      stream_ptr(self.device)))
        return out

    def apply_host(self, psi_host: torch.Tensor, out_host: torch.Tensor) -> torch.Tensor:
        """H_eff psi with page-locked host buffers (torch `pin_memory()` tensors of float64 raw
        data): psi copied in, the product, the result copied out. Asynchronous on the device's
        current stream."""
        for t in (psi_host, out_host):
            if t.is_cuda or not t.is_pinned() or t.dtype != torch.float64:
                raise ValueError("host buffers must be pinned float64 CPU tensors")
        n = self.result.size * (2 if self.result.is_complex else 1)
        if out_host.numel() < n:
            raise ValueError("output buffer smaller than the result")
        check(lib().qltg_matvec_apply_host(self.h, C.c_void_p(psi_host.data_ptr()), C.c_void_p(out_host.data_ptr()),
                                           stream_ptr(self.device)))
        return out_host

    def apply_raw(self, psi_ptr: int, out_ptr: int, stream: Optional[int] = None) -> None:
        s = stream_ptr(self.device) if stream is None else C.c_void_p(stream)
        check(lib().qltg_matvec_apply(self.h, C.c_void_p(psi_ptr), C.c_void_p(out_ptr), s))

    def device_status(self) -> None:
        check(lib().qltg_matvec_device_status(self.h, stream_ptr(self.device)))

    def __del__(self):
        try:
            if self.h:
                lib().qltg_matvec_destroy(self.h)
        except Exception:
            pass


class Lanczos:
    """Lanczos on a `Matvec` (real FP64 or complex128, plain or split precision) with the
    Krylov vectors and all vector operations on the device (full reorthogonalisation, FP64;
    complex dots conjugate their first argument); one CUDA graph per step. The lowest Ritz
    value after each step comes from the tridiagonal matrix (host FP64)."""

    def __init__(self, mv: Matvec, max_iter: int = 20):
        self.mv = mv
        self.max_iter = int(max_iter)
        h = C.c_void_p()
        check(lib().qltg_lanczos_create(mv.h, self.max_iter, C.byref(h)))
        self.h = h

    def start(self, psi0: DTensor) -> None:
        check(lib().qltg_lanczos_start(self.h, C.c_void_p(psi0.ptr), stream_ptr(self.mv.device)))

    def step(self, n: int = 1) -> None:
        for _ in range(n):
            check(lib().qltg_lanczos_step(self.h, stream_ptr(self.mv.device)))

    def coeffs(self):
        """(alpha[0:n], beta[0:n+1]) after n steps; beta[0] = ||psi0||."""
        n = C.c_int32()
        a = np.zeros(self.max_iter, np.float64)
        b = np.zeros(self.max_iter + 1, np.float64)
        check(lib().qltg_lanczos_coeffs(self.h, C.byref(n), a.ctypes.data, b.ctypes.data,
                                        stream_ptr(self.mv.device)))
        return a[: n.value].copy(), b[: n.value + 1].copy()

    @staticmethod
    def ritz_lowest(alpha: np.ndarray, beta: np.ndarray) -> np.ndarray:
        """Lowest eigenvalue of the leading k x k tridiagonal matrix, k = 1 .. len(alpha)."""
        out = []
        for k in range(1, len(alpha) + 1):
            T = np.diag(alpha[:k]) + np.diag(beta[1:k], 1) + np.diag(beta[1:k], -1)
            out.append(np.linalg.eigvalsh(T)[0])
        return np.asarray(out)

    def run(self, psi0: DTensor, n: int) -> np.ndarray:
        """n steps from psi0; the lowest Ritz value after each step."""
        self.start(psi0)
        self.step(n)
        a, b = self.coeffs()
        return self.ritz_lowest(a, b)

    def vector(self, i: int) -> torch.Tensor:
        """Krylov vector v_i as a float64 (complex128 for a complex matvec) CUDA tensor viewing
        the device buffer (no copy)."""
        p = C.c_void_p()
        check(lib().qltg_lanczos_vector(self.h, int(i), C.byref(p)))
        cplx = self.mv.result.is_complex
        n = self.mv.result.size * (2 if cplx else 1)
        with torch.cuda.device(self.mv.device):
            v = torch.as_tensor(_DevView(p.value, n), device=f"cuda:{self.mv.device}")
        return torch.view_as_complex(v.view(-1, 2)) if cplx else v

    def __del__(self):
        try:
            if self.h:
                lib().qltg_lanczos_destroy(self.h)
        except Exception:
            pass


def _decomp_tensors(h, which_list, device: int, dtype_real_for=()):
    out = []
    for w in which_list:
        info = np.zeros(6, np.int64)
        check(lib().qltg_decomp_tensor_info(h, w, info.ctypes.data))
        rank, ncomp, dt, nblk, size, ts = (int(x) for x in info)
        dirs = np.zeros(max(rank, 1), np.int32)
        nsct = np.zeros(max(rank, 1), np.int32)
        qns = np.zeros(max(ts * ncomp, 1), np.int32)
        dims = np.zeros(max(ts, 1), np.int64)
        coords = np.zeros(max(nblk * rank, 1), np.int64)
        offs = np.zeros(max(nblk, 1), np.int64)
        dev = C.c_void_p()
        check(lib().qltg_decomp_tensor_export(h, w, dirs.ctypes.data, nsct.ctypes.data, qns.ctypes.data,
                                              dims.ctypes.data, coords.ctypes.data, offs.ctypes.data,
                                              C.byref(dev)))
        legs = []
        qp = dp = 0
        for l in range(rank):
            n = int(nsct[l])
            legs.append(Leg(int(dirs[l]), qns[qp:qp + n * ncomp].reshape(n, ncomp), dims[dp:dp + n],
                            -1))
            qp += n * ncomp
            dp += n
        meta = BSTensor(legs, coords[: nblk * rank].reshape(nblk, rank),
                        np.complex128 if dt == capi.QLTG_C128 else np.float64, None,
                        offsets=offs[:nblk])
        t = DTensor.empty(meta, device)
        nel = size * (2 if dt == capi.QLTG_C128 else 1)
        if nel:
            # copy out of the library-owned buffer (device to device, stream ordered)
            t.buf[:nel].copy_(torch.as_tensor(_DevView(dev.value, nel), device=f"cuda:{device}"))
        out.append(t)
    return out


class _DevView:
    """A raw float64 device range exposed through __cuda_array_interface__ (no copy)."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 2, "strides": None}


def _set_parity(ts, parity_comp):
    for t in ts:
        for l in t.meta.legs:
            l.parity_comp = parity_comp
    return ts


def SVD(t: DTensor, ldims: int, lqndiv: Sequence[int], trunc_err: float, Dmin: int, Dmax: int):
    """qlten::SVD (tensor_manipulation/ten_decomp/ten_svd.h:244-263) -> (U, S, Vt, err, D)."""
    d = _Desc(t.meta)
    div = np.asarray(lqndiv, np.int32)
    h = C.c_void_p()
    check(lib().qltg_svd(context(t.device).h, d.ref, C.c_void_p(t.ptr), int(ldims), div.ctypes.data,
                         float(trunc_err), int(Dmin), int(Dmax), stream_ptr(t.device), C.byref(h)))
    try:
        err, D = C.c_double(), C.c_int64()
        check(lib().qltg_decomp_info(h, C.byref(err), C.byref(D)))
        u, s, vt = _set_parity(_decomp_tensors(h, (0, 1, 2), t.device), t.meta.parity_comp)
        torch.cuda.current_stream(t.device).synchronize()
        return u, s, vt, err.value, D.value
    finally:
        lib().qltg_decomp_destroy(h)


def QR(t: DTensor, ldims: int, lqndiv: Sequence[int]):
    """qlten::QR (tensor_manipulation/ten_decomp/ten_qr.h:152-162) -> (Q, R)."""
    d = _Desc(t.meta)
    div = np.asarray(lqndiv, np.int32)
    h = C.c_void_p()
    check(lib().qltg_qr(context(t.device).h, d.ref, C.c_void_p(t.ptr), int(ldims), div.ctypes.data,
                        stream_ptr(t.device), C.byref(h)))
    try:
        q, r = _set_parity(_decomp_tensors(h, (0, 1), t.device), t.meta.parity_comp)
        torch.cuda.current_stream(t.device).synchronize()
        return q, r
    finally:
        lib().qltg_decomp_destroy(h)
