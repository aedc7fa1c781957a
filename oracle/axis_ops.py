"""CPU restatement of the reference's bosonic DMRG axis primitives (qlten::dmrg, reference
tensor_manipulation/dmrg/axis_ops.h), block by block with numpy. Test infrastructure only:
pinned against the reference's outputs in tests/golden/axis_ops.npz.

  axis_diagonal        ApplyAxisDiagonal (axis_ops.h:2370-2547): out = beta out + alpha D(in),
                       D multiplying every degeneracy slice of `axis` by its value
  axis_sector_scalars  ApplyAxisSectorScalarsPreserveOrder (axis_ops.h:2655-2744): each block
                       times the value of its sector on `axis`
  axis_rank2           ApplyRank2ToAxisPreserveOrder (axis_ops.h:2862-2993): contract `axis`
                       with the operator's index 0, index 1 takes the axis' place
  axis_two_rank2       ApplyTwoRank2ToAxesPreserveOrder (axis_ops.h:2995-3126): op1 on axis1,
                       then op2 on axis2
  axis_monomial        ApplyAxisMonomial (axis_ops.h:2746-2860, topology :2241-2269, slice add
                       :2306-2332): output blocks = input blocks mapped through every entry whose
                       input sector matches; out = beta out + sum over entries of alpha coef
                       (input slice in_offset -> output slice out_offset)
  project_axis         ProjectAxis (axis_ops.h:2469-2532, copy :2337-2363): keep the listed
                       degeneracies of every sector, drop sectors keeping none
  linear_combine       LinearCombine (tensor_manipulation/ten_linear_combine.h:33-197): sum of
                       coef T over the union of the contributing tensors' blocks, res last
The reference's composed forms (axis_ops.h:3128-3561) are these applied in sequence; the
tests compose them the same way.
"""
from typing import Optional, Sequence

import numpy as np

from oracle import oracle
from tensortoolkit_gb300.tensor import BSTensor, Leg


def _sector_starts(leg: Leg) -> np.ndarray:
    return np.concatenate([[0], np.cumsum(leg.dims)[:-1]]).astype(np.int64)


def axis_diagonal(t: BSTensor, axis: int, values: np.ndarray, alpha=1.0, beta=0.0,
                  out: Optional[BSTensor] = None) -> BSTensor:
    """values: one per (sector, degeneracy) of t's `axis`, sectors in index order."""
    starts = _sector_starts(t.legs[axis])
    res = t.copy()
    shapes = t.block_shapes()
    for b in range(t.nblk):
        s = int(t.coords[b, axis])
        v = np.asarray(values[starts[s]:starts[s] + shapes[b, axis]])
        shp = [1] * t.rank
        shp[axis] = -1
        blk = t.block(b) * v.reshape(shp) * alpha
        if beta != 0 and out is not None:
            blk = blk + beta * out.block(b)
        o = int(t.offsets[b])
        res.data[o:o + blk.size] = blk.reshape(-1)
    return res


def axis_sector_scalars(t: BSTensor, axis: int, values_by_sector: Sequence[float]) -> BSTensor:
    res = t.copy()
    for b in range(t.nblk):
        o = int(t.offsets[b])
        n = int(np.prod(t.block_shapes()[b]))
        res.data[o:o + n] *= values_by_sector[int(t.coords[b, axis])]
    return res


def transpose(t: BSTensor, perm: Sequence[int]) -> BSTensor:
    """Bosonic block-sparse transpose: legs and block coordinates permuted, blocks re-sorted
    to ascending block index."""
    legs = [t.legs[p] for p in perm]
    coords = t.coords[:, list(perm)]
    order = np.lexsort(coords.T[::-1]) if t.nblk else np.zeros(0, np.int64)
    coords_s = coords[order]
    res = BSTensor(legs, coords_s, t.dtype, np.zeros(t.size, t.dtype))
    for nb, b in enumerate(order):
        blk = np.transpose(t.block(int(b)), perm)
        o = int(res.offsets[nb])
        res.data[o:o + blk.size] = blk.reshape(-1)
    return res


def axis_rank2(t: BSTensor, op: BSTensor, axis: int) -> BSTensor:
    c, _ = oracle.contract(t, op, [[axis], [0]])
    r = t.rank
    perm = list(range(axis)) + [r - 1] + list(range(axis, r - 1))
    return transpose(c, perm) if axis != r - 1 else c


def axis_two_rank2(t: BSTensor, op1: BSTensor, axis1: int, op2: BSTensor, axis2: int) -> BSTensor:
    return axis_rank2(axis_rank2(t, op1, axis1), op2, axis2)


def axis_monomial(t: BSTensor, axis: int, out_leg: Leg, entries, coefs, alpha=1.0, beta=0.0,
                  out: Optional[BSTensor] = None) -> BSTensor:
    """entries: rows (in_sector, in_offset, out_sector, out_offset)."""
    legs = list(t.legs)
    legs[axis] = out_leg
    ent = np.asarray(entries, np.int64).reshape(-1, 4)
    seen = {}
    for b in range(t.nblk):
        for e in ent:
            if e[0] != t.coords[b, axis]:
                continue
            c = t.coords[b].copy()
            c[axis] = e[2]
            seen.setdefault(tuple(int(x) for x in c), None)
    coords = sorted(seen.keys(), key=lambda c: tuple(c))
    res = BSTensor(legs, np.array(coords, np.int64).reshape(-1, t.rank), t.dtype,
                   np.zeros(0, t.dtype) if not coords else None)
    res.data = np.zeros(res.size, t.dtype)
    pos = {tuple(int(x) for x in res.coords[q]): q for q in range(res.nblk)}
    if beta != 0 and out is not None:
        res.data[:] = beta * out.data
    for b in range(t.nblk):
        blk = t.block(b)
        for e, cf in zip(ent, coefs):
            if e[0] != t.coords[b, axis] or cf == 0:
                continue
            c = t.coords[b].copy()
            c[axis] = e[2]
            q = pos[tuple(int(x) for x in c)]
            o = int(res.offsets[q])
            shp = res.block_shapes()[q]
            ob = res.data[o:o + int(np.prod(shp))].reshape(shp)
            src = np.take(blk, [int(e[1])], axis=axis)
            idx = [slice(None)] * t.rank
            idx[axis] = slice(int(e[3]), int(e[3]) + 1)
            ob[tuple(idx)] += alpha * cf * src
    return res


def project_axis(t: BSTensor, axis: int, kept: Sequence[Sequence[int]]) -> BSTensor:
    leg = t.legs[axis]
    counts = np.asarray([len(k) for k in kept], np.int64)
    new_sct = np.cumsum(counts > 0) - 1
    legs = list(t.legs)
    legs[axis] = Leg(leg.dir, leg.qns[counts > 0], counts[counts > 0], leg.parity_comp)
    keep_blk = [b for b in range(t.nblk) if counts[t.coords[b, axis]] > 0]
    coords = t.coords[keep_blk].copy()
    coords[:, axis] = new_sct[coords[:, axis]]
    res = BSTensor(legs, coords.reshape(-1, t.rank), t.dtype)
    data = [t.block(b).take(np.asarray(kept[t.coords[b, axis]], np.int64), axis=axis).reshape(-1) for b in keep_blk]
    res.data = np.concatenate(data) if data else np.zeros(0, t.dtype)
    return res


def linear_combine(coefs, tens: Sequence[BSTensor], beta=0.0, res: Optional[BSTensor] = None,
                   keep_res: bool = False) -> BSTensor:
    srcs = [(c, t) for c, t in zip(coefs, tens) if c != 0]
    if res is not None and beta != 0:
        srcs.append((beta, res))
    topo = [t for _, t in srcs] + ([res] if res is not None and keep_res else [])
    ref = tens[0]
    blocks = {}
    for t in topo:
        for b in range(t.nblk):
            blocks.setdefault(int(t.blk_idx()[b]), t.coords[b])
    keys = sorted(blocks)
    out = BSTensor(ref.legs, np.array([blocks[k] for k in keys], np.int64).reshape(-1, ref.rank), ref.dtype)
    out.data = np.zeros(out.size, ref.dtype)
    pos = {int(k): q for q, k in enumerate(out.blk_idx())}
    for c, t in srcs:
        idx = t.blk_idx()
        for b in range(t.nblk):
            q = pos[int(idx[b])]
            o = int(out.offsets[q])
            out.data[o:o + t.block(b).size] += c * t.block(b).reshape(-1)
    return out
