"""Host-side mirror of the reference's block-sparse tensor metadata.

`BSTensor` carries exactly what `qlten::QLTensor` / `BlockSparseDataTensor` carry for the
contraction and decomposition path (reference qltensor/qltensor.h:60-668,
qltensor/blk_spar_data_ten/blk_spar_data_ten.h:53-572):

* legs (`Index`): direction IN/OUT, quantum-number sectors (QN components per sector)
  and sector degeneracies (qltensor/index.h:45-229, qltensor/qnsct.h:34-139);
* stored blocks as sector coordinates in ascending block index, where the block index is
  the row-major linearisation of the coordinates over the sector counts
  (blk_spar_data_ten.h:380-382, utility/utils_inl.h:125-148);
* one raw buffer with every block row-major over its degeneracy dims at cumulative
  offsets (data_blk_operations.h:137-145).

The raw data may live on the host (`data`, a numpy array) or on the device (`dev`, a
torch CUDA tensor); the GPU library takes device pointers and plain metadata arrays.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

IN, OUT = 0, 1


@dataclass
class Leg:
    """One tensor index: direction, QN per sector (nsct x ncomp) and degeneracies."""

    dir: int
    qns: np.ndarray
    dims: np.ndarray
    parity_comp: int = -1  # QN component whose oddness is the fermion parity; -1 bosonic

    def __post_init__(self):
        self.qns = np.ascontiguousarray(self.qns, dtype=np.int32).reshape(len(self.dims), -1)
        self.dims = np.ascontiguousarray(self.dims, dtype=np.int64)

    @property
    def nsct(self) -> int:
        return int(self.dims.shape[0])

    @property
    def ncomp(self) -> int:
        return int(self.qns.shape[1])

    def inverse(self) -> "Leg":
        return Leg(1 - self.dir, self.qns.copy(), self.dims.copy(), self.parity_comp)

    def parities(self) -> np.ndarray:
        if self.parity_comp < 0:
            return np.zeros(self.nsct, dtype=np.uint8)
        return (self.qns[:, self.parity_comp] % 2 != 0).astype(np.uint8)

    def same_space(self, other: "Leg") -> bool:
        return (self.dir == other.dir and np.array_equal(self.qns, other.qns)
                and np.array_equal(self.dims, other.dims))


@dataclass
class BSTensor:
    legs: List[Leg]
    coords: np.ndarray
    dtype: type = np.float64
    data: Optional[np.ndarray] = None
    dev: object = None  # torch CUDA tensor holding the raw buffer, when resident
    offsets: np.ndarray = field(default=None)
    size: int = 0

    def __post_init__(self):
        r = len(self.legs)
        self.coords = np.ascontiguousarray(self.coords, dtype=np.int64).reshape(-1, r) if r else \
            np.zeros((1 if self.size else 0, 0), dtype=np.int64)
        self.dtype = np.dtype(self.dtype).type
        shapes = self.block_shapes()
        sizes = shapes.prod(axis=1) if r else np.ones(len(self.coords), dtype=np.int64)
        offs = np.zeros(len(sizes), dtype=np.int64)
        if len(sizes):
            offs[1:] = np.cumsum(sizes)[:-1]
        if self.offsets is None:
            self.offsets = offs
        else:
            self.offsets = np.ascontiguousarray(self.offsets, dtype=np.int64)
            if not np.array_equal(self.offsets, offs):
                raise ValueError("block offsets are not cumulative in block order")
        self.size = int(sizes.sum()) if len(sizes) else 0
        if self.data is not None:
            self.data = np.ascontiguousarray(self.data, dtype=self.dtype).reshape(-1)
            if self.data.shape[0] != self.size:
                raise ValueError(f"raw data has {self.data.shape[0]} elements, layout needs {self.size}")

    # ------------------------------------------------------------------ shape queries
    @property
    def rank(self) -> int:
        return len(self.legs)

    @property
    def nblk(self) -> int:
        return int(self.coords.shape[0])

    @property
    def is_complex(self) -> bool:
        return self.dtype == np.complex128

    @property
    def ncomp(self) -> int:
        return self.legs[0].ncomp if self.legs else 1

    @property
    def parity_comp(self) -> int:
        return self.legs[0].parity_comp if self.legs else -1

    @property
    def fermionic(self) -> bool:
        return self.parity_comp >= 0

    def block_shapes(self) -> np.ndarray:
        if not self.legs:
            return np.zeros((len(self.coords), 0), dtype=np.int64)
        cols = [self.legs[l].dims[self.coords[:, l]] for l in range(self.rank)]
        return np.stack(cols, axis=1).astype(np.int64) if len(self.coords) else \
            np.zeros((0, self.rank), dtype=np.int64)

    def blk_idx(self) -> np.ndarray:
        idx = np.zeros(self.nblk, dtype=np.int64)
        for l in range(self.rank):
            idx = idx * self.legs[l].nsct + self.coords[:, l]
        return idx

    def shape(self) -> List[int]:
        return [int(l.dims.sum()) for l in self.legs]

    # ------------------------------------------------------------------ constructors
    @staticmethod
    def from_arrays(dirs, nsct, qns, dims, ncomp, parity_comp, coords, data, is_complex, offsets=None):
        legs = []
        qp = dp = 0
        for l in range(len(dirs)):
            n = int(nsct[l])
            legs.append(Leg(int(dirs[l]), np.asarray(qns[qp:qp + n * ncomp]).reshape(n, ncomp),
                            np.asarray(dims[dp:dp + n]), int(parity_comp)))
            qp += n * ncomp
            dp += n
        dt = np.complex128 if is_complex else np.float64
        d = np.asarray(data, dtype=np.float64)
        if is_complex:
            d = d.view(np.complex128)
        return BSTensor(legs, np.asarray(coords).reshape(-1, len(dirs)) if len(dirs) else
                        np.zeros((1 if d.size else 0, 0), np.int64), dt, d, offsets=offsets,
                        size=int(d.size))

    @staticmethod
    def from_record(rec: dict, prefix: str, parity_comp: Optional[int] = None) -> "BSTensor":
        """Build from a fixture dictionary holding `<prefix>.dirs` ... `<prefix>.data`."""
        g = lambda k: np.asarray(rec[f"{prefix}.{k}"])
        dirs, nsct, dims = g("dirs"), g("nsct"), g("dims")
        ncomp = int(g("ncomp").reshape(-1)[0])
        if parity_comp is None:
            key = f"{prefix}.parity_comp"
            parity_comp = int(np.asarray(rec[key]).reshape(-1)[0]) if key in rec else -1
        data = g("data")
        r = len(dirs)
        if r:
            coords = g("coords").reshape(-1, r)
            dp = np.concatenate([[0], np.cumsum(nsct)]).astype(np.int64)
            sizes = np.ones(len(coords), np.int64)
            for l in range(r):
                sizes *= dims[dp[l] + coords[:, l]]
            nel = int(sizes.sum())
        else:
            coords = np.zeros((0, 0), np.int64)
            nel = 1
        is_complex = nel > 0 and data.size == 2 * nel
        return BSTensor.from_arrays(dirs, nsct, g("qns"), dims, ncomp, parity_comp, coords, data,
                                    is_complex, offsets=g("offsets") if r else None)

    # ------------------------------------------------------------------ dense helpers
    def block(self, b: int) -> np.ndarray:
        shp = tuple(int(x) for x in self.block_shapes()[b])
        o = int(self.offsets[b])
        return self.data[o:o + int(np.prod(shp, dtype=np.int64))].reshape(shp)

    def to_dense(self) -> np.ndarray:
        """Full dense array (small tensors only)."""
        if self.rank == 0:
            return np.asarray(self.data[0] if self.size else 0, dtype=self.dtype)
        starts = [np.concatenate([[0], np.cumsum(l.dims)[:-1]]) for l in self.legs]
        out = np.zeros(self.shape(), dtype=self.dtype)
        for b in range(self.nblk):
            sl = tuple(slice(int(starts[l][self.coords[b, l]]),
                             int(starts[l][self.coords[b, l]] + self.legs[l].dims[self.coords[b, l]]))
                       for l in range(self.rank))
            out[sl] = self.block(b)
        return out

    def meta_arrays(self):
        """Flat metadata arrays (dirs, nsct, qns, dims) for the C interfaces."""
        dirs = np.array([l.dir for l in self.legs], dtype=np.int32)
        nsct = np.array([l.nsct for l in self.legs], dtype=np.int32)
        qns = np.ascontiguousarray(np.concatenate([l.qns.reshape(-1) for l in self.legs])
                                   if self.legs else np.zeros(0), dtype=np.int32)
        dims = np.ascontiguousarray(np.concatenate([l.dims for l in self.legs])
                                    if self.legs else np.zeros(0), dtype=np.int64)
        return dirs, nsct, qns, dims

    def raw_f64(self) -> np.ndarray:
        """The raw buffer viewed as float64 (complex interleaved re, im)."""
        return np.ascontiguousarray(self.data).view(np.float64)

    def copy(self) -> "BSTensor":
        return BSTensor([Leg(l.dir, l.qns.copy(), l.dims.copy(), l.parity_comp) for l in self.legs],
                        self.coords.copy(), self.dtype,
                        None if self.data is None else self.data.copy(), size=self.size)


def same_topology(a: BSTensor, b: BSTensor) -> bool:
    """Bit-exact equality of legs (directions, QN sectors, dims), block set and offsets."""
    if a.rank != b.rank or len(a.legs) != len(b.legs):
        return False
    if not all(x.same_space(y) for x, y in zip(a.legs, b.legs)):
        return False
    return np.array_equal(a.coords, b.coords) and np.array_equal(a.offsets, b.offsets)


def rel_frob(x: np.ndarray, ref: np.ndarray) -> float:
    """Relative Frobenius error ||x - ref|| / ||ref||."""
    x = np.asarray(x).reshape(-1)
    ref = np.asarray(ref).reshape(-1)
    d = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (d if d > 0 else 1.0))
