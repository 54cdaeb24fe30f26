"""Flat block-sparse containers (host side) and their C-ABI views.

``Blocks`` is the Python counterpart of the ``vmps_blocks`` table: one row per
dense block, all blocks stored column-major in one float64 array.

* a site tensor ``vector<Biped> A`` (tensors/Biped.h:62-320) or a
  ``PivotVector::data`` (pivot/DmrgPivotVector.h:8-117): ``leg`` = physical
  index s, block = ``A[s].block[q]``;
* a ``Tripod`` = ``Multipede<3>`` (tensors/Multipede.h:30-236): ``leg`` = MPO
  auxiliary index a, ``qmid`` = middle QN, block = ``T.block[q][a][0]``.

``MpoSite`` mirrors ``W[s1][s2][k]`` = ``Biped<Symmetry,SparseMatrix>``
(MpoTerms.h:1175-1232) as a COO list.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

QN = tuple  # tuple of ints


@dataclass
class Symmetry:
    """Component kinds: 'U1' (additive) or 'SU2' (q = 2S+1)."""
    kinds: tuple = ("U1",)

    @property
    def nq(self) -> int:
        return len(self.kinds)

    @property
    def nonabelian(self) -> bool:
        return "SU2" in self.kinds

    def vacuum(self) -> QN:
        return tuple(1 if k == "SU2" else 0 for k in self.kinds)

    def fuse(self, a: QN, b: QN) -> list:
        out = [()]
        for i, k in enumerate(self.kinds):
            if k == "U1":
                vals = [a[i] + b[i]]
            else:
                vals = list(range(abs(a[i] - b[i]) + 1, a[i] + b[i], 2))
            out = [q + (v,) for q in out for v in vals]
        return out

    def flip(self, a: QN) -> QN:
        return tuple(-x if k == "U1" else x for x, k in zip(a, self.kinds))

    def dot_weight(self, q: QN) -> float:
        w = 1.0
        for x, k in zip(q, self.kinds):
            if k == "SU2":
                w *= x
        return w

    def c_struct(self) -> N.vmps_symmetry:
        s = N.vmps_symmetry()
        s.nq = self.nq
        for i, k in enumerate(self.kinds):
            s.kind[i] = N.SYM_SU2 if k == "SU2" else N.SYM_U1
        return s


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


class Blocks:
    """Block-sparse tensor: table + compact column-major data."""

    def __init__(self, nq, qin, qout, leg, rows, cols, data=None, qmid=None, offset=None):
        self.nq = nq
        self.qin = _i32(np.reshape(qin, (-1, nq)))
        self.qout = _i32(np.reshape(qout, (-1, nq)))
        self.qmid = None if qmid is None else _i32(np.reshape(qmid, (-1, nq)))
        self.leg = _i32(leg)
        self.rows = _i64(rows)
        self.cols = _i64(cols)
        if offset is None:
            sz = self.rows * self.cols
            offset = np.concatenate([[0], np.cumsum(sz)[:-1]]) if len(sz) else np.zeros(0, np.int64)
        self.offset = _i64(offset)
        total = int((self.offset + self.rows * self.cols).max()) if len(self.rows) else 0
        self.data = np.zeros(total) if data is None else np.ascontiguousarray(data, dtype=np.float64)
        assert self.data.size >= total
        self._dict = None

    # ---- construction -------------------------------------------------------
    @classmethod
    def from_entries(cls, nq, entries, tripod=False):
        """entries: list of (leg, qin, qout, matrix) or (leg, qin, qout, qmid, matrix)."""
        if tripod:
            legs = [e[0] for e in entries]
            qin = [e[1] for e in entries]
            qout = [e[2] for e in entries]
            qmid = [e[3] for e in entries]
            mats = [np.asarray(e[4], dtype=np.float64) for e in entries]
        else:
            legs = [e[0] for e in entries]
            qin = [e[1] for e in entries]
            qout = [e[2] for e in entries]
            qmid = None
            mats = [np.asarray(e[3], dtype=np.float64) for e in entries]
        rows = [m.shape[0] for m in mats]
        cols = [m.shape[1] for m in mats]
        b = cls(nq, np.reshape(np.array(qin, dtype=np.int32), (-1, nq)),
                np.reshape(np.array(qout, dtype=np.int32), (-1, nq)), legs, rows, cols,
                qmid=None if qmid is None else np.reshape(np.array(qmid, dtype=np.int32), (-1, nq)))
        for i, m in enumerate(mats):
            b.block(i)[...] = m
        return b

    def like(self, data=None):
        """Same layout, new data (zeros by default)."""
        return Blocks(self.nq, self.qin, self.qout, self.leg, self.rows, self.cols,
                      data=np.zeros_like(self.data) if data is None else data, qmid=self.qmid, offset=self.offset)

    # ---- access -------------------------------------------------------------
    @property
    def n(self) -> int:
        return len(self.rows)

    def block(self, i) -> np.ndarray:
        r, c, o = int(self.rows[i]), int(self.cols[i]), int(self.offset[i])
        return self.data[o:o + r * c].reshape((r, c), order="F")

    def key(self, i):
        k = (int(self.leg[i]), tuple(self.qin[i]), tuple(self.qout[i]))
        if self.qmid is not None:
            k = k + (tuple(self.qmid[i]),)
        return k

    def find(self, *key):
        if self._dict is None:
            self._dict = {self.key(i): i for i in range(self.n)}
        return self._dict.get(tuple(key), -1)

    def nlegs(self) -> int:
        return int(self.leg.max()) + 1 if self.n else 0

    def norm(self) -> float:
        return float(np.linalg.norm(self.data))

    # ---- C view -------------------------------------------------------------
    def c_struct(self):
        s = N.vmps_blocks()
        s.nblocks = self.n
        s.qin = self.qin.ctypes.data_as(N.i32p)
        s.qout = self.qout.ctypes.data_as(N.i32p)
        s.qmid = self.qmid.ctypes.data_as(N.i32p) if self.qmid is not None else C.cast(None, N.i32p)
        s.leg = self.leg.ctypes.data_as(N.i32p)
        s.rows = self.rows.ctypes.data_as(N.i64p)
        s.cols = self.cols.ctypes.data_as(N.i64p)
        s.offset = self.offset.ctypes.data_as(N.i64p)
        return s

    def data_ptr(self):
        return self.data.ctypes.data_as(N.f64p)


@dataclass
class MpoSite:
    """One MPO site tensor W[s1][s2][k].block[qW](row, col) as COO entries."""
    nq: int
    qloc: list
    qop: list
    s1: list = field(default_factory=list)
    s2: list = field(default_factory=list)
    k: list = field(default_factory=list)
    qin: list = field(default_factory=list)
    qout: list = field(default_factory=list)
    row: list = field(default_factory=list)
    col: list = field(default_factory=list)
    val: list = field(default_factory=list)

    def add(self, s1, s2, k, qin, qout, row, col, val):
        self.s1.append(s1); self.s2.append(s2); self.k.append(k)
        self.qin.append(tuple(qin)); self.qout.append(tuple(qout))
        self.row.append(row); self.col.append(col); self.val.append(float(val))

    @property
    def nnz(self):
        return len(self.val)

    def arrays(self):
        """numpy arrays (cached) used by the C view and by the oracle."""
        if getattr(self, "_arr", None) is None or len(self._arr["val"]) != self.nnz:
            nq = self.nq
            self._arr = dict(
                s1=_i32(self.s1), s2=_i32(self.s2), k=_i32(self.k),
                qin=_i32(np.reshape(np.array(self.qin, dtype=np.int32), (-1, nq))),
                qout=_i32(np.reshape(np.array(self.qout, dtype=np.int32), (-1, nq))),
                row=_i32(self.row), col=_i32(self.col), val=np.ascontiguousarray(self.val, dtype=np.float64),
                qloc=_i32(np.reshape(np.array(self.qloc, dtype=np.int32), (-1, nq))),
                qop=_i32(np.reshape(np.array(self.qop, dtype=np.int32), (-1, nq))))
        return self._arr

    def c_struct(self):
        a = self.arrays()
        s = N.vmps_mpo_site()
        s.nnz = self.nnz
        for name in ("s1", "s2", "k", "qin", "qout", "row", "col"):
            setattr(s, name, a[name].ctypes.data_as(N.i32p))
        s.val = a["val"].ctypes.data_as(N.f64p)
        s.nloc = len(self.qloc)
        s.qloc = a["qloc"].ctypes.data_as(N.i32p)
        s.nop = len(self.qop)
        s.qop = a["qop"].ctypes.data_as(N.i32p)
        return s

    def dense(self, aux_in, aux_out):
        """W as a dense array [a_in, a_out, s1, s2] given the aux bases
        (lists of QNs in global aux order)."""
        nloc = len(self.qloc)
        pos_in, pos_out = _aux_positions(aux_in), _aux_positions(aux_out)
        W = np.zeros((len(aux_in), len(aux_out), nloc, nloc))
        for i in range(self.nnz):
            a = pos_in[(tuple(self.qin[i]), self.row[i])]
            b = pos_out[(tuple(self.qout[i]), self.col[i])]
            W[a, b, self.s1[i], self.s2[i]] += self.val[i]
        return W


def _aux_positions(aux):
    """global aux index of (QN, index within the QN sector)."""
    cnt, pos = {}, {}
    for g, q in enumerate(aux):
        q = tuple(q)
        pos[(q, cnt.get(q, 0))] = g
        cnt[q] = cnt.get(q, 0) + 1
    return pos
