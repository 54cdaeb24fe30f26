"""Union pivots: several pivots of one Hamiltonian with different quantum-number
layouts (sectors) as one pivot, so that one grouped HxV launch serves vectors of
all of them.

The reference advances each start vector of a polynomial expansion in its own
sector and layout (polyIter, DmrgLinearAlgebra.h:550-566; one MpsCompressor per
vector, solvers/MpsCompressor.h:1372-1564).  Here every block of part p gets one
more abelian quantum number, a tag equal to p, on its bond legs (the MPO's local
and auxiliary bases carry tag 0), so the task builder never pairs blocks of
different parts: the union's H is block diagonal over the parts and its HxV on
part p equals that part's own HxV.  A union vector holds one vector of each part
side by side; vmps_hxv_multi / vmps_chebyshev_moments_parts then run all parts of
all right-hand sides in one launch per step.
"""
from __future__ import annotations

import numpy as np

from .blocks import Blocks, MpoSite, Symmetry
from .pivot import PivotMatrix2


def tagged_symmetry(sym: Symmetry) -> Symmetry:
    """sym with one more U(1) component, the part tag"""
    return Symmetry(tuple(sym.kinds) + ("U1",))


def _with_tag(q: np.ndarray, tag: int) -> np.ndarray:
    q = np.asarray(q, dtype=np.int32).reshape(len(q), -1)
    return np.concatenate([q, np.full((len(q), 1), tag, dtype=np.int32)], axis=1)


def tag_blocks(B: Blocks, tag: int) -> Blocks:
    """B with the tag appended to its bond quantum numbers (qin, qout); a Tripod's
    middle (MPO auxiliary) quantum number gets tag 0"""
    return Blocks(B.nq + 1, _with_tag(B.qin, tag), _with_tag(B.qout, tag), B.leg, B.rows, B.cols,
                  data=B.data, qmid=None if B.qmid is None else _with_tag(B.qmid, 0), offset=B.offset)


def tag_mpo(W: MpoSite) -> MpoSite:
    """W with tag 0 on its local, operator and auxiliary quantum numbers"""
    t = MpoSite(W.nq + 1, [tuple(q) + (0,) for q in W.qloc], [tuple(q) + (0,) for q in W.qop])
    for i in range(W.nnz):
        t.add(W.s1[i], W.s2[i], W.k[i], tuple(W.qin[i]) + (0,), tuple(W.qout[i]) + (0,), W.row[i], W.col[i], W.val[i])
    return t


def concat_blocks(parts: list) -> Blocks:
    """the blocks of several tables one after the other (data concatenated)"""
    nq = parts[0].nq
    mid = parts[0].qmid is not None
    qin = np.concatenate([b.qin for b in parts])
    qout = np.concatenate([b.qout for b in parts])
    qmid = np.concatenate([b.qmid for b in parts]) if mid else None
    leg = np.concatenate([b.leg for b in parts])
    rows = np.concatenate([b.rows for b in parts])
    cols = np.concatenate([b.cols for b in parts])
    offs, data, base = [], [], 0
    for b in parts:
        offs.append(b.offset + base)
        data.append(b.data)
        base += b.data.size
    return Blocks(nq, qin, qout, leg, rows, cols, data=np.concatenate(data), qmid=qmid, offset=np.concatenate(offs))


class UnionPivot2:
    """PivotMatrix2 over the parts (Lenv_p, Renv_p, V_p), p = 0..P-1, of one two-site
    MPO (W1, W2).  Attributes: H (the union pivot), parts (block-index boundaries of
    the parts in the union layout, for chebyshev_moments(parts=...)), offsets (element
    boundaries of the parts in the union's compact vectors), dims (per part)."""

    def __init__(self, ctx, sym: Symmetry, W1: MpoSite, W2: MpoSite, parts: list):
        if not 1 <= len(parts) <= 8:
            raise ValueError("a union pivot takes 1 to 8 parts")
        if sym.nq >= 4:
            raise ValueError("no quantum-number component left for the tag (at most 4 components)")
        self.sym = tagged_symmetry(sym)
        L = concat_blocks([tag_blocks(Lp, p) for p, (Lp, _, _) in enumerate(parts)])
        R = concat_blocks([tag_blocks(Rp, p) for p, (_, Rp, _) in enumerate(parts)])
        self.V = concat_blocks([tag_blocks(Vp, p) for p, (_, _, Vp) in enumerate(parts)])
        self.H = PivotMatrix2(ctx, self.sym, L, R, tag_mpo(W1), tag_mpo(W2), self.V)
        nb = np.cumsum([0] + [Vp.n for _, _, Vp in parts])
        self.parts = [int(x) for x in nb]
        self.dims = [int(Vp.data.size) for _, _, Vp in parts]
        self.offsets = [int(x) for x in np.cumsum([0] + self.dims)]
        if self.H.dim != self.offsets[-1]:
            raise ValueError("union layout does not concatenate the parts")

    def join(self, vecs: list) -> np.ndarray:
        """one union vector (or a stack: rows) from one vector (stack) per part"""
        return np.concatenate([np.atleast_2d(v) for v in vecs], axis=1) if np.ndim(vecs[0]) == 2 \
            else np.concatenate(vecs)

    def split(self, v: np.ndarray) -> list:
        """the parts of a union vector (or of the rows of a stack)"""
        return [v[..., self.offsets[p]:self.offsets[p + 1]] for p in range(len(self.dims))]

    def chebyshev_moments(self, v0: np.ndarray, nmom: int, a: float, b: float, precision="fp64"):
        """moments of every part of every row of v0: mu[k, p, n]"""
        return self.H.chebyshev_moments(v0, nmom, a, b, precision, parts=self.parts)

    def close(self):
        self.H.close()


def bra_ket_tag(E: Blocks, side: str) -> Blocks:
    """an operator environment between bra (tag 1) and ket (tag 0): an L block's rows are
    the bra's (qin), an R block's rows the ket's (contract_L = Abra^dagger L Aket,
    contract_R = Aket R Abra^dagger); the middle (auxiliary) quantum number carries the
    difference, tag 1"""
    def t(q, v):
        q = np.asarray(q, dtype=np.int32).reshape(len(q), -1)
        return np.concatenate([q, np.full((len(q), 1), v, dtype=np.int32)], axis=1)
    tin, tout = (1, 0) if side == "L" else (0, 1)
    return Blocks(E.nq + 1, t(E.qin, tin), t(E.qout, tout), E.leg, E.rows, E.cols, data=E.data, qmid=t(E.qmid, 1),
                  offset=E.offset)


def aux_tag(W: MpoSite) -> MpoSite:
    """an operator site between the tagged bases: auxiliary quantum numbers tag 1, local and
    operator ones tag 0"""
    t = MpoSite(W.nq + 1, [tuple(q) + (0,) for q in W.qloc], [tuple(q) + (0,) for q in W.qop])
    for i in range(W.nnz):
        t.add(W.s1[i], W.s2[i], W.k[i], tuple(W.qin[i]) + (1,), tuple(W.qout[i]) + (1,), W.row[i], W.col[i], W.val[i])
    return t
