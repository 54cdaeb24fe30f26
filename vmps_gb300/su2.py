"""Two-site contraction and truncated split for SU(2) (and SU(2) x U(1)) MPS: the
non-abelian branches of contract_AA2 and split_AA2 (tensors/DmrgContractions.h:
1870-1927 and 2461-2631) with Biped::truncateSVD (tensors/Biped.h:744-932).

Quantum numbers of SU(2) components are multiplet dimensions q = 2S + 1; blocks hold
reduced matrices.  The recoupling factors are those of symmetry/SU2.h, per SU(2)
component (U(1) components contribute 1):

    coeff_twoSiteGate(q1..q6)  = {q1 q2 q3; q4 q5 q6} sqrt(q3 q6) (-1)^((q1+q2+q4+q5-4)/2)   (:434-441)
    coeff_splitAA(q1..q6)      = {q1 q2 q3; q4 q5 q6} sqrt(q2 q3) (-1)^((q1+q5+q6-3)/2)     (:401-408)
    coeff_splitAA(q1, q2, q3)  = (-1)^((q1-q2-q3-3)/2) sqrt(q1 / q2)                         (:345-351)

The 6j symbols come from the engine's Racah evaluation (vmps_su2_coupling_6j).

contract: V[s12](qin, q2) = sum over qm of coeff_twoSiteGate(qin, q(s1), qm, q(s2), q2,
q(s12)) A1[s1](qin, qm) A2[s2](qm, q2), one FP64 grouped launch of coefficient-scaled
block products on the device (vmps_block_products) or numpy on the host.

split: per middle multiplet Q the matrix M_Q[(ql, sl), (qr, sr)] collects coeff_splitAA *
V[s(sl,sr,q)](ql, qr) over Q in (ql x q(sl)) and (qr x flip(q(sr))); its SVD; the Dmax
largest singular values over all sectors (each one multiplet) above eps_svd times the
largest, renormalised with the multiplet weights dim(Q) sigma^2 (the norm of a reduced
state); A1[s1](ql, Q) = U rows of (ql, s1), A2[s2](Q, qr) = coeff_splitAA(Q, qr, q(s2))
times the (S V^T or V^T) columns of (qr, s2).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .blocks import Blocks, Symmetry
from .mps import site_layout, two_site_layout

_SIXJ: dict = {}


def sixj(args: list) -> list:
    """6j symbols of argument sets (q1..q6, multiplet dimensions), memoised"""
    todo = [a for a in dict.fromkeys(args) if a not in _SIXJ]
    if todo:
        q = np.ascontiguousarray(np.array(todo, dtype=np.int32).reshape(-1, 6))
        out = np.zeros(len(todo))
        N.check(N.lib().vmps_su2_coupling_6j(len(todo), q.ctypes.data_as(N.i32p), out.ctypes.data_as(N.f64p)))
        for a, v in zip(todo, out):
            _SIXJ[a] = float(v)
    return [_SIXJ[a] for a in args]


def _half(n: int) -> int:
    if n % 2:
        raise ValueError("phase exponent of an SU(2) coefficient is not an integer")
    return n // 2


def _sign(n: int) -> float:
    return -1.0 if n % 2 else 1.0


class Recoupling:
    """coefficients of one symmetry, per SU(2) component, with 6j values batched"""

    def __init__(self, sym: Symmetry):
        self.sym = sym
        self.su2 = [i for i, k in enumerate(sym.kinds) if k == "SU2"]

    def degeneracy(self, q) -> int:
        d = 1
        for i in self.su2:
            d *= int(q[i])
        return d

    def two_site_gate(self, rows: list) -> np.ndarray:
        """coeff_twoSiteGate for rows (q1, ..., q6) of QN tuples"""
        out = np.ones(len(rows))
        for i in self.su2:
            args = [tuple(int(q[i]) for q in r) for r in rows]
            six = sixj(args)
            for n, (a, v) in enumerate(zip(args, six)):
                q1, q2, q3, q4, q5, q6 = a
                out[n] *= v * np.sqrt(q3 * q6) * _sign(_half(q1 + q2 + q4 + q5 - 4))
        return out

    def split6(self, rows: list) -> np.ndarray:
        """coeff_splitAA(q1, ..., q6)"""
        out = np.ones(len(rows))
        for i in self.su2:
            args = [tuple(int(q[i]) for q in r) for r in rows]
            six = sixj(args)
            for n, (a, v) in enumerate(zip(args, six)):
                q1, q2, q3, q4, q5, q6 = a
                out[n] *= v * np.sqrt(q2 * q3) * _sign(_half(q1 + q5 + q6 - 3))
        return out

    def split3(self, q1, q2, q3) -> float:
        """coeff_splitAA(q1, q2, q3)"""
        c = 1.0
        for i in self.su2:
            a, b, d = int(q1[i]), int(q2[i]), int(q3[i])
            c *= _sign(_half(a - b - d - 3)) * np.sqrt(a / b)
        return c


def contract_two_sites_su2(sym, A1: Blocks, A2: Blocks, qloc12, qloc34, ctx=None):
    """(V, comb): the SU(2) two-site tensor of A1 A2 in the layout of two_site_layout"""
    nq = sym.nq
    din = {tuple(A1.qin[i]): int(A1.rows[i]) for i in range(A1.n)}
    dout = {tuple(A2.qout[i]): int(A2.cols[i]) for i in range(A2.n)}
    V, comb = two_site_layout(sym, qloc12, qloc34, din, dout, nq)
    a2 = {}
    for j in range(A2.n):
        a2.setdefault((int(A2.leg[j]), tuple(A2.qin[j])), []).append(j)
    prods, rows = [], []
    for i in range(A1.n):
        s1, qin, qm = int(A1.leg[i]), tuple(A1.qin[i]), tuple(A1.qout[i])
        for s2 in range(len(qloc34)):
            for j in a2.get((s2, qm), ()):
                q2 = tuple(A2.qout[j])
                for q12, s12 in comb["index"].get((s1, s2), ()):
                    k = V.find(s12, qin, q2)
                    if k >= 0:
                        prods.append((k, i, j))
                        rows.append((qin, tuple(qloc12[s1]), qm, tuple(qloc34[s2]), q2, tuple(q12)))
    coef = Recoupling(sym).two_site_gate(rows) if rows else np.zeros(0)
    keep = np.abs(coef) >= np.finfo(float).eps
    prods = [p for p, k in zip(prods, keep) if k]
    coef = coef[keep]
    if ctx is not None and getattr(ctx, "device", -1) >= 0 and prods:
        tri = np.ascontiguousarray(np.array(prods, dtype=np.int64).reshape(-1, 3))
        cf = np.ascontiguousarray(coef, dtype=np.float64)
        s_, a, b, c = sym.c_struct(), A1.c_struct(), A2.c_struct(), V.c_struct()
        N.check(N.lib().vmps_block_products(ctx._h, C.byref(s_), C.byref(a), A1.data_ptr(), C.byref(b),
                                            A2.data_ptr(), C.byref(c), V.data_ptr(), len(prods),
                                            tri.ctypes.data_as(N.i64p), cf.ctypes.data_as(N.f64p)))
    else:
        for (k, i, j), c in zip(prods, coef):
            V.block(k)[...] += c * (A1.block(i) @ A2.block(j))
    return V, comb


def split_two_site_su2(V: Blocks, comb, sym, qloc12, qloc34, din, dout, Dmax, move="right", eps_svd=1e-14,
                       renormalise=True):
    """(A1, A2, discarded weight, {Q: kept multiplets}) of the SU(2) two-site tensor V;
    move="right": A1 = U (left-orthonormal), A2 = S V^T; move="left": A1 = U S, A2 = V^T.
    renormalise=False keeps the kept singular values as they are (the truncated state
    keeps its norm instead of getting norm 1)."""
    nq = sym.nq
    rc = Recoupling(sym)
    inv = {}
    for (s1, s3), lst in comb["index"].items():
        for q, s13 in lst:
            inv[s13] = (s1, s3, tuple(q))
    # row (column) blocks of every middle multiplet: (ql, sl) with Q in ql x q(sl), in sorted order
    rows, cols = {}, {}
    for sl, q1 in enumerate(qloc12):
        for ql in sorted(din):
            for Q in sym.fuse(ql, tuple(q1)):
                rows.setdefault(Q, []).append((ql, sl))
    for sr, q3 in enumerate(qloc34):
        for qr in sorted(dout):
            for Q in sym.fuse(qr, sym.flip(tuple(q3))):
                cols.setdefault(Q, []).append((qr, sr))
    roff, coff, shape = {}, {}, {}
    for Q in set(rows) & set(cols):
        r = 0
        for ql, sl in rows[Q]:
            roff[(Q, ql, sl)] = r
            r += din[ql]
        c = 0
        for qr, sr in cols[Q]:
            coff[(Q, qr, sr)] = c
            c += dout[qr]
        shape[Q] = (r, c)
    M = {Q: np.zeros(shape[Q]) for Q in shape}
    entries, args = [], []
    for b in range(V.n):
        sl, sr, q = inv[int(V.leg[b])]
        ql, qr = tuple(V.qin[b]), tuple(V.qout[b])
        for Q in sym.fuse(ql, tuple(qloc12[sl])):
            if Q not in shape or Q not in sym.fuse(qr, sym.flip(tuple(qloc34[sr]))):
                continue
            entries.append((b, Q, ql, sl, qr, sr))
            args.append((ql, qr, q, tuple(qloc34[sr]), tuple(qloc12[sl]), Q))
    fac = rc.split6(args) if args else np.zeros(0)
    for (b, Q, ql, sl, qr, sr), f in zip(entries, fac):
        if abs(f) < np.finfo(float).eps:
            continue
        r0, c0 = roff[(Q, ql, sl)], coff[(Q, qr, sr)]
        blk = V.block(b)
        M[Q][r0:r0 + blk.shape[0], c0:c0 + blk.shape[1]] += f * blk
    svd = {}
    allsv = []
    for Q in sorted(M):
        if min(M[Q].shape) == 0:
            continue
        U, S, Vt = np.linalg.svd(M[Q], full_matrices=False)
        svd[Q] = (U, S, Vt)
        allsv += [(float(s), Q, i) for i, s in enumerate(S)]
    allsv.sort(key=lambda t: -t[0])
    smax = allsv[0][0] if allsv else 0.0
    kept = [t for t in allsv if t[0] > eps_svd * smax][:max(int(Dmax), 0)]
    tot = sum(rc.degeneracy(Q) * s * s for s, Q, _ in allsv)
    kw = sum(rc.degeneracy(Q) * s * s for s, Q, _ in kept)
    disc = max(0.0, tot - kw) / tot if tot > 0 else 0.0
    nkeep = {}
    for _, Q, i in kept:
        nkeep[Q] = max(nkeep.get(Q, 0), i + 1)
    dmid = {Q: n for Q, n in sorted(nkeep.items())}
    norm = np.sqrt(kw) if kw > 0 and renormalise else 1.0
    A1 = site_layout(qloc12, din, dmid, nq, sym)
    A2 = site_layout(qloc34, dmid, dout, nq, sym)
    for i in range(A1.n):
        s1, ql, Q = int(A1.leg[i]), tuple(A1.qin[i]), tuple(A1.qout[i])
        if (Q, ql, s1) not in roff:
            continue
        U, S, _ = svd[Q]
        k = dmid[Q]
        r0 = roff[(Q, ql, s1)]
        X = U[r0:r0 + din[ql], :k]
        if move != "right":
            X = X * (S[:k] / norm)
        A1.block(i)[...] = X
    for j in range(A2.n):
        s2, Q, qr = int(A2.leg[j]), tuple(A2.qin[j]), tuple(A2.qout[j])
        if (Q, qr, s2) not in coff:
            continue
        _, S, Vt = svd[Q]
        k = dmid[Q]
        c0 = coff[(Q, qr, s2)]
        Y = Vt[:k, c0:c0 + dout[qr]]
        if move == "right":
            Y = (S[:k] / norm)[:, None] * Y
        A2.block(j)[...] = rc.split3(Q, qr, tuple(qloc34[s2])) * Y
    return A1, A2, disc, dmid
