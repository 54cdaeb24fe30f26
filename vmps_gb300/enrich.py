"""Subspace expansion of single-site DMRG (DMRG::BROOM::RICH_SVD), abelian symmetries.

The reference enlarges the bond a single-site step is about to cross before its
SVD (Mps::enrich_right / enrich_left, Mps.h:3181-3600, called from
rightSweepStep / leftSweepStep at Mps.h:2016-2043, 2287-2310):

    moving right at site l:  P[s1](Lin, (qA, qW, b, j)) = alpha * sum w(a, b) L[Lin, Lout, Lmid; a] A[s2](Lout, qA)_(:, j)
                             A'[s1] = [A[s1] | P[s1]] (outgoing bond enlarged), A[l+1]' = [A[l+1]; 0]
    moving left at site l:   P[s1]((qA, qW, a, i), Rout) = alpha * sum w(a, b) A[s2](qA, Rin)_(i, :) R[Rin, Rout, Rmid; b]
                             A'[s1] = [A[s1]; P[s1]] (incoming bond enlarged), A[l-1]' = [A[l-1] | 0]

with w the entries of W[s1][s2][k], qW the auxiliary QN of the MPO bond beside
the enlarged one and qP = qA + qW the enlarged bond's QN.  The MPS is unchanged by
the zero padding; the truncated SVD of A' that follows keeps the Dmax largest
singular values over all sectors and moves S V^T (or U S) into the neighbour, so
the kept bond basis now also spans directions the Hamiltonian reaches from the
state.  Here the products run as one FP64 grouped GEMM on the device
(vmps_block_products) and the truncated SVD is the two-site split
(vmps_two_site_split[_device]) with a trivial partner site.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .blocks import Blocks
from .mps import site_layout, split_two_site


def _aux_dims(aux):
    """sector dimensions of an MPO bond's auxiliary basis (list of (name, QN))"""
    d = {}
    for _, q in aux:
        q = tuple(q)
        d[q] = d.get(q, 0) + 1
    return d


def _block_products(ctx, sym, Atab, Btab, Ctab, prods, coef):
    """C[k] = sum coef * A[i] @ B[j] over prods (k, i, j) on the device"""
    if not prods:
        return
    tri = np.ascontiguousarray(np.array(prods, dtype=np.int64).reshape(-1, 3))
    cf = np.ascontiguousarray(coef, dtype=np.float64)
    s_, a, b, c = sym.c_struct(), Atab.c_struct(), Btab.c_struct(), Ctab.c_struct()
    N.check(N.lib().vmps_block_products(ctx._h, C.byref(s_), C.byref(a), Atab.data_ptr(), C.byref(b), Btab.data_ptr(),
                                        C.byref(c), Ctab.data_ptr(), len(prods), tri.ctypes.data_as(N.i64p),
                                        cf.ctypes.data_as(N.f64p)))


def _add(a, b):
    return tuple(x + y for x, y in zip(a, b))


def enrich_right(ctx, model, mps, l, Lenv, alpha, Dmax, pool=None):
    """Expand bond l+1 (between sites l and l+1) with alpha * L A W, truncate back to at
    most Dmax states, leave site l left-orthonormal; updates mps.A[l], mps.A[l+1] and
    mps.dims[l+1].  Returns the discarded weight."""
    sym, nq, qloc = model.sym, model.sym.nq, model.qloc
    A, W = mps.A[l], model.W[l]
    qaux = _aux_dims(model.aux[l + 1])
    din = {tuple(A.qin[i]): int(A.rows[i]) for i in range(A.n)}
    dout_old = {tuple(A.qout[i]): int(A.cols[i]) for i in range(A.n)}
    dA = dict(dout_old)
    # enlarged outgoing basis: per qP the old states, then sources (qA, qW) in sorted order
    src = {}
    for qA, da in sorted(dA.items()):
        for qW, dw in sorted(qaux.items()):
            src.setdefault(_add(qA, qW), []).append((qA, qW, da, dw))
    dout = dict(dout_old)
    src_off = {}
    for qP, lst in src.items():
        off = dout.get(qP, 0)
        for qA, qW, da, dw in sorted(lst):
            src_off[(qP, qA, qW)] = off
            off += da * dw
        dout[qP] = off
    # expansion sub-blocks: (s1, Lin, qA, qW, b) -> din(Lin) x dA(qA)
    Lkeys = {}
    for i in range(Lenv.n):
        Lkeys.setdefault((tuple(Lenv.qmid[i]), int(Lenv.leg[i])), []).append(i)
    Aby = {}
    for j in range(A.n):
        Aby.setdefault((int(A.leg[j]), tuple(A.qin[j])), []).append(j)
    arr = W.arrays()
    sub, ent, prods, coef = {}, [], [], []
    for e in range(W.nnz):
        s1, s2, a, b = int(arr["s1"][e]), int(arr["s2"][e]), int(arr["row"][e]), int(arr["col"][e])
        Lmid, qW, w = tuple(arr["qin"][e]), tuple(arr["qout"][e]), float(arr["val"][e])
        for i in Lkeys.get((Lmid, a), ()):
            Lin, Lout = tuple(Lenv.qin[i]), tuple(Lenv.qout[i])
            if Lin not in din:
                continue
            for j in Aby.get((s2, Lout), ()):
                qA = tuple(A.qout[j])
                key = (s1, Lin, qA, qW, b)
                k = sub.get(key)
                if k is None:
                    k = sub[key] = len(ent)
                    ent.append((0, Lin, qA, np.zeros((din[Lin], dA[qA]))))
                prods.append((k, i, j))
                coef.append(alpha * w)
    P = Blocks.from_entries(nq, ent) if ent else None
    if P is not None:
        _block_products(ctx, sym, Lenv, A, P, prods, coef)
    # A' = [A | P] in the site layout over (din, dout)
    blocks = []
    Aold = {(int(A.leg[i]), tuple(A.qin[i])): A.block(i) for i in range(A.n)}
    for s1, q1 in enumerate(qloc):
        for qin, dr in sorted(din.items()):
            qP = _add(qin, q1)
            if dout.get(qP, 0) == 0:
                continue
            M = np.zeros((dr, dout[qP]))
            if (s1, qin) in Aold:
                M[:, :dout_old[qP]] = Aold[(s1, qin)]
            blocks.append((s1, qin, qP, M))
    if P is not None:
        pos = {(s1, qin, qP): m for m, (s1, qin, qP, _) in enumerate(blocks)}
        for (s1, Lin, qA, qW, b), k in sub.items():
            qP = _add(Lin, qloc[s1])
            c0 = src_off[(qP, qA, qW)] + b * dA[qA]
            blocks[pos[(s1, Lin, qP)]][3][:, c0:c0 + dA[qA]] += P.block(k)
    V = Blocks.from_entries(nq, [(s1, qin, qP, M) for s1, qin, qP, M in blocks])
    vac = sym.vacuum()
    comb = {"n": len(qloc), "index": {(s1, 0): [(tuple(q1), s1)] for s1, q1 in enumerate(qloc)}}
    A1, A2, disc, dmid = split_two_site(V, comb, qloc, [vac], din, dout, nq, Dmax, move="right", pool=pool, ctx=ctx)
    # the split renormalises the kept singular values; truncateSVD does not (Biped.h:744-932),
    # so S V^T gets back its scale and the state is unchanged when nothing is discarded
    A2.data *= float(np.linalg.norm(V.data)) * np.sqrt(max(0.0, 1.0 - disc))
    # S V^T into site l+1 (only its columns of the old states meet A[l+1]); site l+1 gets
    # the full layout over the new bond basis (zero blocks for sectors the expansion added)
    SV = {tuple(A2.qin[i]): A2.block(i) for i in range(A2.n)}
    Nx = mps.A[l + 1]
    new = site_layout(qloc, dmid, mps.dims[l + 2], nq)
    for i in range(Nx.n):
        q = tuple(Nx.qin[i])
        if q in SV:
            k = new.find(int(Nx.leg[i]), q, tuple(Nx.qout[i]))
            if k >= 0:
                new.block(k)[...] = SV[q][:, :dout_old[q]] @ Nx.block(i)
    mps.A[l] = A1
    mps.A[l + 1] = new
    mps.dims[l + 1] = dmid
    return disc


def enrich_left(ctx, model, mps, l, Renv, alpha, Dmax, pool=None):
    """Expand bond l (between sites l-1 and l) with alpha * A W R, truncate back to at
    most Dmax states, leave site l right-orthonormal; updates mps.A[l-1], mps.A[l] and
    mps.dims[l].  Returns the discarded weight."""
    sym, nq, qloc = model.sym, model.sym.nq, model.qloc
    A, W = mps.A[l], model.W[l]
    qaux = _aux_dims(model.aux[l])
    dout = {tuple(A.qout[i]): int(A.cols[i]) for i in range(A.n)}
    din_old = {tuple(A.qin[i]): int(A.rows[i]) for i in range(A.n)}
    dA = dict(din_old)
    src = {}
    for qA, da in sorted(dA.items()):
        for qW, dw in sorted(qaux.items()):
            src.setdefault(_add(qA, qW), []).append((qA, qW, da, dw))
    din = dict(din_old)
    src_off = {}
    for qP, lst in src.items():
        off = din.get(qP, 0)
        for qA, qW, da, dw in sorted(lst):
            src_off[(qP, qA, qW)] = off
            off += da * dw
        din[qP] = off
    Rkeys = {}
    for i in range(Renv.n):
        Rkeys.setdefault((tuple(Renv.qmid[i]), int(Renv.leg[i])), []).append(i)
    Aby = {}
    for j in range(A.n):
        Aby.setdefault((int(A.leg[j]), tuple(A.qout[j])), []).append(j)
    arr = W.arrays()
    sub, ent, prods, coef = {}, [], [], []
    for e in range(W.nnz):
        s1, s2, a, b = int(arr["s1"][e]), int(arr["s2"][e]), int(arr["row"][e]), int(arr["col"][e])
        qW, Rmid, w = tuple(arr["qin"][e]), tuple(arr["qout"][e]), float(arr["val"][e])
        for i in Rkeys.get((Rmid, b), ()):
            Rin, Rout = tuple(Renv.qin[i]), tuple(Renv.qout[i])
            if Rout not in dout:
                continue
            for j in Aby.get((s2, Rin), ()):
                qA = tuple(A.qin[j])
                key = (s1, qA, qW, a, Rout)
                k = sub.get(key)
                if k is None:
                    k = sub[key] = len(ent)
                    ent.append((0, qA, Rout, np.zeros((dA[qA], dout[Rout]))))
                prods.append((k, j, i))
                coef.append(alpha * w)
    P = Blocks.from_entries(nq, ent) if ent else None
    if P is not None:
        _block_products(ctx, sym, A, Renv, P, prods, coef)
    blocks = []
    Aold = {(int(A.leg[i]), tuple(A.qout[i])): A.block(i) for i in range(A.n)}
    for s3, q3 in enumerate(qloc):
        for qout, dc in sorted(dout.items()):
            qP = tuple(x - y for x, y in zip(qout, q3))
            if din.get(qP, 0) == 0:
                continue
            M = np.zeros((din[qP], dc))
            if (s3, qout) in Aold:
                M[:din_old[qP], :] = Aold[(s3, qout)]
            blocks.append((s3, qP, qout, M))
    if P is not None:
        pos = {(s3, qP, qout): m for m, (s3, qP, qout, _) in enumerate(blocks)}
        for (s1, qA, qW, a, Rout), k in sub.items():
            qP = tuple(x - y for x, y in zip(Rout, qloc[s1]))
            r0 = src_off[(qP, qA, qW)] + a * dA[qA]
            blocks[pos[(s1, qP, Rout)]][3][r0:r0 + dA[qA], :] += P.block(k)
    V = Blocks.from_entries(nq, [(s3, qP, qout, M) for s3, qP, qout, M in blocks])
    vac = sym.vacuum()
    comb = {"n": len(qloc), "index": {(0, s3): [(tuple(q3), s3)] for s3, q3 in enumerate(qloc)}}
    A1, A2, disc, dmid = split_two_site(V, comb, [vac], qloc, din, dout, nq, Dmax, move="left", pool=pool, ctx=ctx)
    A1.data *= float(np.linalg.norm(V.data)) * np.sqrt(max(0.0, 1.0 - disc))   # U S at its own scale
    # U S into site l-1 (only its rows of the old states meet A[l-1]), over the full layout
    US = {tuple(A1.qout[i]): A1.block(i) for i in range(A1.n)}
    Pv = mps.A[l - 1]
    new = site_layout(qloc, mps.dims[l - 1], dmid, nq)
    for i in range(Pv.n):
        q = tuple(Pv.qout[i])
        if q in US:
            k = new.find(int(Pv.leg[i]), tuple(Pv.qin[i]), q)
            if k >= 0:
                new.block(k)[...] = Pv.block(i) @ US[q][:din_old[q], :]
    mps.A[l] = A2
    mps.A[l - 1] = new
    mps.dims[l] = dmid
    return disc
