"""Random block-sparse MPS (host-side state layer), abelian or SU(2) bond bases.

The reference initialises an Mps through outerResize/innerResize and
setRandom (Mps.h:1124-1262, :1380-1560, :1639-1665) and grows the bond bases
during its sweeps.  The synthetic states used here fix the bond bases up front:

* the QNs allowed at bond l are those reachable from the left vacuum and from
  the right target Qtot (the quantum-number graph of Mps::outerResize);
* sector dimensions follow either the reference's innerResize rule (Dmax split
  evenly over the sectors, capped by the Hilbert-space count) -- profile
  "even" -- or a Gaussian profile around the mean filling -- profile
  "gaussian", the shape of the Schmidt spectrum of a ground state, used for the
  large-D frozen-site workloads;
* blocks are N(0,1) from a seeded generator, then left-normalised (QR) left of
  the pivot and right-normalised (LQ) right of it.

With SU(2) components the QNs are multiplets q = 2S+1 and fuse by the
Clebsch-Gordan series; blocks are reduced matrices.  Right-normalisation then
weights every block by sqrt(q_out/q_in) before the LQ and removes the weight
after (Mps.h:2664-2692, Symmetry::coeff_leftSweep), so that
sum_{s,qout} (q_out/q_in) A A^dagger = 1 (coeff_rightOrtho); left-normalisation
is a plain QR per outgoing multiplet (Mps.h:2600-2616).
"""
from __future__ import annotations

import math

import numpy as np

from .blocks import Blocks


def _add(a, b):
    return tuple(x + y for x, y in zip(a, b))


def _sub(a, b):
    return tuple(x - y for x, y in zip(a, b))


def _fwd(sym, q, s):
    """QNs reachable from bond QN q through local QN s"""
    return [_add(q, s)] if sym is None else sym.fuse(tuple(q), tuple(s))


def _bwd(sym, q, s):
    """bond QNs q' with q reachable from q' through local QN s"""
    return [_sub(q, s)] if sym is None else sym.fuse(tuple(q), sym.flip(tuple(s)))


def _ortho_weight(sym, qin, qout):
    """sqrt(q_out / q_in) over the SU(2) components (1 for abelian ones)"""
    if sym is None:
        return 1.0
    w = 1.0
    for a, b, k in zip(qin, qout, sym.kinds):
        if k == "SU2":
            w *= b / a
    return math.sqrt(w)


def bond_bases(qloc, L, Qtot, Dmax, profile="even", sigma=None, sym=None):
    """dims[l] : dict QN -> sector dimension at bond l (l = 0..L).  sym = None:
    additive (U(1)-type) QNs; otherwise the symmetry's fusion rules."""
    vac = tuple(0 for _ in Qtot) if sym is None else sym.vacuum()
    # exact Hilbert-space counts from the left and from the right (capped to avoid huge ints)
    cap = 10 ** 12
    fromL = [dict() for _ in range(L + 1)]
    fromL[0][vac] = 1
    for l in range(L):
        for q, n in fromL[l].items():
            for s in qloc:
                for q2 in _fwd(sym, q, s):
                    fromL[l + 1][q2] = min(cap, fromL[l + 1].get(q2, 0) + n)
    fromR = [dict() for _ in range(L + 1)]
    fromR[L][tuple(Qtot)] = 1
    for l in range(L, 0, -1):
        for q, n in fromR[l].items():
            for s in qloc:
                for q2 in _bwd(sym, q, s):
                    fromR[l - 1][q2] = min(cap, fromR[l - 1].get(q2, 0) + n)
    dims = []
    for l in range(L + 1):
        allowed = {q: min(fromL[l][q], fromR[l][q]) for q in fromL[l] if q in fromR[l]}
        if l == 0 or l == L:
            dims.append({q: 1 for q in allowed})
            continue
        qs = sorted(allowed)
        if profile == "even":
            per = max(1, Dmax // len(qs))
            d = {q: min(allowed[q], per) for q in qs}
        else:
            mean = [Qtot[i] * l / L for i in range(len(Qtot))]
            sig = sigma if sigma is not None else [2.5] * len(Qtot)
            w = {q: math.exp(-sum(((q[i] - mean[i]) / sig[i]) ** 2 for i in range(len(q))) / 2.0) for q in qs}
            tot = sum(w.values())
            d = {}
            for q in qs:
                x = int(round(Dmax * w[q] / tot))
                if x > 0:
                    d[q] = min(allowed[q], x)
            if not d:
                q0 = max(qs, key=lambda q: w[q])
                d[q0] = 1
        dims.append(d)
    # make neighbouring bonds consistent: dim_{l+1}(q) <= sum_s dim_l(q - s) and vice versa
    for _ in range(4):
        changed = False
        for l in range(1, L + 1):
            for q in list(dims[l]):
                lim = sum(dims[l - 1].get(qp, 0) for s in qloc for qp in _bwd(sym, q, s))
                if dims[l][q] > lim:
                    changed = True
                    if lim == 0:
                        del dims[l][q]
                    else:
                        dims[l][q] = lim
        for l in range(L - 1, -1, -1):
            for q in list(dims[l]):
                lim = sum(dims[l + 1].get(qn, 0) for s in qloc for qn in _fwd(sym, q, s))
                if dims[l][q] > lim:
                    changed = True
                    if lim == 0:
                        del dims[l][q]
                    else:
                        dims[l][q] = lim
        if not changed:
            break
    return dims


def site_layout(qloc, din, dout, nq, sym=None):
    """Block table of A[s] with blocks (qin -> qout in qin x qloc[s]) present in both bases."""
    ent = []
    for s, qs in enumerate(qloc):
        for qin in sorted(din):
            for qout in _fwd(sym, qin, qs):
                if qout in dout:
                    ent.append((s, qin, qout, din[qin], dout[qout]))
    return Blocks(nq, [e[1] for e in ent], [e[2] for e in ent], [e[0] for e in ent],
                  [e[3] for e in ent], [e[4] for e in ent])


def random_site(qloc, din, dout, nq, rng, sym=None):
    A = site_layout(qloc, din, dout, nq, sym)
    A.data[:] = rng.standard_normal(A.data.size)
    return A


def left_normalize(A, nq, carry=None, sym=None, pool=None):
    """QR per outgoing sector: A -> Q (left-orthonormal), returns (Q, R dict qout->R).
    `carry` (dict qin -> matrix) multiplies the incoming bond first.  `pool`
    (hostla.SectorPool) runs the sector QRs in parallel."""
    A = A.like(A.data.copy())
    if carry is not None:
        for i in range(A.n):
            qin = tuple(A.qin[i])
            A.block(i)[...] = carry[qin] @ A.block(i) if qin in carry else A.block(i)
    groups = {}
    for i in range(A.n):
        groups.setdefault(tuple(A.qout[i]), []).append(i)
    mats = [np.vstack([A.block(i) for i in idx]) for idx in groups.values()]
    qrs = pool.map(np.linalg.qr, mats) if pool is not None else [np.linalg.qr(M) for M in mats]
    Rs = {}
    for (qout, idx), (Q, R) in zip(groups.items(), qrs):
        r0 = 0
        for i in idx:
            r = A.block(i).shape[0]
            A.block(i)[...] = Q[r0:r0 + r]
            r0 += r
        Rs[qout] = R
    return A, Rs


def gauge_step(A, N, nq, move, sym=None, pool=None):
    """One gauge step of a single-site sweep: move="right" makes A left-orthonormal
    (QR per outgoing sector) and multiplies the right neighbour N by R; move="left"
    makes A right-orthonormal (LQ per incoming sector, SU(2) weights as in
    right_normalize) and multiplies the left neighbour N by L.  A and N are updated
    in place, in the native library (vmps_gauge_step, sectors on the pool's threads)
    when numpy's LAPACK can be bound to it, else by left/right_normalize."""
    from .hostla import native_lapack
    if native_lapack():
        import ctypes as C
        from . import _native as N_
        w = None
        if move == "left" and sym is not None and sym.nonabelian:
            w = np.array([_ortho_weight(sym, tuple(A.qin[i]), tuple(A.qout[i])) for i in range(A.n)])
        ab, nb = A.c_struct(), N.c_struct()
        N_.check(N_.lib().vmps_gauge_step(nq, int(move == "right"), C.byref(ab), A.data_ptr(),
                                          w.ctypes.data_as(N_.f64p) if w is not None else C.cast(None, N_.f64p),
                                          C.byref(nb), N.data_ptr(), pool.threads if pool is not None else 1))
        return
    if move == "right":
        Q, Rf = left_normalize(A, nq, sym=sym)
        for i in range(N.n):
            q = tuple(N.qin[i])
            if q in Rf:
                N.block(i)[...] = Rf[q] @ N.block(i)
    else:
        Q, Lf = right_normalize(A, nq, sym=sym)
        for i in range(N.n):
            q = tuple(N.qout[i])
            if q in Lf:
                N.block(i)[...] = N.block(i) @ Lf[q]
    A.data[:] = Q.data


def right_normalize(A, nq, carry=None, sym=None, pool=None):
    """LQ per incoming sector: A -> Q (right-orthonormal), returns (Q, Lfac dict qin->L).
    `carry` (dict qout -> matrix) multiplies the outgoing bond first (A @ carry).
    SU(2) blocks carry the weight sqrt(q_out/q_in) through the LQ.  `pool`
    (hostla.SectorPool) runs the sector QRs in parallel."""
    A = A.like(A.data.copy())
    if carry is not None:
        for i in range(A.n):
            qout = tuple(A.qout[i])
            if qout in carry:
                A.block(i)[...] = A.block(i) @ carry[qout]
    groups = {}
    for i in range(A.n):
        groups.setdefault(tuple(A.qin[i]), []).append(i)
    weights = {qin: [_ortho_weight(sym, qin, tuple(A.qout[i])) for i in idx] for qin, idx in groups.items()}
    mats = [np.hstack([A.block(i) * wi for i, wi in zip(idx, weights[qin])]).T for qin, idx in groups.items()]
    qrs = pool.map(np.linalg.qr, mats) if pool is not None else [np.linalg.qr(M) for M in mats]
    Ls = {}
    for (qin, idx), (Q, R) in zip(groups.items(), qrs):
        w = weights[qin]
        Qt = Q.T
        c0 = 0
        for i, wi in zip(idx, w):
            c = A.block(i).shape[1]
            A.block(i)[...] = Qt[:, c0:c0 + c] / wi
            c0 += c
        Ls[qin] = R.T
    return A, Ls


class RandomMPS:
    """Seeded random MPS, mixed-canonical about a pivot bond range."""

    def __init__(self, model, Qtot, Dmax, seed=1, profile="even", sigma=None):
        self.model = model
        self.L = model.L
        self.nq = model.sym.nq
        self.qloc = model.qloc
        self.Qtot = tuple(Qtot)
        self.sym = model.sym if model.sym.nonabelian else None
        self.dims = bond_bases(model.qloc, model.L, Qtot, Dmax, profile=profile, sigma=sigma, sym=self.sym)
        rng = np.random.default_rng(seed)
        self.A = [random_site(self.qloc, self.dims[l], self.dims[l + 1], self.nq, rng, self.sym)
                  for l in range(self.L)]

    def canonicalize(self, pivot_lo, pivot_hi):
        """Sites < pivot_lo left-normalised, sites > pivot_hi right-normalised;
        the factors are pushed into the pivot sites."""
        carry = None
        for l in range(pivot_lo):
            self.A[l], carry = left_normalize(self.A[l], self.nq, carry, self.sym)
        if carry is not None:
            A = self.A[pivot_lo]
            for i in range(A.n):
                q = tuple(A.qin[i])
                A.block(i)[...] = carry[q] @ A.block(i)
        carry = None
        for l in range(self.L - 1, pivot_hi, -1):
            self.A[l], carry = right_normalize(self.A[l], self.nq, carry, self.sym)
        if carry is not None:
            A = self.A[pivot_hi]
            for i in range(A.n):
                q = tuple(A.qout[i])
                A.block(i)[...] = A.block(i) @ carry[q]
        return self

    def bond_dim(self, l):
        return sum(self.dims[l].values())


def two_site_layout(sym, qloc12, qloc34, din, dout, nq):
    """PivotVector layout of a two-site tensor: leg = combined index s1s3 of
    Qbasis::combine (tensors/Qbasis.h:685-798); QNs of combined states in the
    order the combined basis lists them."""
    comb = combined_basis(sym, qloc12, qloc34)
    qins = sorted(din)
    abelian = not sym.nonabelian
    # the (qin, qout) pairs depend only on the merged QN: made once per distinct one
    pairs = {}
    for qm in comb["q_of"]:
        if qm in pairs:
            continue
        lst = []
        for qin in qins:
            # abelian: the one fused QN is the sum (Symmetry.fuse gives the same)
            for qout in ((tuple(a + b for a, b in zip(qin, qm)),) if abelian else sym.fuse(qin, qm)):
                if qout in dout:
                    lst.append((qin, qout, din[qin], dout[qout]))
        pairs[qm] = lst
    qi, qo, leg, rows, cols = [], [], [], [], []
    for s13, qm in enumerate(comb["q_of"]):
        for qin, qout, r, c in pairs[qm]:
            qi.append(qin)
            qo.append(qout)
            leg.append(s13)
            rows.append(r)
            cols.append(c)
    return Blocks(nq, qi, qo, leg, rows, cols), comb


def combined_basis(sym, q12, q34):
    """Combined basis of two local bases (restating Qbasis::combine + leftOffset
    for bases whose QNs are pairwise distinct or repeated)."""
    def pull(qs):
        distinct, dim, inner = [], [], []
        for q in qs:
            if q not in distinct:
                distinct.append(q)
                dim.append(0)
            d = distinct.index(q)
            inner.append(dim[d])
            dim[d] += 1
        return distinct, dim, inner
    d1, dim1, in1 = pull([tuple(q) for q in q12])
    d2, dim2, in2 = pull([tuple(q) for q in q34])
    hist = {}
    for i, a in enumerate(d1):
        for j, b in enumerate(d2):
            for q in sym.fuse(a, b):
                h = hist.setdefault(q, [])
                if not any(e[0] == a and e[1] == b for e in h):
                    h.append((a, b, dim1[i], dim2[j]))
    for q in hist:
        hist[q].sort(key=lambda e: (e[0], e[1]))
    start, q_of, cur = {}, [], 0
    for q in sorted(hist):
        start[q] = cur
        tot = sum(e[2] * e[3] for e in hist[q])
        q_of += [q] * tot
        cur += tot
    index = {}
    for s1, a in enumerate(q12):
        for s3, b in enumerate(q34):
            for q in sym.fuse(tuple(a), tuple(b)):
                off = 0
                for e in hist[q]:
                    if e[0] == tuple(a) and e[1] == tuple(b):
                        off += in1[s1] + e[2] * in2[s3]
                        break
                    off += e[2] * e[3]
                index.setdefault((s1, s3), []).append((q, start[q] + off))
    return {"q_of": q_of, "index": index, "n": cur}


def contract_two_sites(sym, A1, A2, qloc12, qloc34, nq, return_basis=False, pool=None, ctx=None):
    """Two-site tensor AA[s1s3](qin, qout) = sum_qmid A1[s1](qin,qmid) A2[s3](qmid,qout)
    (abelian case of contract_AA2, tensors/DmrgContractions.h:1870-1927).  With
    abelian QNs every (s1, s3) is one combined state and every A2 block is fixed
    by (s3, qmid), so each two-site block is one product.  return_basis: also
    return the combined basis (for split_two_site); `pool` (hostla.SectorPool)
    runs the block products in parallel on the host; `ctx` (a device Context)
    runs them as one grouped GEMM on the GPU (vmps_two_site_contract)."""
    din = {tuple(A1.qin[i]): int(A1.rows[i]) for i in range(A1.n)}
    dout = {tuple(A2.qout[i]): int(A2.cols[i]) for i in range(A2.n)}
    V, comb = two_site_layout(sym, qloc12, qloc34, din, dout, nq)
    if ctx is not None and getattr(ctx, "device", -1) >= 0 and not sym.nonabelian:
        # the products are found in the native library (vmps_two_site_contract_pairs)
        from . import _native as N
        import ctypes as C
        n1, n3 = len(qloc12), len(qloc34)
        pair = np.full(n1 * n3, -1, dtype=np.int32)
        for (s1, s3), lst in comb["index"].items():
            pair[s1 * n3 + s3] = lst[0][1]
        s_, b1, b2, bv = sym.c_struct(), A1.c_struct(), A2.c_struct(), V.c_struct()
        N.check(N.lib().vmps_two_site_contract_pairs(ctx._h, C.byref(s_), C.byref(b1), A1.data_ptr(), C.byref(b2),
                                                     A2.data_ptr(), C.byref(bv), V.data_ptr(), n1, n3,
                                                     pair.ctypes.data_as(N.i32p)))
        return (V, comb) if return_basis else V
    a2 = {}
    for j in range(A2.n):
        a2.setdefault((int(A2.leg[j]), tuple(A2.qin[j])), []).append(j)
    prods = []
    for i in range(A1.n):
        s1, qin, qmid = int(A1.leg[i]), tuple(A1.qin[i]), tuple(A1.qout[i])
        for s3 in range(len(qloc34)):
            for j in a2.get((s3, qmid), ()):
                qout = tuple(A2.qout[j])
                for _, s13 in comb["index"][(s1, s3)]:
                    k = V.find(s13, qin, qout)
                    if k >= 0:
                        prods.append((k, i, j))
    if ctx is not None and getattr(ctx, "device", -1) >= 0 and prods:
        from . import _native as N
        import ctypes as C
        tri = np.ascontiguousarray(np.array(prods, dtype=np.int64).reshape(-1, 3))
        s_, b1, b2, bv = sym.c_struct(), A1.c_struct(), A2.c_struct(), V.c_struct()
        N.check(N.lib().vmps_two_site_contract(ctx._h, C.byref(s_), C.byref(b1), A1.data_ptr(), C.byref(b2),
                                               A2.data_ptr(), C.byref(bv), V.data_ptr(), len(prods),
                                               tri.ctypes.data_as(N.i64p)))
        return (V, comb) if return_basis else V
    if pool is not None:
        # each two-site block receives one product in the abelian case
        outs = pool.map(lambda t: A1.block(t[1]) @ A2.block(t[2]), prods)
        for (k, _, _), b in zip(prods, outs):
            V.block(k)[...] += b
    else:
        for k, i, j in prods:
            V.block(k)[...] += A1.block(i) @ A2.block(j)
    return (V, comb) if return_basis else V


def _sector_factor_svd(M, move):
    """_sector_factor through LAPACK's SVD (gesdd)"""
    U, S, Vt = np.linalg.svd(M, full_matrices=False)
    return S, (U if move == "right" else Vt.T)


def _sector_factor(M, move):
    """Singular values (descending) and the orthonormal factor of a sector matrix M
    that the sweep direction keeps: the left singular vectors U (move="right") or
    the right singular vectors V (move="left"), from the eigendecomposition of the
    Gram matrix M M^T (M^T M): the density-matrix form of the truncated SVD.  The
    factor is orthonormal to working precision; singular values below ~1e-8 of the
    largest lose accuracy, which touches only states of negligible weight."""
    G = M @ M.T if move == "right" else M.T @ M
    w, Q = np.linalg.eigh(G)
    k = min(M.shape)
    order = np.argsort(w)[::-1][:k]
    return np.sqrt(np.maximum(w[order], 0.0)), Q[:, order]


def _split_native(V, comb, qloc12, qloc34, din, dout, nq, Dmax, move, eps_svd, threads, ctx=None):
    """split_two_site through the native routine (vmps_two_site_split): the same
    sectors, Gram-matrix eigensystems (LAPACK dsyevd), truncation and block order,
    without per-block Python work; the sectors run on `threads` threads.  With a
    device context `ctx` the large sectors run on the GPU in FP64
    (vmps_two_site_split_device)."""
    import ctypes as C
    from . import _native as N
    n13 = int(comb["n"])
    pair1 = np.full(n13, -1, dtype=np.int32)
    pair3 = np.full(n13, -1, dtype=np.int32)
    for (s1, s3), lst in comb["index"].items():
        for _, s13 in lst:
            pair1[s13], pair3[s13] = s1, s3
    qin = sorted(din)
    qout = sorted(dout)
    arr = dict(qloc1=np.ascontiguousarray(np.reshape(qloc12, (-1, nq)), dtype=np.int32),
               qloc3=np.ascontiguousarray(np.reshape(qloc34, (-1, nq)), dtype=np.int32),
               qin=np.ascontiguousarray(np.reshape(qin, (-1, nq)), dtype=np.int32),
               din=np.array([din[q] for q in qin], dtype=np.int64),
               qout=np.ascontiguousarray(np.reshape(qout, (-1, nq)), dtype=np.int32),
               dout=np.array([dout[q] for q in qout], dtype=np.int64))
    a = N.vmps_split_args()
    a.nq, a.n1, a.n3, a.n13 = nq, len(qloc12), len(qloc34), n13
    a.qloc1 = arr["qloc1"].ctypes.data_as(N.i32p)
    a.qloc3 = arr["qloc3"].ctypes.data_as(N.i32p)
    a.pair1 = pair1.ctypes.data_as(N.i32p)
    a.pair3 = pair3.ctypes.data_as(N.i32p)
    a.nin, a.qin, a.din = len(qin), arr["qin"].ctypes.data_as(N.i32p), arr["din"].ctypes.data_as(N.i64p)
    a.nout, a.qout, a.dout = len(qout), arr["qout"].ctypes.data_as(N.i32p), arr["dout"].ctypes.data_as(N.i64p)
    a.dmax, a.eps_svd, a.move_right, a.threads = int(Dmax), float(eps_svd), int(move == "right"), int(threads)
    vb = V.c_struct()
    h = C.c_void_p()
    lib = N.lib()
    if ctx is not None and getattr(ctx, "device", -1) >= 0:
        N.check(lib.vmps_two_site_split_device(ctx._h, C.byref(a), C.byref(vb), V.data_ptr(), C.byref(h)))
    else:
        N.check(lib.vmps_two_site_split(C.byref(a), C.byref(vb), V.data_ptr(), C.byref(h)))
    try:
        nmid, disc = C.c_int(), C.c_double()
        nb1, sz1, nb2, sz2 = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        N.check(lib.vmps_split_info(h, C.byref(nmid), C.byref(disc), C.byref(nb1), C.byref(sz1), C.byref(nb2),
                                    C.byref(sz2)))
        m, b1, b2 = nmid.value, nb1.value, nb2.value
        qmid = np.zeros((max(m, 1), nq), np.int32)
        dm = np.zeros(max(m, 1), np.int64)
        t1 = dict(leg=np.zeros(max(b1, 1), np.int32), qin=np.zeros((max(b1, 1), nq), np.int32),
                  qout=np.zeros((max(b1, 1), nq), np.int32), rows=np.zeros(max(b1, 1), np.int64),
                  cols=np.zeros(max(b1, 1), np.int64), data=np.zeros(max(sz1.value, 1)))
        t2 = dict(leg=np.zeros(max(b2, 1), np.int32), qin=np.zeros((max(b2, 1), nq), np.int32),
                  qout=np.zeros((max(b2, 1), nq), np.int32), rows=np.zeros(max(b2, 1), np.int64),
                  cols=np.zeros(max(b2, 1), np.int64), data=np.zeros(max(sz2.value, 1)))
        ptr = lambda x, t: x.ctypes.data_as(t)
        N.check(lib.vmps_split_get(h, ptr(qmid, N.i32p), ptr(dm, N.i64p),
                                   *[ptr(t1[k], N.i32p) for k in ("leg", "qin", "qout")],
                                   ptr(t1["rows"], N.i64p), ptr(t1["cols"], N.i64p), ptr(t1["data"], N.f64p),
                                   *[ptr(t2[k], N.i32p) for k in ("leg", "qin", "qout")],
                                   ptr(t2["rows"], N.i64p), ptr(t2["cols"], N.i64p), ptr(t2["data"], N.f64p)))
    finally:
        lib.vmps_split_destroy(h)
    dmid = {tuple(int(x) for x in qmid[i]): int(dm[i]) for i in range(m)}

    def blocks(t, n, size):
        return Blocks(nq, t["qin"][:n], t["qout"][:n], t["leg"][:n], t["rows"][:n], t["cols"][:n],
                      data=t["data"][:size])
    return blocks(t1, b1, sz1.value), blocks(t2, b2, sz2.value), disc.value, dmid


def split_two_site(V, comb, qloc12, qloc34, din, dout, nq, Dmax, move="right", eps_svd=1e-14, pool=None,
                   factor="eigh", native=True, ctx=None):
    """Truncated SVD of a two-site tensor back into two site tensors (abelian QNs):
    split_AA2 with Biped::truncateSVD (tensors/DmrgContractions.h:2461-2631,
    tensors/Biped.h:744-932).  For every middle QN qmid the matrix
    Psi[(s1, qin), (s3, qout)] = V[s13(s1, s3)](qin, qout), qin + q(s1) = qmid, is
    decomposed; the Dmax largest singular values over all sectors are kept (none
    below eps_svd times the largest) and renormalised.
    move="right": A1 = U (left-orthonormal), A2 = S Vt (the new centre);
    move="left":  A1 = U S (the new centre), A2 = Vt (right-orthonormal).
    Returns A1, A2, the discarded weight and the middle bond basis {qmid: dim}.
    `pool` (hostla.SectorPool) runs the sector factorisations in parallel; `factor`:
    "eigh" (Gram matrix, default) or "svd".  Either way the orthonormal factor's
    columns are the singular vectors for the sweep direction.  native=True (with
    "eigh") runs the whole split in the native library (vmps_two_site_split) on
    the pool's thread count when numpy's LAPACK can be bound to it; with a device
    context `ctx` its large sectors run on the GPU in FP64."""
    if native and factor == "eigh":
        from .hostla import native_lapack
        if native_lapack():
            return _split_native(V, comb, qloc12, qloc34, din, dout, nq, Dmax, move, eps_svd,
                                 pool.threads if pool is not None else 1, ctx=ctx)
    # each two-site block (s13, qin, qout) is one (s1, s3) pair (abelian): scatter the
    # blocks into their middle-QN sector matrices in one pass over the blocks
    pair_of = {}
    for (s1, s3), lst in comb["index"].items():
        pair_of[lst[0][1]] = (s1, s3)
    rows, cols = {}, {}
    for s1, q1 in enumerate(qloc12):
        for qin in sorted(din):
            rows.setdefault(_add(qin, q1), []).append((s1, qin))
    for s3, q3 in enumerate(qloc34):
        for qout in sorted(dout):
            cols.setdefault(_sub(qout, q3), []).append((s3, qout))
    roff, coff, shape = {}, {}, {}
    for qm in set(rows) & set(cols):
        r0 = 0
        for s1, qin in rows[qm]:
            roff[(s1, qin)] = (qm, r0)
            r0 += din[qin]
        c0 = 0
        for s3, qout in cols[qm]:
            coff[(s3, qout)] = (qm, c0)
            c0 += dout[qout]
        shape[qm] = (r0, c0)
    mats_by_q = {}
    qins, qouts, legs = [tuple(x) for x in V.qin.tolist()], [tuple(x) for x in V.qout.tolist()], V.leg.tolist()
    for k in range(V.n):
        s1, s3 = pair_of[legs[k]]
        ro, co = roff.get((s1, qins[k])), coff.get((s3, qouts[k]))
        if ro is None or co is None or ro[0] != co[0]:
            continue
        qm = ro[0]
        M = mats_by_q.get(qm)
        if M is None:
            M = mats_by_q[qm] = np.zeros(shape[qm])
        r, c = int(V.rows[k]), int(V.cols[k])
        M[ro[1]:ro[1] + r, co[1]:co[1] + c] = V.block(k)
    sectors = []
    for qm in sorted(mats_by_q):
        r_off = [(s1, qin, roff[(s1, qin)][1]) for s1, qin in rows[qm]]
        c_off = [(s3, qout, coff[(s3, qout)][1]) for s3, qout in cols[qm]]
        sectors.append((qm, r_off, c_off, mats_by_q[qm]))
    mats = [t[3] for t in sectors]
    f = _sector_factor if factor == "eigh" else _sector_factor_svd
    fac = (lambda M: f(M, move))
    svds = pool.map(fac, mats) if pool is not None else [fac(M) for M in mats]
    allsv = np.concatenate([sv[0] for sv in svds]) if svds else np.zeros(0)
    smax = float(allsv.max()) if allsv.size else 0.0
    keep_vals = np.sort(allsv[allsv > eps_svd * smax])[::-1][:Dmax]
    thresh = keep_vals[-1] if keep_vals.size else np.inf
    kept, disc = {}, 0.0
    # ties at the threshold: keep in sector order until Dmax is reached
    budget = keep_vals.size
    for (qm, _, _, _), (S, _) in zip(sectors, svds):
        k = int(np.sum(S > thresh))
        kept[qm] = k
        budget -= k
    for (qm, _, _, _), (S, _) in zip(sectors, svds):
        if budget <= 0:
            break
        extra = int(np.sum(S == thresh))
        take = min(extra, budget)
        kept[qm] += take
        budget -= take
    norm2 = sum(float(np.sum(S[:kept[qm]] ** 2)) for (qm, _, _, _), (S, _) in zip(sectors, svds))
    tot2 = float(np.sum(allsv ** 2))
    disc = max(0.0, tot2 - norm2) / tot2 if tot2 > 0 else 0.0
    scale = 1.0 / np.sqrt(norm2) if norm2 > 0 else 1.0
    dmid = {qm: kept[qm] for qm in kept if kept[qm] > 0}
    A1 = site_layout(qloc12, din, dmid, nq)
    A2 = site_layout(qloc34, dmid, dout, nq)
    for (qm, r_off, c_off, M), (S, Q) in zip(sectors, svds):
        k = kept[qm]
        if k == 0:
            continue
        if move == "right":       # A1 = U (orthonormal), A2 = S V^T = U^T M
            Uk = Q[:, :k]
            Vk = (Uk.T @ M) * scale
        else:                     # A2 = V^T (orthonormal), A1 = U S = M V
            Vk = Q[:, :k].T
            Uk = (M @ Q[:, :k]) * scale
        for s1, qin, ra in r_off:
            i = A1.find(s1, qin, qm)
            if i >= 0:
                A1.block(i)[...] = Uk[ra:ra + din[qin]]
        for s3, qout, ca in c_off:
            j = A2.find(s3, qm, qout)
            if j >= 0:
                A2.block(j)[...] = Vk[:, ca:ca + dout[qout]]
    return A1, A2, disc, dmid
