"""MPS-level compression on the engine: variational fitting of a sum of operator-MPS
products by two-site sweeps (MpsCompressor::prodCompress / polyCompress,
solvers/MpsCompressor.h:961-1564), and the Chebyshev recursion of whole MPS built on
it (polyIter, DmrgLinearAlgebra.h:550-566).  Abelian symmetries, and SU(2) (or SU(2) x U(1))
for operators that keep the total quantum number (the SU(2) two-site contraction and split
of su2.py, reduced tensors throughout).

fit(phi, terms): phi ~ sum_i c_i O_i psi_i, with O_i an MPO (the Hamiltonian, or the
identity for a plain MPS term).  phi is right-canonical with its centre on site 0; per
two-site step (l, l+1) the optimal two-site tensor of phi, with its other sites
orthonormal, is

    T = sum_i c_i  L_i[l] W_i[l] W_i[l+1] Psi_i(l, l+1) R_i[l+2],

L_i / R_i the environments of O_i between phi (bra) and psi_i (ket) (contract_L /
contract_R with Abra != Aket).  Each term is one two-site pivot application from psi_i's
layout into phi's; the two layouts differ, so it runs as a pivot whose blocks carry a tag
(0: ket, 1: bra; union.bra_ket_tag / aux_tag).  T is split by the truncated SVD (at most
Dmax states over all sectors of the middle bond, the state's norm kept), and the
environment of the sweep direction is updated.  The middle bond grows and shrinks with
the split, so phi's bond dimensions adapt to the target.

chebyshev_moments(psi0, nmom, a, b): t_0 = psi0, t_1 = (H - b)/a t_0, t_{n+1} =
2 (H - b)/a t_n - t_{n-1}, each fitted as above (terms H t_n, t_n, t_{n-1}), and
mu_n = <psi0|t_n> from the overlap environments.
"""
from __future__ import annotations

import contextlib
import copy

import numpy as np

from .blocks import Blocks, MpoSite
from .hostla import SectorPool
from .mps import contract_two_sites, right_normalize, split_two_site, two_site_layout
from .su2 import contract_two_sites_su2, split_two_site_su2
from .pivot import EnvUpdate, PivotMatrix2, left_vacuum
from .union import aux_tag, bra_ket_tag, concat_blocks, tag_blocks, tagged_symmetry


def identity_mpo(model) -> list:
    """the identity as an MPO (one auxiliary state, quantum number vacuum)"""
    vac = model.sym.vacuum()
    W = []
    for _ in range(model.L):
        w = MpoSite(model.sym.nq, list(model.qloc), [vac])
        for s in range(len(model.qloc)):
            w.add(s, s, 0, vac, vac, 0, 0, 1.0)
        W.append(w)
    return W


def mpo_sum(mpos: list, coefs: list, end_q, vac=None) -> list:
    """sum_i c_i O_i of MPOs (site lists) as one MPO: the auxiliary bases of the inner bonds
    side by side (the states of O_i after those of O_0..O_i-1 in each quantum-number
    sector), the boundary states shared, c_i on site 0's entries of O_i.  Every O_i starts
    in the vacuum state (index 0) and ends in state 0 of quantum number end_q (the charge
    the operators carry; vac: the vacuum, all zeros by default, (1, ...) for SU(2)
    components); entries of the boundary sites that leave other boundary states are never
    reached from the environments and are dropped."""
    L, nq = len(mpos[0]), mpos[0][0].nq
    vac = tuple(0 for _ in range(nq)) if vac is None else tuple(vac)
    end_q = tuple(end_q)
    out = [MpoSite(nq, list(mpos[0][l].qloc), []) for l in range(L)]
    qops = [[] for _ in range(L)]
    base = [dict() for _ in range(L + 1)]      # bond -> {aux QN: states placed so far}
    for W, c in zip(mpos, coefs):
        nstate = [dict() for _ in range(L + 1)]
        for l in range(L):
            w = W[l]
            kmap = []
            for q in w.qop:
                if tuple(q) not in qops[l]:
                    qops[l].append(tuple(q))
                kmap.append(qops[l].index(tuple(q)))
            for i in range(w.nnz):
                q_in, q_out, r, col = tuple(w.qin[i]), tuple(w.qout[i]), w.row[i], w.col[i]
                nstate[l][q_in] = max(nstate[l].get(q_in, 0), r + 1)
                nstate[l + 1][q_out] = max(nstate[l + 1].get(q_out, 0), col + 1)
                if l == 0 and (q_in != vac or r != 0):
                    continue
                if l == L - 1 and (q_out != end_q or col != 0):
                    continue
                r += base[l].get(q_in, 0) if l > 0 else 0
                col += base[l + 1].get(q_out, 0) if l < L - 1 else 0
                out[l].add(w.s1[i], w.s2[i], kmap[w.k[i]], q_in, q_out, r, col, (c if l == 0 else 1.0) * w.val[i])
        for b in range(1, L):
            for q, n in nstate[b].items():
                base[b][q] = base[b].get(q, 0) + n
    for l in range(L):
        out[l].qop = qops[l]
    return out


def _bond_sectors(W: list) -> list:
    """auxiliary sector dimensions of an MPO at every bond: [{QN: states}] (L + 1 bonds)"""
    L = len(W)
    dims = [dict() for _ in range(L + 1)]
    for l, w in enumerate(W):
        for i in range(w.nnz):
            qi, qo = tuple(w.qin[i]), tuple(w.qout[i])
            dims[l][qi] = max(dims[l].get(qi, 0), w.row[i] + 1)
            dims[l + 1][qo] = max(dims[l + 1].get(qo, 0), w.col[i] + 1)
    return dims


def _clean(W: list, what: str):
    dims = _bond_sectors(W)
    for b in (0, len(W)):
        if sum(dims[b].values()) != 1:
            raise ValueError(f"{what}: the MPO needs a single auxiliary state at both ends")


def mpo_adjoint(W: list) -> list:
    """O^dagger of a real MPO with abelian quantum numbers: every site's local matrices
    transposed, operator and auxiliary quantum numbers negated"""
    out = []
    for w in W:
        t = MpoSite(w.nq, list(w.qloc), [tuple(-x for x in q) for q in w.qop])
        for i in range(w.nnz):
            t.add(w.s2[i], w.s1[i], w.k[i], tuple(-x for x in w.qin[i]), tuple(-x for x in w.qout[i]), w.row[i],
                  w.col[i], w.val[i])
        out.append(t)
    return out


def mpo_product(A: list, B: list) -> list:
    """the operator product A B (B acts first) of two MPOs with abelian quantum numbers and a
    single auxiliary state at both ends: W[s1, s3] = sum_s2 A[s1, s2] B[s2, s3] on the product
    of the auxiliary bases, the states of each product sector in (QN_A, index_A, QN_B, index_B)
    order, so that the two end states stay state 0; equal entries summed"""
    _clean(A, "mpo_product")
    _clean(B, "mpo_product")
    L = len(A)
    da, db = _bond_sectors(A), _bond_sectors(B)
    index = []                      # bond -> {(qa, ia, qb, ib): (q, position in sector q)}
    for b in range(L + 1):
        pos, idx = {}, {}
        for qa in sorted(da[b]):
            for ia in range(da[b][qa]):
                for qb in sorted(db[b]):
                    for ib in range(db[b][qb]):
                        q = tuple(x + y for x, y in zip(qa, qb))
                        idx[(qa, ia, qb, ib)] = (q, pos.get(q, 0))
                        pos[q] = pos.get(q, 0) + 1
        index.append(idx)
    out = []
    for l in range(L):
        wa, wb = A[l], B[l]
        by_s2 = {}
        for j in range(wb.nnz):
            by_s2.setdefault(wb.s1[j], []).append(j)
        qops, acc = [], {}
        for i in range(wa.nnz):
            for j in by_s2.get(wa.s2[i], ()):
                qop = tuple(x + y for x, y in zip(wa.qop[wa.k[i]], wb.qop[wb.k[j]]))
                if qop not in qops:
                    qops.append(qop)
                qi, ri = index[l][(tuple(wa.qin[i]), wa.row[i], tuple(wb.qin[j]), wb.row[j])]
                qo, co = index[l + 1][(tuple(wa.qout[i]), wa.col[i], tuple(wb.qout[j]), wb.col[j])]
                key = (wa.s1[i], wb.s2[j], qops.index(qop), qi, qo, ri, co)
                acc[key] = acc.get(key, 0.0) + wa.val[i] * wb.val[j]
        t = MpoSite(wa.nq, list(wa.qloc), qops)
        for (s1, s3, k, qi, qo, ri, co), v in acc.items():
            if v != 0.0:
                t.add(s1, s3, k, qi, qo, ri, co, v)
        out.append(t)
    return out


def _dims_of(A: Blocks, side: str) -> dict:
    q = A.qin if side == "in" else A.qout
    n = A.rows if side == "in" else A.cols
    return {tuple(q[i]): int(n[i]) for i in range(A.n)}


def copy_mps(psi):
    """a copy of an MPS object (its site tensors and bond bases copied)"""
    m = copy.copy(psi)
    m.A = [a.like(a.data.copy()) for a in psi.A]
    m.dims = [dict(d) for d in psi.dims]
    return m


def right_canonical(psi, pool=None):
    """psi with sites 1..L-1 right-orthonormal (the factors pushed into site 0), in place"""
    sym = psi.model.sym if psi.model.sym.nonabelian else None   # SU(2): the weighted normalisation
    carry = None
    for l in range(psi.L - 1, 0, -1):
        psi.A[l], carry = right_normalize(psi.A[l], psi.model.sym.nq, carry, sym=sym, pool=pool)
    A = psi.A[0]
    for i in range(A.n):
        q = tuple(A.qout[i])
        if q in carry:
            A.block(i)[...] = A.block(i) @ carry[q]
    return psi


class Compressor:
    """fits and overlaps of MPS of one model on the engine.  precision: that of the
    two-site applications ("fp64" or a split form; the environments are FP64).
    env(side, E, Abra, W, Aket) and apply2(sym, L, R, W1, W2, V, x) replace the engine's
    environment update and two-site HxV (a host check runs the same sweeps on a CPU
    restatement).  factor: the sector factorisation of the split, "svd" (LAPACK's SVD
    on the host: singular values accurate down to the working precision, so a cut at
    eps_svd = 1e-14 of the largest drops only rounding noise, as Biped::truncateSVD's
    does) or "eigh" (the native Gram-matrix split, large sectors on the GPU: faster,
    singular values below ~1e-8 of the largest are noise, so give eps_svd >= 1e-7).  The
    host's share (sector factorisations, QRs) runs on `threads` threads (hostla.SectorPool;
    default: up to 16 cores)."""

    def __init__(self, ctx, model, precision="fp64", env=None, apply2=None, factor="svd", threads=None):
        self.ctx, self.model, self.sym = ctx, model, model.sym
        self.precision = precision
        self.I = identity_mpo(model)
        self.tsym = tagged_symmetry(self.sym)
        self._env = env or self._engine_env
        self.apply2 = apply2 or self._engine_apply2
        self.factor = factor
        self.threads = threads
        self._pool = None
        self.applications = 0

    # ---- engine steps
    def _engine_env(self, side, E, Abra, W, Aket):
        e = EnvUpdate(self.ctx, self.sym, side, E, Abra, W, Aket)
        try:
            return e.run(E, Abra, Aket, "fp64")
        finally:
            e.close()

    def _engine_apply2(self, sym, L, R, W1, W2, V, x):
        H = PivotMatrix2(self.ctx, sym, L, R, W1, W2, V)
        try:
            return H.apply(x, self.precision)
        finally:
            H.close()

    def _apply(self, L, R, W1, W2, Vket: Blocks, Vbra: Blocks) -> np.ndarray:
        """the two-site application of (L, W1, W2, R) to Vket, into Vbra's layout"""
        V = concat_blocks([tag_blocks(Vket, 0), tag_blocks(Vbra, 1)])
        x = np.concatenate([Vket.data, np.zeros(Vbra.data.size)])
        y = self.apply2(self.tsym, bra_ket_tag(L, "L"), bra_ket_tag(R, "R"), aux_tag(W1), aux_tag(W2), V, x)
        self.applications += 1
        return y[Vket.data.size:]

    def overlap(self, bra, ket) -> float:
        """<bra|ket> of two MPS with the same total quantum number"""
        return self.matrix_element(bra, self.I, ket)

    def matrix_element(self, bra, W, ket) -> float:
        """<bra|O|ket> of an MPO O (site list) that keeps the total quantum number
        (avg(bra, O, ket)): contract_L through the chain"""
        E = left_vacuum(self.sym)
        for l in range(self.model.L):
            E = self._env("L", E, bra.A[l], W[l], ket.A[l])
        return float(E.data.sum())

    # ---- the fit
    def fit(self, phi, terms: list, Dmax: int, sweeps: int = 2, eps_svd: float = 1e-14, target_norm2=None,
            tol=None, min_sweeps: int = 1):
        """phi ~ sum c_i O_i psi_i, terms = [(W_i (MPO site list), psi_i (MPS), c_i)]; phi is
        updated in place (brought to right-canonical form first; it ends so, with its
        centre on site 0).  The operators may change the charge: O_i carries phi.Qtot -
        psi_i.Qtot (its MPO ends in that auxiliary quantum number).  Terms on the same
        psi_i run as one MPO (mpo_sum), so each step costs one two-site application and
        one environment update per distinct psi_i.  Returns the largest discarded weight
        of the last sweep.  With target_norm2 = <T|T> of the target and tol, the sweeps stop
        as soon as the squared distance |phi - T|^2 = <T|T> - <phi|phi> (the fit is the
        projection of T: <phi|T> = <phi|phi>) is at most tol, after min_sweeps and at most
        `sweeps` full sweeps (two half-sweeps each, as MpsCompressor runs an even number);
        self.last_fit holds the sweeps run and the last squared distance."""
        ctl = (target_norm2, tol, min_sweeps)
        if self._pool is not None:
            return self._fit(phi, terms, Dmax, sweeps, eps_svd, self._pool, ctl)
        with self._host_pool():
            return self._fit(phi, terms, Dmax, sweeps, eps_svd, self._pool, ctl)

    @contextlib.contextmanager
    def _host_pool(self):
        """one SectorPool for a batch of fits (opening one changes OpenBLAS's thread count)"""
        if self._pool is not None:
            yield self._pool
            return
        self._pool = SectorPool(self.threads)
        try:
            yield self._pool
        finally:
            self._pool.close()
            self._pool = None

    def _fit(self, phi, terms, Dmax, sweeps, eps_svd, pool, ctl=(None, None, 1)):
        sym, nq, qloc, L = self.sym, self.sym.nq, self.model.qloc, self.model.L
        right_canonical(phi, pool)
        ctx = self.ctx if getattr(self.ctx, "device", -1) >= 0 else None
        groups = {}
        for W, psi, c in terms:
            groups.setdefault(id(psi), (psi, []))[1].append((W, c))
        plan = []
        su2 = sym.nonabelian
        for psi, lst in groups.values():
            if tuple(phi.Qtot) == tuple(psi.Qtot):
                dq = tuple(sym.vacuum())
            elif su2:
                raise ValueError("SU(2) fits take operators that keep the total quantum number")
            else:
                dq = tuple(int(a - b) for a, b in zip(phi.Qtot, psi.Qtot))
            if len(lst) == 1:
                W, c = lst[0]
            else:
                W, c = mpo_sum([w for w, _ in lst], [c for _, c in lst], dq, sym.vacuum()), 1.0
            # contract_R's right boundary: rows the ket's total charge, columns the bra's
            RT = Blocks.from_entries(nq, [(0, tuple(psi.Qtot), tuple(phi.Qtot), dq, np.ones((1, 1)))], tripod=True)
            plan.append((W, psi, c, RT))
        nt = len(plan)
        envL = [[None] * (L + 1) for _ in range(nt)]
        envR = [[None] * (L + 1) for _ in range(nt)]
        for t, (W, psi, _, RT) in enumerate(plan):
            envL[t][0] = left_vacuum(sym)
            envR[t][L] = RT
            for l in range(L - 1, 1, -1):
                envR[t][l] = self._env("R", envR[t][l + 1], phi.A[l], W[l], psi.A[l])
        disc_max = 0.0
        two_site = {}
        target_norm2, tol, min_sweeps = ctl
        self.last_fit = {"sweeps": 0, "sqdist": None}
        for sweep in range(sweeps):
            disc_max = 0.0
            for move, bonds in (("right", range(L - 1)), ("left", range(L - 2, -1, -1))):
                for l in bonds:
                    din, dout = _dims_of(phi.A[l], "in"), _dims_of(phi.A[l + 1], "out")
                    Vb, comb = two_site_layout(sym, qloc, qloc, din, dout, nq)
                    x = np.zeros(Vb.data.size)
                    for t, (W, psi, c, _) in enumerate(plan):
                        # the sources do not change during the fit: their two-site tensors are made once
                        Vk = two_site.get((t, l))
                        if Vk is None:
                            if su2:
                                Vk = contract_two_sites_su2(sym, psi.A[l], psi.A[l + 1], qloc, qloc, ctx=ctx)[0]
                            else:
                                Vk = contract_two_sites(sym, psi.A[l], psi.A[l + 1], qloc, qloc, nq, ctx=ctx,
                                                        pool=pool)
                            two_site[(t, l)] = Vk
                        x += c * self._apply(envL[t][l], envR[t][l + 2], W[l], W[l + 1], Vk, Vb)
                    Vb.data[:] = x
                    if su2:
                        # the kept multiplets keep their singular values (and the state its norm)
                        A1, A2, disc, dmid = split_two_site_su2(Vb, comb, sym, qloc, qloc, din, dout, Dmax,
                                                                move=move, eps_svd=eps_svd, renormalise=False)
                    else:
                        nrm = float(np.linalg.norm(x))
                        A1, A2, disc, dmid = split_two_site(Vb, comb, qloc, qloc, din, dout, nq, Dmax, move=move,
                                                            eps_svd=eps_svd, factor=self.factor,
                                                            native=self.factor == "eigh", ctx=ctx, pool=pool)
                        # the split renormalises the kept singular values: the fitted state keeps its norm
                        scale = nrm * np.sqrt(max(0.0, 1.0 - disc))
                        (A2 if move == "right" else A1).data[:] *= scale
                    phi.A[l], phi.A[l + 1] = A1, A2
                    phi.dims[l + 1] = dmid
                    disc_max = max(disc_max, disc)
                    for t, (W, psi, _, _) in enumerate(plan):
                        if move == "right":
                            envL[t][l + 1] = self._env("L", envL[t][l], A1, W[l], psi.A[l])
                        else:
                            envR[t][l + 1] = self._env("R", envR[t][l + 2], A2, W[l + 1], psi.A[l + 1])
            self.last_fit["sweeps"] = sweep + 1
            if target_norm2 is not None:
                # centre on site 0, the other sites right-orthonormal: <phi|phi> is site 0's norm
                n2 = self.overlap(phi, phi) if su2 else float(np.dot(phi.A[0].data, phi.A[0].data))
                self.last_fit["sqdist"] = float(target_norm2 - n2)
                if tol is not None and sweep + 1 >= min_sweeps and self.last_fit["sqdist"] <= tol:
                    break
        return disc_max

    # ---- the MpsCompressor operations (solvers/MpsCompressor.h:60-126)
    def state_compress(self, psi, Dmax: int, tol: float = 1e-4, max_sweeps: int = 20, min_sweeps: int = 1,
                       eps_svd: float = 1e-14):
        """stateCompress: phi ~ psi with at most Dmax states per bond, sweeps until
        |phi - psi|^2 <= tol; returns (phi, info)"""
        phi = copy_mps(psi)
        disc = self.fit(phi, [(self.I, psi, 1.0)], Dmax, max_sweeps, eps_svd, self.overlap(psi, psi), tol, min_sweeps)
        return phi, dict(self.last_fit, discarded=disc)

    def prod_compress(self, W, psi, Dmax: int, tol: float = 1e-4, max_sweeps: int = 20, min_sweeps: int = 1,
                      phi=None, Wdag=None, eps_svd: float = 1e-14):
        """prodCompress: phi ~ W psi, sweeps until |phi - W psi|^2 <= tol (<psi|W^dagger W|psi>
        from the product MPO of Wdag = W^dagger and W; abelian symmetries).  phi: the start
        (a copy of psi by default; give one of the target charge for operators that change
        it).  Returns (phi, info)."""
        if self.sym.nonabelian:
            raise ValueError("prod_compress needs the product MPO W^dagger W: abelian symmetries")
        P = mpo_product(Wdag if Wdag is not None else mpo_adjoint(W), W)
        t2 = self.matrix_element(psi, P, psi)
        phi = copy_mps(psi) if phi is None else phi
        disc = self.fit(phi, [(W, psi, 1.0)], Dmax, max_sweeps, eps_svd, t2, tol, min_sweeps)
        return phi, dict(self.last_fit, discarded=disc, target_norm2=t2)

    def poly_compress(self, H, psi1, polyB: float, psi2, Dmax: int, tol: float = 1e-4, max_sweeps: int = 20,
                      min_sweeps: int = 1, phi=None, eps_svd: float = 1e-14):
        """polyCompress: phi ~ H psi1 - polyB psi2 for a Hermitian H (rescaled by the caller),
        the step of an orthogonal-polynomial recursion; |T|^2 = <psi1|H H|psi1> - 2 polyB
        <psi2|H|psi1> + polyB^2 <psi2|psi2>.  Returns (phi, info)."""
        if self.sym.nonabelian:
            raise ValueError("poly_compress needs the product MPO H H: abelian symmetries")
        t2 = (self.matrix_element(psi1, mpo_product(H, H), psi1) - 2 * polyB * self.matrix_element(psi2, H, psi1)
              + polyB * polyB * self.overlap(psi2, psi2))
        phi = copy_mps(psi1) if phi is None else phi
        disc = self.fit(phi, [(H, psi1, 1.0), (self.I, psi2, -polyB)], Dmax, max_sweeps, eps_svd, t2, tol,
                        min_sweeps)
        return phi, dict(self.last_fit, discarded=disc, target_norm2=t2)

    def lincombo_compress(self, psis: list, factors: list, Dmax: int, guess=None, tol: float = 1e-4,
                          max_sweeps: int = 20, min_sweeps: int = 1, eps_svd: float = 1e-14):
        """lincomboCompress: phi ~ sum_i f_i psi_i (|T|^2 from the overlaps); guess: the
        start (a copy of psis[0] by default).  Returns (phi, info)."""
        t2 = sum(fi * fj * self.overlap(pi, pj) for pi, fi in zip(psis, factors) for pj, fj in zip(psis, factors))
        phi = copy_mps(psis[0] if guess is None else guess)
        disc = self.fit(phi, [(self.I, p, f) for p, f in zip(psis, factors)], Dmax, max_sweeps, eps_svd, t2, tol,
                        min_sweeps)
        return phi, dict(self.last_fit, discarded=disc, target_norm2=t2)

    # ---- the Chebyshev recursion of MPS
    def chebyshev_moments(self, psi0, nmom: int, a: float, b: float, Dmax: int, sweeps: int = 2,
                          eps_svd: float = 1e-14):
        """mu_n = <psi0| T_n((H - b)/a) |psi0>, n < nmom, the vectors t_n fitted as MPS of at
        most Dmax states per bond; returns (mu, info)"""
        with self._host_pool():
            return self._chebyshev(psi0, nmom, a, b, Dmax, sweeps, eps_svd)

    def _chebyshev(self, psi0, nmom, a, b, Dmax, sweeps, eps_svd):
        H = self.model.W
        mu = np.zeros(nmom)
        t0 = copy_mps(psi0)
        mu[0] = self.overlap(psi0, t0)
        disc = []
        if nmom == 1:
            return mu, {"discarded": disc}
        t1 = copy_mps(t0)
        disc.append(self.fit(t1, [(H, t0, 1.0 / a), (self.I, t0, -b / a)], Dmax, sweeps, eps_svd))
        mu[1] = self.overlap(psi0, t1)
        tp, tc = t0, t1
        for n in range(2, nmom):
            tn = copy_mps(tc)
            disc.append(self.fit(tn, [(H, tc, 2.0 / a), (self.I, tc, -2.0 * b / a), (self.I, tp, -1.0)], Dmax,
                                 sweeps, eps_svd))
            mu[n] = self.overlap(psi0, tn)
            tp, tc = tc, tn
        return mu, {"discarded": disc, "max_bond": max(sum(d.values()) for d in tc.dims)}
