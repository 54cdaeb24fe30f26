"""Nearest-neighbour chain Hamiltonians as MPOs (host-side model layer).

The reference builds W through MpoTerms (MpoTerms.h:1175-1232) from the site
operator algebras of bases/SpinBase.h and bases/FermionBase.h.  This module
produces the same object -- W[s1][s2][k] blocks keyed by auxiliary QNs -- for
the chains the benchmark configurations use, from a finite-state-machine MPO:

    aux states at every inner bond: IDLE, OPEN_t (one per two-site term t), DONE
    W[IDLE->IDLE] = 1,  W[IDLE->OPEN_t] = A_t,  W[OPEN_t->DONE] = c_t B_t,
    W[IDLE->DONE] = onsite,  W[DONE->DONE] = 1

so H = sum_i (onsite_i + sum_t c_t A_t,i B_t,i+1).  An auxiliary state carries
the QN of the operators placed to its left (vacuum for IDLE and DONE), which
makes every W block QN-conserving: qout_aux = qin_aux + q(operator).

Local bases (QN conventions of the reference's U(1) kinds, M = 2 S^z):
  spin-1/2, U(1) M            : s=0 |up> M=+1, s=1 |dn> M=-1
  Hubbard, U(1)xU(1) (N, M)   : s=0 |0> (0,0), s=1 |up> (1,1), s=2 |dn> (1,-1), s=3 |updn> (2,0)
with |updn> = c+_up c+_dn |0>; fermion signs by Jordan-Wigner (site order,
up before down inside a site).
"""
from __future__ import annotations

import numpy as np

from .blocks import MpoSite, Symmetry


class ChainModel:
    """MPO of a chain: sites W[l], aux bases aux[l] (l = 0..L), local bases."""

    def __init__(self, sym, L, qloc, ops, terms, onsite, name="", site_coef=None):
        self.sym = sym
        self.L = L
        self.qloc = qloc            # list of QN tuples (same on every site)
        self.name = name
        self.ops = ops              # name -> (matrix, QN)
        self.terms = terms          # list of (opA, opB, coef)
        self.onsite = onsite        # list of (op, coef)
        self.site_coef = site_coef  # per-site factor of the on-site terms (None: 1 everywhere)
        self._build()

    @property
    def d(self):
        return len(self.qloc)

    def _build(self):
        vac = self.sym.vacuum()
        inner = [("IDLE", vac)] + [(f"OPEN{t}", self.ops[a][1]) for t, (a, b, c) in enumerate(self.terms)] + \
                [("DONE", vac)]
        self.aux = []
        for l in range(self.L + 1):
            if l == 0:
                self.aux.append([("IDLE", vac)])
            elif l == self.L:
                self.aux.append([("DONE", vac)])
            else:
                self.aux.append(list(inner))
        self.W = [self._site(l) for l in range(self.L)]
        self.wdim = len(inner)

    @staticmethod
    def _sector_index(aux):
        cnt, idx = {}, {}
        for name, q in aux:
            idx[name] = (q, cnt.get(q, 0))
            cnt[q] = cnt.get(q, 0) + 1
        return idx

    def _site(self, l):
        d = self.d
        ain, aout = self._sector_index(self.aux[l]), self._sector_index(self.aux[l + 1])
        I = np.eye(d)
        entries = []   # (state_in, state_out, matrix)
        if "IDLE" in ain and "IDLE" in aout:
            entries.append(("IDLE", "IDLE", I))
        if "DONE" in ain and "DONE" in aout:
            entries.append(("DONE", "DONE", I))
        if "IDLE" in ain and "DONE" in aout and self.onsite:
            h = sum(c * self.ops[o][0] for o, c in self.onsite)
            if self.site_coef is not None:
                h = self.site_coef[l] * h
            entries.append(("IDLE", "DONE", h))
        for t, (a, b, c) in enumerate(self.terms):
            if "IDLE" in ain and f"OPEN{t}" in aout:
                entries.append(("IDLE", f"OPEN{t}", self.ops[a][0]))
            if f"OPEN{t}" in ain and "DONE" in aout:
                entries.append((f"OPEN{t}", "DONE", c * self.ops[b][0]))
        # operator QNs: distinct q(s1) - q(s2) over nonzeros, sorted (a std::set in the reference)
        qops = set()
        nz = []
        for sin, sout, M in entries:
            for s1 in range(d):
                for s2 in range(d):
                    v = M[s1, s2]
                    if abs(v) < 1e-15:
                        continue
                    qop = tuple(x - y for x, y in zip(self.qloc[s1], self.qloc[s2]))
                    qops.add(qop)
                    nz.append((s1, s2, qop, ain[sin], aout[sout], v))
        qop_list = sorted(qops)
        kidx = {q: i for i, q in enumerate(qop_list)}
        site = MpoSite(nq=self.sym.nq, qloc=list(self.qloc), qop=qop_list)
        for s1, s2, qop, (qi, ri), (qo, co), v in nz:
            # QN conservation of the aux flow: qout_aux = qin_aux + qop
            assert tuple(x + y for x, y in zip(qi, qop)) == tuple(qo), (qi, qop, qo)
            site.add(s1, s2, kidx[qop], qi, qo, ri, co, v)
        return site

    def basis_order_map(self, l):
        """basis_order_map of bond l: (aux QN, index inside its QN sector) -> position in the bond's aux list"""
        cnt, out = {}, {}
        for pos, (_, q) in enumerate(self.aux[l]):
            q = tuple(q)
            out[(q, cnt.get(q, 0))] = pos
            cnt[q] = cnt.get(q, 0) + 1
        return out

    # dense representation (tests, exact diagonalisation)
    def aux_qns(self, l):
        return [q for _, q in self.aux[l]]

    def dense_W(self, l):
        return self.W[l].dense(self.aux_qns(l), self.aux_qns(l + 1))


def _spin_half_ops():
    Sz = np.diag([0.5, -0.5])
    Sp = np.array([[0.0, 1.0], [0.0, 0.0]])   # |up><dn|
    Sm = Sp.T.copy()
    return {"Sz": (Sz, (0,)), "Sp": (Sp, (2,)), "Sm": (Sm, (-2,))}


def heisenberg_u1(L, J=1.0, Jxy=None, Jz=None):
    """Spin-1/2 XXZ chain, H = sum (Jz Sz Sz + Jxy (S+S- + S-S+)/2), U(1) M = 2 S^z;
    Jxy = Jz = J by default (XXX).  The couplings follow models/HeisenbergU1.h, which
    places 0.5*Jxy on S+S- and S-S+ and Jz on SzSz."""
    Jxy = J if Jxy is None else Jxy
    Jz = J if Jz is None else Jz
    sym = Symmetry(("U1",))
    qloc = [(1,), (-1,)]
    terms = [("Sp", "Sm", 0.5 * Jxy), ("Sm", "Sp", 0.5 * Jxy), ("Sz", "Sz", Jz)]
    return ChainModel(sym, L, qloc, _spin_half_ops(), terms, [], name=f"HeisenbergU1(L={L},Jxy={Jxy},Jz={Jz})")


def spin_half_local_sum(L, coef, op="Sz"):
    """MPO of the one-site observable sum_l coef[l] op_l on a spin-1/2 U(1) chain (bond
    dimension 2), e.g. the staggered magnetisation with coef[l] = (-1)^l / L."""
    sym = Symmetry(("U1",))
    return ChainModel(sym, L, [(1,), (-1,)], _spin_half_ops(), [], [(op, 1.0)], name=f"sum_l c_l {op}_l (L={L})",
                      site_coef=list(coef))


def hubbard_u1xu1(L, t=1.0, U=4.0):
    """Hubbard chain, H = -t sum_s (c+_i,s c_i+1,s + h.c.) + U sum n_up n_dn, U(1)xU(1) (N, M)."""
    sym = Symmetry(("U1", "U1"))
    qloc = [(0, 0), (1, 1), (1, -1), (2, 0)]
    cdu = np.zeros((4, 4)); cdu[1, 0] = 1.0; cdu[3, 2] = 1.0           # c+_up
    cdd = np.zeros((4, 4)); cdd[2, 0] = 1.0; cdd[3, 1] = -1.0          # c+_dn (sign from c+_dn c+_up = -c+_up c+_dn)
    F = np.diag([1.0, -1.0, -1.0, 1.0])
    cu, cd = cdu.T.copy(), cdd.T.copy()
    nupdn = np.diag([0.0, 0.0, 0.0, 1.0])
    ops = {
        "cdu_F": (cdu @ F, (1, 1)), "cdd_F": (cdd @ F, (1, -1)),
        "F_cu": (F @ cu, (-1, -1)), "F_cd": (F @ cd, (-1, 1)),
        "cu": (cu, (-1, -1)), "cd": (cd, (-1, 1)), "cdu": (cdu, (1, 1)), "cdd": (cdd, (1, -1)),
        "nupdn": (nupdn, (0, 0)),
    }
    # c+_i c_i+1 = (c+ F)_i (c)_i+1 ;  c+_i+1 c_i = (F c)_i (c+)_i+1
    terms = [("cdu_F", "cu", -t), ("cdd_F", "cd", -t), ("F_cu", "cdu", -t), ("F_cd", "cdd", -t)]
    onsite = [("nupdn", U)] if U != 0 else []
    return ChainModel(sym, L, qloc, ops, terms, onsite, name=f"HubbardU1xU1(L={L},t={t},U={U})")


class SU2ChainModel(ChainModel):
    """A ChainModel whose local basis and operators are SU(2)-reduced: every
    operator is (reduced matrix over the local multiplets, operator multiplet),
    and W holds the reduced matrix elements, as MpoTerms::calc_W does
    (MpoTerms.h:1175-1232: W[s1][s2][k](row, col) = op.data(s1, s2) with
    qOp[k] = op.Q); the Clebsch-Gordan structure lives in the contraction
    coefficients (coeff_HPsi, coeff_buildL/R)."""

    def _site(self, l):
        d = self.d
        ain, aout = self._sector_index(self.aux[l]), self._sector_index(self.aux[l + 1])
        entries = []   # (state_in, state_out, matrix, operator QN)
        vac = self.sym.vacuum()
        I = np.eye(d)
        if "IDLE" in ain and "IDLE" in aout:
            entries.append(("IDLE", "IDLE", I, vac))
        if "DONE" in ain and "DONE" in aout:
            entries.append(("DONE", "DONE", I, vac))
        for t, (a, b, c) in enumerate(self.terms):
            if "IDLE" in ain and f"OPEN{t}" in aout:
                entries.append(("IDLE", f"OPEN{t}", c * self.ops[a][0], self.ops[a][1]))
            if f"OPEN{t}" in ain and "DONE" in aout:
                entries.append((f"OPEN{t}", "DONE", self.ops[b][0], self.ops[b][1]))
        qop_list = sorted({tuple(e[3]) for e in entries})
        kidx = {q: i for i, q in enumerate(qop_list)}
        site = MpoSite(nq=self.sym.nq, qloc=list(self.qloc), qop=qop_list)
        for sin, sout, M, qop in entries:
            (qi, ri), (qo, co) = ain[sin], aout[sout]
            assert tuple(qo) in self.sym.fuse(tuple(qi), tuple(qop)), (qi, qop, qo)
            for s1 in range(d):
                for s2 in range(d):
                    if abs(M[s1, s2]) >= 1e-15:
                        site.add(s1, s2, kidx[tuple(qop)], qi, qo, ri, co, M[s1, s2])
        return site


def heisenberg_su2(L, J=1.0):
    """Spin-1/2 XXX chain with SU(2) symmetry, H = J sum S_i . S_i+1, as the reference's
    HeisenbergSU2 builds it (models/HeisenbergSU2.h:270-283): the bond term is
    sqrt(3) J (S^dagger_i x S_i+1) coupled to a singlet.  One local multiplet (q = 2);
    reduced elements <1/2||S||1/2> = sqrt(S(S+1)) (sites/SpinSiteSU2.h:60) and
    S^dagger = the adjoint with coeff_adjoint(2, 2, 3) = -1 (tensors/SiteOperatorQ.h:292-305,
    symmetry/SU2.h:336-341)."""
    sym = Symmetry(("SU2",))
    qloc = [(2,)]
    s = np.array([[np.sqrt(0.75)]])
    sdag = -s
    ops = {"Sdag": (sdag, (3,)), "S": (s, (3,))}
    terms = [("Sdag", "S", np.sqrt(3.0) * J)]
    return SU2ChainModel(sym, L, qloc, ops, terms, [], name=f"HeisenbergSU2(L={L},J={J})")


def cylinder_bonds(Lx, W, t=1.0):
    """Bonds (i, j, t) of a width-W cylinder of Lx rings mapped to a snake: site x*W + y,
    hoppings around each ring (periodic in y) and between neighbouring rings (range W)."""
    bonds = set()
    for x in range(Lx):
        for y in range(W):
            i = x * W + y
            if W > 1:
                j = x * W + (y + 1) % W
                if j != i:
                    bonds.add((min(i, j), max(i, j)))
            if x + 1 < Lx:
                bonds.add((i, i + W))
    return [(i, j, t) for i, j in sorted(bonds)]


class LatticeModel(ChainModel):
    """MPO of a lattice Hamiltonian on a chain ordering (a two-dimensional lattice mapped to
    a snake): for every bond (i < j, t_ij) and every term (A, B, c) the product
    c t_ij A_i S_{i+1} ... S_{j-1} B_j, with the string operator S (the fermionic sign,
    a singlet), plus on-site terms.  This is the finite-state machine that the reference's
    MpoTerms builds from push_full / push_tight pushlists (MpoTerms.h, models/HubbardSU2xU1.h:
    188-233): auxiliary states IDLE, DONE and OPEN(term, k) = "A applied k sites to the
    left", present only on bonds that a lattice bond crosses (w = 2 + #terms x range in the
    bulk).  `reduced`: operators are SU(2)-reduced (matrix, operator multiplet) pairs and W
    holds reduced elements, as in SU2ChainModel; otherwise operator QNs follow from the
    local basis as in ChainModel."""

    def __init__(self, sym, L, qloc, ops, terms, bonds, onsite, string, reduced=False, name=""):
        self.bonds = {}
        for i, j, tij in bonds:
            if not (0 <= i < j < L):
                raise ValueError(f"bond ({i}, {j}) outside the chain")
            self.bonds[(i, j)] = self.bonds.get((i, j), 0.0) + tij
        self.string = string
        self.reduced = reduced
        super().__init__(sym, L, qloc, ops, terms, onsite, name=name)

    def _build(self):
        vac = self.sym.vacuum()
        need = [set() for _ in range(self.L + 1)]   # (term, k) open at bond l
        for (i, j) in self.bonds:
            for l in range(i + 1, j + 1):
                for t in range(len(self.terms)):
                    need[l].add((t, l - i))
        self.aux = []
        for l in range(self.L + 1):
            if l == 0:
                self.aux.append([("IDLE", vac)])
            elif l == self.L:
                self.aux.append([("DONE", vac)])
            else:
                opened = [(f"OPEN{t}_{k}", self.ops[self.terms[t][0]][1]) for t, k in sorted(need[l])]
                self.aux.append([("IDLE", vac)] + opened + [("DONE", vac)])
        self.W = [self._site(l) for l in range(self.L)]
        self.wdim = max(len(a) for a in self.aux)

    def _site(self, l):
        d = self.d
        ain, aout = self._sector_index(self.aux[l]), self._sector_index(self.aux[l + 1])
        vac = self.sym.vacuum()
        I = np.eye(d)
        S, qS = self.ops[self.string] if self.string else (I, vac)
        entries = []   # (state_in, state_out, matrix, operator QN)
        if "IDLE" in ain and "IDLE" in aout:
            entries.append(("IDLE", "IDLE", I, vac))
        if "DONE" in ain and "DONE" in aout:
            entries.append(("DONE", "DONE", I, vac))
        if "IDLE" in ain and "DONE" in aout and self.onsite:
            entries.append(("IDLE", "DONE", sum(c * self.ops[o][0] for o, c in self.onsite), vac))
        for t, (a, b, c) in enumerate(self.terms):
            if "IDLE" in ain and f"OPEN{t}_1" in aout:
                entries.append(("IDLE", f"OPEN{t}_1", self.ops[a][0], self.ops[a][1]))
            for k in range(1, l + 1):
                src = f"OPEN{t}_{k}"
                if src not in ain:
                    continue
                if f"OPEN{t}_{k + 1}" in aout:
                    entries.append((src, f"OPEN{t}_{k + 1}", S, qS))
                tij = self.bonds.get((l - k, l))
                if tij is not None and "DONE" in aout:
                    entries.append((src, "DONE", c * tij * self.ops[b][0], self.ops[b][1]))
        nz = []
        for sin, sout, M, qop in entries:
            for s1 in range(d):
                for s2 in range(d):
                    v = M[s1, s2]
                    if abs(v) < 1e-15:
                        continue
                    q = tuple(qop) if self.reduced else tuple(x - y for x, y in zip(self.qloc[s1], self.qloc[s2]))
                    nz.append((s1, s2, q, ain[sin], aout[sout], v))
        qop_list = sorted({e[2] for e in nz})
        kidx = {q: i for i, q in enumerate(qop_list)}
        site = MpoSite(nq=self.sym.nq, qloc=list(self.qloc), qop=qop_list)
        for s1, s2, q, (qi, ri), (qo, co), v in nz:
            if self.reduced:
                assert tuple(qo) in self.sym.fuse(tuple(qi), q), (qi, q, qo)
            else:
                assert tuple(x + y for x, y in zip(qi, q)) == tuple(qo), (qi, q, qo)
            site.add(s1, s2, kidx[q], qi, qo, ri, co, v)
        return site


def _hubbard_u1xu1_ops(U):
    qloc = [(0, 0), (1, 1), (1, -1), (2, 0)]
    cdu = np.zeros((4, 4)); cdu[1, 0] = 1.0; cdu[3, 2] = 1.0
    cdd = np.zeros((4, 4)); cdd[2, 0] = 1.0; cdd[3, 1] = -1.0
    F = np.diag([1.0, -1.0, -1.0, 1.0])
    cu, cd = cdu.T.copy(), cdd.T.copy()
    ops = {"cdu_F": (cdu @ F, (1, 1)), "cdd_F": (cdd @ F, (1, -1)), "F_cu": (F @ cu, (-1, -1)),
           "F_cd": (F @ cd, (-1, 1)), "cu": (cu, (-1, -1)), "cd": (cd, (-1, 1)), "cdu": (cdu, (1, 1)),
           "cdd": (cdd, (1, -1)), "nupdn": (np.diag([0.0, 0.0, 0.0, 1.0]), (0, 0)), "F": (F, (0, 0))}
    terms = [("cdu_F", "cu", -1.0), ("cdd_F", "cd", -1.0), ("F_cu", "cdu", -1.0), ("F_cd", "cdd", -1.0)]
    onsite = [("nupdn", U)] if U != 0 else []
    return qloc, ops, terms, onsite


def hubbard_u1xu1_lattice(L, bonds, U=4.0):
    """Hubbard model with U(1)xU(1) (N, 2Sz) on the bonds [(i, j, t_ij)] of a chain ordering."""
    qloc, ops, terms, onsite = _hubbard_u1xu1_ops(U)
    return LatticeModel(Symmetry(("U1", "U1")), L, qloc, ops, terms, bonds, onsite, "F", reduced=False,
                        name=f"HubbardU1xU1(L={L},bonds={len(bonds)},U={U})")


def _hubbard_su2xu1_ops(U):
    """SU(2)xU(1) local multiplets (2S+1, N): empty (1,0), single (2,1), double (1,2); reduced
    elements of FermionSite<SU2xU1> (sites/FermionSiteSU2xU1.h:100-123): <empty||c||single> =
    sqrt(2), <single||c||double> = 1; c^dagger = c.adjoint() with coeff_adjoint
    (tensors/SiteOperatorQ.h:292-305, symmetry/SU2.h:335-341), so <single||c^dag||empty> = 1,
    <double||c^dag||single> = -sqrt(2); the sign F = diag(1, -1, 1); products with the
    singlet F are plain matrix products (coeff_prod with a scalar factor is 1)."""
    qloc = [(1, 0), (2, 1), (1, 2)]
    c = np.zeros((3, 3)); c[0, 1] = np.sqrt(2.0); c[1, 2] = 1.0
    cdag = np.zeros((3, 3)); cdag[1, 0] = 1.0; cdag[2, 1] = -np.sqrt(2.0)
    F = np.diag([1.0, -1.0, 1.0])
    ops = {"cdagF": (cdag @ F, (2, 1)), "cF": (c @ F, (2, -1)), "c": (c, (2, -1)), "cdag": (cdag, (2, 1)),
           "d": (np.diag([0.0, 0.0, 1.0]), (1, 0)), "F": (F, (1, 0))}
    # hopping of HubbardSU2xU1 (models/HubbardSU2xU1.h:429-430): -sqrt(2) t [(c^dag F)_i c_j + (c F)_i c^dag_j]
    terms = [("cdagF", "c", -np.sqrt(2.0)), ("cF", "cdag", -np.sqrt(2.0))]
    onsite = [("d", U)] if U != 0 else []
    return qloc, ops, terms, onsite


def hubbard_su2xu1_lattice(L, bonds, U=8.0):
    """Hubbard model with SU(2)xU(1) (spin multiplet, N) on the bonds [(i, j, t_ij)] of a chain
    ordering, as the reference's HubbardSU2xU1 builds it."""
    qloc, ops, terms, onsite = _hubbard_su2xu1_ops(U)
    return LatticeModel(Symmetry(("SU2", "U1")), L, qloc, ops, terms, bonds, onsite, "F", reduced=True,
                        name=f"HubbardSU2xU1(L={L},bonds={len(bonds)},U={U})")


def hubbard_su2xu1(L, t=1.0, U=4.0):
    """Hubbard chain with SU(2)xU(1) symmetry (open, nearest-neighbour hopping)."""
    return hubbard_su2xu1_lattice(L, [(i, i + 1, t) for i in range(L - 1)], U=U)


# ---------------------------------------------------------------------------
# exact dense Hamiltonians (independent of the MPO), for the oracle's pins
# ---------------------------------------------------------------------------
def dense_heisenberg(L, J=1.0):
    """Full 2^L x 2^L XXX Hamiltonian, basis index = sum_i s_i 2^(L-1-i), s=0 up."""
    Sz = np.diag([0.5, -0.5]); Sp = np.array([[0.0, 1.0], [0.0, 0.0]]); Sm = Sp.T
    I = np.eye(2)

    def op(o, i):
        m = np.array([[1.0]])
        for j in range(L):
            m = np.kron(m, o if j == i else I)
        return m
    H = np.zeros((2 ** L, 2 ** L))
    for i in range(L - 1):
        H += J * (op(Sz, i) @ op(Sz, i + 1) + 0.5 * (op(Sp, i) @ op(Sm, i + 1) + op(Sm, i) @ op(Sp, i + 1)))
    return H


def dense_hubbard(L, t=1.0, U=4.0, bonds=None):
    """Full 4^L Hubbard Hamiltonian built from fermion modes (i,up),(i,dn) in order
    (0,up),(0,dn),(1,up),... with explicit Jordan-Wigner strings over all modes.
    `bonds` [(i, j, t_ij)] replaces the open chain's nearest-neighbour hoppings."""
    nm = 2 * L
    a = np.array([[0.0, 1.0], [0.0, 0.0]])   # annihilator on one mode (|0>,|1>)
    Z = np.diag([1.0, -1.0])
    I = np.eye(2)

    def ann(m):
        o = np.array([[1.0]])
        for j in range(nm):
            o = np.kron(o, Z if j < m else (a if j == m else I))
        return o
    c = [ann(m) for m in range(nm)]
    H = np.zeros((2 ** nm, 2 ** nm))
    for i, j, tij in (bonds if bonds is not None else [(i, i + 1, t) for i in range(L - 1)]):
        for s in range(2):
            m1, m2 = 2 * i + s, 2 * j + s
            hop = c[m1].T @ c[m2]
            H += -tij * (hop + hop.T)
    for i in range(L):
        H += U * (c[2 * i].T @ c[2 * i]) @ (c[2 * i + 1].T @ c[2 * i + 1])
    return H
