"""Momentum-resolved single-particle start vectors P c_{k,s}|0> on a two-site pivot, and
the pivots of their sectors (config C5: a Chebyshev spectral function of the Hubbard
chain from a ground state |0>).

The reference builds c_k|0> as an MPS (an MPO of the momentum-resolved annihilator
applied to the ground state, then compressed) and runs one polynomial recursion per
start vector (polyIter, DmrgLinearAlgebra.h:550-566; MpsCompressor::prodCompress /
polyCompress, solvers/MpsCompressor.h:961-1564).  Here the start vectors live in one
two-site pivot space, that of sites (l, l+1) of the ground state, in the sector of
c_{k,s}|0>:

    P c_{k,s}|0>[aL, s1 s2, aR] = <aL s1 s2 aR| sum_j f_k(j) c_{j,s} |0>,

with |aL> the ground state's left basis and |aR> its right basis re-labelled for the
new total quantum number.  With the Jordan-Wigner string of the model (c_j = F_0 ..
F_{j-1} a_j, models.hubbard_u1xu1) the annihilator sum is an MPO of bond dimension 2
(pending: F; applied: identity; the step between them f_k(j) a_j), so the projection
is one effective-operator application: its environments L_O, R_O come from the
engine's contract_L / contract_R between the ground state (ket) and its re-labelled
copy (bra), and the two-site step is a pivot whose blocks carry a tag (0: ket, 1:
bra; union.py), since the operator changes the sector.  When the pivot's bond bases
are complete this is c_{k,s}|0> itself (tested against exact diagonalisation).
f_k(j) = sqrt(2/(L+1)) sin(k (j+1)), k = pi n/(L+1): the standing waves of the open
chain.
"""
from __future__ import annotations

import numpy as np

from .blocks import Blocks, MpoSite
from .mps import contract_two_sites, two_site_layout
from .pivot import EnvUpdate, PivotMatrix2, left_vacuum, right_target
from .union import UnionPivot2, aux_tag, bra_ket_tag, concat_blocks, tag_blocks, tagged_symmetry


def standing_wave(L: int, n: int) -> np.ndarray:
    """f_k(j) = sqrt(2/(L+1)) sin(k (j+1)), k = pi n / (L+1), j = 0..L-1"""
    k = np.pi * n / (L + 1)
    return np.sqrt(2.0 / (L + 1)) * np.sin(k * (np.arange(L) + 1))


def _add(a, b):
    return tuple(x + y for x, y in zip(a, b))


def annihilator(model, spin: str):
    """(a_s, its quantum number, the local parity F) of a U(1)xU(1) Hubbard chain"""
    a, q = model.ops["cu" if spin == "up" else "cd"]
    F = np.diag([(-1.0) ** int(ql[0]) for ql in model.qloc])
    return np.asarray(a), tuple(q), F


def annihilator_mpo(model, coef, spin: str) -> list:
    """MPO of sum_j coef[j] c_{j,spin}: per site, auxiliary states P (quantum number
    vacuum, the operator still to come: F) and D (the operator's quantum number,
    applied: identity), W[P, D] = coef[j] a_j"""
    a, dq, F = annihilator(model, spin)
    vac = model.sym.vacuum()
    qop = [vac, dq]
    W = []
    for j in range(model.L):
        w = MpoSite(model.sym.nq, list(model.qloc), qop)
        for s in range(len(model.qloc)):
            w.add(s, s, 0, vac, vac, 0, 0, F[s, s])
            w.add(s, s, 0, dq, dq, 0, 0, 1.0)
        if coef[j] != 0.0:
            for s1 in range(len(model.qloc)):
                for s2 in range(len(model.qloc)):
                    if a[s1, s2] != 0.0:
                        w.add(s1, s2, 1, vac, dq, 0, 0, coef[j] * a[s1, s2])
        W.append(w)
    return W


def relabel(A: Blocks, dq) -> Blocks:
    """a site tensor with its bond quantum numbers shifted by dq (the same states as a
    basis for total quantum number Qtot + dq)"""
    d = np.asarray(dq, dtype=np.int32)
    return Blocks(A.nq, A.qin + d, A.qout + d, A.leg, A.rows, A.cols, data=A.data, offset=A.offset)


def _shift_dims(dims: dict, dq) -> dict:
    return {_add(q, dq): n for q, n in dims.items()}


class SpectralPivot:
    """The two-site pivot (l, l+1) of a ground state `mps` (sites < l left-, > l+1 right-
    normalised) and the sectors of c_{k,s}|0> for the given spins.

    start_vectors(ns, spin): P c_{k,s}|0> for k = pi n/(L+1), n in ns (rows), in the
    layout of the sector's pivot; sector(spin): (Lenv, Renv, V layout) of H in that
    sector; union(): the UnionPivot2 of the spins' sectors.

    env(side, E, Abra, W, Aket) and apply2(sym, L, R, W1, W2, V, x) are the environment
    update and the FP64 two-site pivot application; by default the engine's."""

    def __init__(self, ctx, model, mps, l: int, spins=("up", "dn"), env=None, apply2=None):
        self.ctx, self.model, self.mps, self.l = ctx, model, mps, l
        self.sym = model.sym
        self.spins = list(spins)
        self.env = env or self._engine_env
        self.apply2 = apply2 or self._engine_apply2
        self.V0 = contract_two_sites(self.sym, mps.A[l], mps.A[l + 1], model.qloc, model.qloc, self.sym.nq)
        # H's left environment (sector independent) at bond l
        Lenv = left_vacuum(self.sym)
        for j in range(l):
            Lenv = self.env("L", Lenv, mps.A[j], model.W[j], mps.A[j])
        self.LH = Lenv
        self._sectors = {}

    def _engine_env(self, side, E, Abra, W, Aket):
        e = EnvUpdate(self.ctx, self.sym, side, E, Abra, W, Aket)
        try:
            return e.run(E, Abra, Aket)
        finally:
            e.close()

    def _engine_apply2(self, sym, L, R, W1, W2, V, x):
        H = PivotMatrix2(self.ctx, sym, L, R, W1, W2, V)
        try:
            return H.apply(x, "fp64")
        finally:
            H.close()

    def _dq(self, spin):
        return annihilator(self.model, spin)[1]

    def sector(self, spin):
        """(Lenv, Renv, V layout) of H in the sector Qtot + dq(spin)"""
        if spin not in self._sectors:
            m, mps, l, dq = self.model, self.mps, self.l, self._dq(spin)
            Q = _add(mps.Qtot, dq)
            R = right_target(self.sym, Q)
            for j in range(m.L - 1, l + 1, -1):
                Ar = relabel(mps.A[j], dq)
                R = self.env("R", R, Ar, m.W[j], Ar)
            V, _ = two_site_layout(self.sym, m.qloc, m.qloc, dict(mps.dims[l]), _shift_dims(mps.dims[l + 2], dq),
                                   self.sym.nq)
            self._sectors[spin] = (self.LH, R, V)
        return self._sectors[spin]

    def start_vectors(self, ns, spin) -> np.ndarray:
        """rows P c_{k_n,spin}|0>, n in ns, in the layout of sector(spin)"""
        _, _, Vb = self.sector(spin)
        return np.stack([self.project(standing_wave(self.model.L, n), spin) for n in ns]) if len(ns) else \
            np.zeros((0, Vb.data.size))

    def project(self, coef, spin) -> np.ndarray:
        """P sum_j coef[j] c_{j,spin} |0> in the layout of sector(spin)"""
        m, mps, l, dq = self.model, self.mps, self.l, self._dq(spin)
        sym = self.sym
        _, _, Vb = self.sector(spin)
        W = annihilator_mpo(m, coef, spin)
        LO = left_vacuum(sym)
        for j in range(l):
            LO = self.env("L", LO, mps.A[j], W[j], mps.A[j])
        # the right boundary: the operator applied (state D), ket total Qtot (rows), bra Qtot + dq
        RO = Blocks.from_entries(sym.nq, [(0, tuple(mps.Qtot), _add(mps.Qtot, dq), tuple(dq), np.ones((1, 1)))],
                                 tripod=True)
        for j in range(m.L - 1, l + 1, -1):
            RO = self.env("R", RO, relabel(mps.A[j], dq), W[j], mps.A[j])
        # the charge-changing step as a tagged pivot: ket blocks tag 0, bra blocks tag 1
        tsym = tagged_symmetry(sym)
        Lt, Rt = bra_ket_tag(LO, "L"), bra_ket_tag(RO, "R")
        W1, W2 = aux_tag(W[l]), aux_tag(W[l + 1])
        V = concat_blocks([tag_blocks(self.V0, 0), tag_blocks(Vb, 1)])
        x = np.concatenate([self.V0.data, np.zeros(Vb.data.size)])
        y = self.apply2(tsym, Lt, Rt, W1, W2, V, x)
        return np.array(y[self.V0.data.size:])

    def union(self, ctx=None) -> UnionPivot2:
        """one pivot over the spins' sectors (parts in the order of self.spins)"""
        return UnionPivot2(ctx or self.ctx, self.sym, self.model.W[self.l], self.model.W[self.l + 1],
                           [self.sector(s) for s in self.spins])
