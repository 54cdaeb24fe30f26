"""Infinite-MPS quantities of config C4 (vmps_gb300/uniform.py) on the host, with the
oracle's contract_L / contract_R, transfer operator and pivots in the engine's place:

* gauge fixing of a uniform SU(2) MPS with a two-site cell: AL C = C AR, and the
  identity is the fixed point of the left (AL) and right (AR) transfer with W = 1;
* the energy density from the MPO environments (VumpsSolver::build_L / build_R, the
  GMRES slot solved to 1e-12) equals the mean of the two bond energies computed
  directly as two-site expectation values <AC AR| h |AC AR> (gauge invariant), and
  e_L = e_R;
* the gradient norm is the same for the left and right contraction orders of its terms."""
import numpy as np
import pytest

import oracle
from oracle.vumps_cpu import transfer_hxv
from vmps_gb300 import models
from vmps_gb300.blocks import Blocks
from vmps_gb300.su2 import contract_two_sites_su2
from vmps_gb300.uniform import UniformEnvironment, UniformMPS, bond_bases_su2
from vmps_gb300.vumps import MpoTransferMatrix


def oracle_hooks(sym):
    def env(side, mode, fixed_ab, order, E, Abra, W, Aket):
        return oracle.OracleEnv(side, sym.nq, E, Abra, W, Aket, mode=mode, fixed_ab=fixed_ab, order=order,
                                sym=sym).run(E, Abra, Aket)

    class Transfer(MpoTransferMatrix):
        def __init__(self, side, A, W, LR, ab, order, V):
            self.sym, self.V, self.ab = sym, V, ab
            self.ab_key = {v: k for k, v in order.items()}[ab]
            self.args = (side, A, W, LR, ab, order)

        def hxv(self, vin, precision="fp64"):
            side, A, W, LR, ab, order = self.args
            return transfer_hxv(side, sym.nq, A, A, W, LR, ab, order, self.V, vin, sym.dot_weight, sym=sym)

        def close(self):
            pass

    def transfer(side, A, W, LR, ab, order, V, b):
        return Transfer(side, A, W, LR, ab, order, V).solve_linear(b, tol=1e-12, dimK=100)

    def apply(kind, L, R, W, V, x):
        if kind == 1:
            return oracle.OraclePivot(1, sym.nq, L, R, V, W, sym=sym).hxv(x)
        return oracle.OraclePivot(0, sym.nq, L, R, V, sym=sym).hxv(x)
    return env, transfer, apply


def _case(nmult=16, qmax=8, seed=3):
    m = models.heisenberg_su2(8)
    u = UniformMPS(m, bond_bases_su2(nmult, qmax), seed=seed)
    g = u.gauge()
    return m, u, g


def test_gauge_fixing_two_site_cell():
    m, u, g = _case()
    assert g["gauge_err"] < 1e-12 and g["left"] < 500 and g["right"] < 500
    order = m.basis_order_map(4)
    E = UniformEnvironment(None, m, u, [m.W[4], m.W[5]], order, env=oracle_hooks(m.sym)[0])
    Lid = E._identity(E.first, 0)
    L1 = oracle.OracleEnv("L", 1, Lid, u.AL[0], m.W[4], u.AL[0], mode="FIXED_COLS", fixed_ab=E.first, order=order,
                          sym=m.sym).run(Lid, u.AL[0], u.AL[0])
    for i in range(L1.n):
        assert np.abs(L1.block(i) - np.eye(L1.rows[i])).max() < 1e-12
    Rid = E._identity(E.last, 1)
    R0 = oracle.OracleEnv("R", 1, Rid, u.AR[0], m.W[4], u.AR[0], mode="FIXED_ROWS", fixed_ab=E.last, order=order,
                          sym=m.sym).run(Rid, u.AR[0], u.AR[0])
    for i in range(R0.n):
        assert np.abs(R0.block(i) - np.eye(R0.rows[i])).max() < 1e-12


def test_energy_density_equals_bond_expectation_values():
    m, u, _ = _case()
    sym, order, W = m.sym, m.basis_order_map(4), [m.W[4], m.W[5]]
    env, transfer, apply = oracle_hooks(sym)
    E = UniformEnvironment(None, m, u, W, order, env=env, transfer=transfer, apply=apply)
    E.left()
    E.right()
    assert E.info["gmres_left"]["residual"] < 1e-11 and E.info["gmres_right"]["residual"] < 1e-11
    assert abs(E.eL - E.eR) < 1e-12
    bonds = []
    for l in range(2):
        V, _ = contract_two_sites_su2(sym, u.AC[l], u.AR[(l + 1) % 2], m.qloc, m.qloc)
        Lid, Rid = E._identity(E.first, l), E._identity(E.last, l)
        op = oracle.OraclePivot(2, 1, Lid, Rid, V, W[l], W[(l + 1) % 2], sym=sym)
        w = oracle.dot_weights(V, sym) ** 2
        assert abs(np.sum(w * V.data ** 2) - 1) < 1e-12        # normalised state
        bonds.append(float(np.sum(w * V.data * op.hxv(V.data))))
    assert abs(E.energy_density() - np.mean(bonds)) < 1e-12
    g, parts = E.gradient()
    assert g > 0 and len(parts) == 2 and abs(g - np.sqrt(sum(p * p for p in parts))) < 1e-14
