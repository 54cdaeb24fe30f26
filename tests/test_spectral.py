"""Start vectors of config C5 on the host: P c_{k,s}|psi> built by vmps_gb300.spectral
(annihilator MPO with the model's Jordan-Wigner string, operator environments
between the state and its re-labelled copy, the charge-changing two-site step as a
tagged pivot) with the oracle's contract_L / contract_R and two-site HxV in place
of the engine's, against c_{k,s}|psi> from dense matrices, on a chain whose pivot
bases are complete (so P = 1 on the sector)."""
import numpy as np
import pytest

import oracle
from oracle import ed
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS
from vmps_gb300.spectral import SpectralPivot, annihilator, relabel, standing_wave


def _oracle_env(side, E, Abra, W, Aket):
    return (oracle.contract_L if side == "L" else oracle.contract_R)(W.nq, E, Abra, W, Aket)


def _oracle_apply2(sym, L, R, W1, W2, V, x):
    return oracle.OraclePivot(2, sym.nq, L, R, V, W1, W2).hxv(x)


def _dense_c(model, coef, spin):
    """sum_j coef[j] F_0..F_{j-1} a_j in the kron basis (site 0 most significant)"""
    a, _, F = annihilator(model, spin)
    d, L = len(model.qloc), model.L
    out = 0
    for j in range(L):
        op = np.ones((1, 1))
        for i in range(L):
            op = np.kron(op, F if i < j else (a if i == j else np.eye(d)))
        out = out + coef[j] * op
    return out


def _relabelled(mps, l, dq):
    """the MPS with sites > l+1 (and their bonds) re-labelled by dq, for isometries"""
    import copy
    m = copy.copy(mps)
    m.A = list(mps.A)
    m.dims = list(mps.dims)
    for j in range(l + 2, mps.L):
        m.A[j] = relabel(mps.A[j], dq)
    m.Qtot = tuple(x + y for x, y in zip(mps.Qtot, dq))
    for b in range(l + 2, mps.L + 1):
        m.dims[b] = {tuple(x + y for x, y in zip(q, dq)): n for q, n in mps.dims[b].items()}
    return m


@pytest.mark.parametrize("spin,n", [("up", 1), ("dn", 3), ("up", 6)])
def test_projected_annihilator_equals_dense(spin, n):
    L, l = 6, 2
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 64, seed=11).canonicalize(l, l + 1)
    assert mps.bond_dim(l) == 16 and mps.bond_dim(l + 2) == 16   # complete bases
    sp = SpectralPivot(None, model, mps, l, spins=(spin,), env=_oracle_env, apply2=_oracle_apply2)
    coef = standing_wave(L, n)
    y = sp.project(coef, spin)
    _, _, Vb = sp.sector(spin)
    from vmps_gb300.mps import two_site_layout
    _, comb = two_site_layout(model.sym, model.qloc, model.qloc, dict(mps.dims[l]), dict(mps.dims[l + 2]), 2)
    P0 = ed.pivot2_isometry(mps, sp.V0, comb, l)
    psi = P0 @ sp.V0.data
    dq = annihilator(model, spin)[1]
    Pb = ed.pivot2_isometry(_relabelled(mps, l, dq), Vb, comb, l)
    ref = _dense_c(model, coef, spin) @ psi
    assert np.linalg.norm(ref) > 1e-3
    assert np.linalg.norm(Pb @ y - ref) < 1e-12 * np.linalg.norm(ref)
