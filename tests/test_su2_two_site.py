"""SU(2) two-site contraction and split (vmps_gb300/su2.py, the non-abelian
contract_AA2 / split_AA2) on the host:

* split after contract with room for every multiplet gives back the same state
  (the two-site tensor of the split sites equals the original, up to the split's
  normalisation), the left factor is left-orthonormal and the right factor right-
  orthonormal with the SU(2) weights q_out/q_in (coeff_rightOrtho);
* with an abelian symmetry every coefficient is 1 and the results equal the abelian
  routines of mps.py;
* truncation keeps the Dmax largest multiplets and reports the discarded weight
  with multiplet degeneracies."""
import numpy as np
import pytest

from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.su2 import Recoupling, contract_two_sites_su2, split_two_site_su2


def _case(kind, L=8, D=16, l=3, seed=3):
    if kind == "su2":
        model = models.heisenberg_su2(L)
        Q = (1,)
    else:
        model = models.hubbard_su2xu1_lattice(L, [(i, i + 1, 1.0) for i in range(L - 1)], U=4.0)
        Q = (1, L)
    mps = RandomMPS(model, Q, D, seed=seed).canonicalize(l, l + 1)
    return model, mps, l


def _dense(V):
    return {V.key(i): V.block(i).copy() for i in range(V.n)}


@pytest.mark.parametrize("kind", ["su2", "su2xu1"])
@pytest.mark.parametrize("move", ["right", "left"])
def test_split_after_contract_is_the_same_state(kind, move):
    model, mps, l = _case(kind)
    sym, q = model.sym, model.qloc
    V, comb = contract_two_sites_su2(sym, mps.A[l], mps.A[l + 1], q, q)
    din = {tuple(mps.A[l].qin[i]): int(mps.A[l].rows[i]) for i in range(mps.A[l].n)}
    dout = {tuple(mps.A[l + 1].qout[i]): int(mps.A[l + 1].cols[i]) for i in range(mps.A[l + 1].n)}
    A1, A2, disc, dmid = split_two_site_su2(V, comb, sym, q, q, din, dout, 10_000, move=move, eps_svd=1e-13)
    assert disc < 1e-12
    W, _ = contract_two_sites_su2(sym, A1, A2, q, q)
    a, b = _dense(V), _dense(W)
    scale = np.linalg.norm(W.data) / np.linalg.norm(V.data)
    for k, B in a.items():
        G = b.get(k)
        if G is None:
            assert np.abs(B).max() < 1e-12
            continue
        assert np.abs(G - scale * B).max() < 1e-11 * max(1.0, np.abs(B).max()), k
    rc = Recoupling(sym)
    # left-orthonormal: sum over (s, qin) of A^T A = 1 per outgoing multiplet (move right);
    # right-orthonormal: sum over (s, qout) of (q_out / q_in) A A^T = 1 (move left)
    if move == "right":
        for Q in dmid:
            G = sum(A1.block(i).T @ A1.block(i) for i in range(A1.n) if tuple(A1.qout[i]) == Q)
            assert np.abs(G - np.eye(dmid[Q])).max() < 1e-12
    else:
        for Q in dmid:
            G = sum(rc.degeneracy(tuple(A2.qout[j])) / rc.degeneracy(Q) * A2.block(j) @ A2.block(j).T
                    for j in range(A2.n) if tuple(A2.qin[j]) == Q)
            assert np.abs(G - np.eye(dmid[Q])).max() < 1e-12


def test_abelian_symmetry_reproduces_the_abelian_routines():
    model = models.hubbard_u1xu1(6, t=1.0, U=4.0)
    mps = RandomMPS(model, (6, 0), 12, seed=2).canonicalize(2, 3)
    q = model.qloc
    V1, _ = contract_two_sites_su2(model.sym, mps.A[2], mps.A[3], q, q)
    V2 = contract_two_sites(model.sym, mps.A[2], mps.A[3], q, q, model.sym.nq)
    assert np.array_equal(V1.data, V2.data)


def test_truncation_keeps_the_largest_multiplets():
    model, mps, l = _case("su2", L=10, D=24, l=4, seed=5)
    sym, q = model.sym, model.qloc
    V, comb = contract_two_sites_su2(sym, mps.A[l], mps.A[l + 1], q, q)
    din = {tuple(mps.A[l].qin[i]): int(mps.A[l].rows[i]) for i in range(mps.A[l].n)}
    dout = {tuple(mps.A[l + 1].qout[i]): int(mps.A[l + 1].cols[i]) for i in range(mps.A[l + 1].n)}
    _, _, d_all, m_all = split_two_site_su2(V, comb, sym, q, q, din, dout, 10_000)
    _, _, disc, dmid = split_two_site_su2(V, comb, sym, q, q, din, dout, 5)
    assert sum(dmid.values()) == 5 and sum(m_all.values()) > 5
    assert 0 < disc < 1 and d_all < 1e-12
