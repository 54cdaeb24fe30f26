"""Subspace expansion of single-site DMRG (RICH_SVD: Mps::enrich_left / enrich_right,
Mps.h:3181-3600), abelian symmetries.

* An expansion step with room for every state changes the bond basis but not the
  state: the two-site tensor across the enlarged bond is the same to 1e-12, and the
  site left behind is orthonormal.
* Single-site DMRG cannot change its bond dimensions; with the expansion it grows
  them from a random D=4 MPS and reaches the exact ground energy (the reference's
  DMRG-vs-ED check, programs/test_Hubbard/test_Hubbard.cc:227-300), where the plain
  sweeps stay at the D=4 energy."""
import copy

import numpy as np
import pytest

from oracle import ed
from vmps_gb300 import models
from vmps_gb300.dmrg import dmrg1
from vmps_gb300.enrich import enrich_left, enrich_right
from vmps_gb300.mps import RandomMPS, contract_two_sites

from helpers import oracle_envs

pytestmark = pytest.mark.gpu


def _two_site_dense(model, mps, l):
    V = contract_two_sites(model.sym, mps.A[l], mps.A[l + 1], model.qloc, model.qloc, model.sym.nq)
    return {V.key(i): V.block(i) for i in range(V.n)}


@pytest.mark.parametrize("move", ["right", "left"])
def test_expansion_keeps_the_state(gpu_ctx, move):
    model = models.hubbard_u1xu1(8, t=1.0, U=4.0)
    l = 3
    mps = RandomMPS(model, (8, 0), 8, seed=4).canonicalize(l, l)
    ref = _two_site_dense(model, mps, l if move == "right" else l - 1)
    Lenv, Renv = oracle_envs(model, mps, l, l)
    d_old = mps.bond_dim(l + 1 if move == "right" else l)
    if move == "right":
        enrich_right(gpu_ctx, model, mps, l, Lenv, 0.1, 10_000)
        bond, site, pair = l + 1, l, l
    else:
        enrich_left(gpu_ctx, model, mps, l, Renv, 0.1, 10_000)
        bond, site, pair = l, l, l - 1
    assert mps.bond_dim(bond) > d_old
    got = _two_site_dense(model, mps, pair)
    for k, B in ref.items():
        G = got.get(k)
        assert G is not None and np.abs(G - B).max() < 1e-12 * max(1.0, np.abs(B).max()), k
    A = mps.A[site]
    for q in set(tuple(x) for x in (A.qout if move == "right" else A.qin)):
        blks = [A.block(i) for i in range(A.n) if tuple((A.qout if move == "right" else A.qin)[i]) == q]
        M = np.vstack(blks) if move == "right" else np.hstack(blks)
        G = M.T @ M if move == "right" else M @ M.T
        assert np.abs(G - np.eye(len(G))).max() < 1e-12


def _hubbard_sector(L, N, M):
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == N and sum(bits[0::2]) - sum(bits[1::2]) == M)
    return np.array(mask)


@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_single_site_with_expansion_reaches_ed(gpu_ctx, precision):
    L = 6
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 4, seed=5).canonicalize(0, 0)
    H = ed.permute_to_reference(ed.mpo_to_dense(model), model)
    e_ed = ed.ground_energy(H, _hubbard_sector(L, L, 0))
    kw = dict(tol_eigval=1e-11, tol_state=1e-7, refine_iters=10) if precision == "bf16x3" else {}
    plain = dmrg1(gpu_ctx, model, copy.deepcopy(mps), n_sweeps=4, precision=precision, **kw)
    assert plain["energies"][-1] - e_ed > 1e-4    # stuck at D=4
    rich = dmrg1(gpu_ctx, model, mps, n_sweeps=8, precision=precision, enrich=0.1, enrich_decay=0.3, Dmax=64, **kw)
    assert max(mps.bond_dim(b) for b in range(L + 1)) > 4
    assert abs(rich["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (rich["energies"], e_ed)
