"""Union pivots (vmps_gb300/union.py) on the host: the part tag keeps the parts'
task lists apart, so the union's chains are exactly the parts' chains and its
layout is their concatenation (no GPU: host-only context, plans only)."""
import numpy as np

from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import Context, PivotMatrix2
from vmps_gb300.union import UnionPivot2, tag_blocks, tag_mpo, tagged_symmetry

from helpers import oracle_envs


def _part(model, Q, D, seed, site):
    mps = RandomMPS(model, Q, D, seed=seed).canonicalize(site, site + 1)
    Lenv, Renv = oracle_envs(model, mps, site, site + 1)
    V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, model.sym.nq)
    return Lenv, Renv, V


def test_union_chains_are_the_parts_chains():
    L, site = 8, 3
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    parts = [_part(model, (L - 1, -1), 16, 3, site), _part(model, (L - 1, 1), 16, 4, site),
             _part(model, (L, 0), 12, 5, site)]
    ctx = Context(-1)
    U = UnionPivot2(ctx, model.sym, model.W[site], model.W[site + 1], parts)
    su = U.H.stats("fp64")
    tot = {"n_chains": 0, "n_tasks": 0, "n_out_blocks": 0}
    for Lp, Rp, Vp in parts:
        H = PivotMatrix2(ctx, model.sym, Lp, Rp, model.W[site], model.W[site + 1], Vp)
        s = H.stats("fp64")
        for k in tot:
            tot[k] += s[k]
        H.close()
    for k, v in tot.items():
        assert su[k] == v, (k, su[k], v)
    assert U.H.dim == sum(U.dims)
    assert U.parts == [0, parts[0][2].n, parts[0][2].n + parts[1][2].n, sum(p[2].n for p in parts)]
    U.close()


def test_tagging_round_trip():
    model = models.hubbard_u1xu1(6, t=1.0, U=4.0)
    _, _, V = _part(model, (6, 0), 8, 1, 2)
    T = tag_blocks(V, 3)
    assert T.nq == V.nq + 1 and np.all(T.qin[:, -1] == 3) and np.all(T.qout[:, -1] == 3)
    assert np.array_equal(T.qin[:, :-1], V.qin) and T.data is V.data
    W = tag_mpo(model.W[2])
    assert W.nq == 3 and all(q[-1] == 0 for q in W.qin + W.qout + W.qloc + W.qop)
    assert tagged_symmetry(model.sym).kinds == ("U1", "U1", "U1")
