"""Element-wise GPU parity with SU(2) symmetry: the engine's HxV (1- and 2-site)
and contract_L / contract_R against the oracle's SU(2) restatement on the same
seeded inputs, for the spin-1/2 Heisenberg chain with SU(2) and the Hubbard
model with SU(2)xU(1) on a cylinder (the C3 model family: reduced fermion
operators, sign strings, range-2 hoppings).  Tolerances as in test_gpu_parity:
FP64 1e-12, BF16x3 2e-4 relative."""
import numpy as np
import pytest

import oracle
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import EnvUpdate, PivotMatrix1, PivotMatrix2

from helpers import compare_tripods, rel_err
from test_oracle_su2 import su2_envs

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_SPLIT = 2e-4


def _cases():
    heis = models.heisenberg_su2(16)
    hub = models.hubbard_su2xu1_lattice(12, models.cylinder_bonds(6, 2), U=8.0)
    cyl = models.hubbard_su2xu1_lattice(16, models.cylinder_bonds(4, 4), U=8.0)
    return {"heisenberg_su2_L16_D48": (heis, (1,), 48, 7),
            "hubbard_su2xu1_ladder_L12_D64": (hub, (1, 12), 64, 5),
            "hubbard_su2xu1_cylinder_4x4_N14_D120": (cyl, (1, 14), 120, 7)}


@pytest.mark.parametrize("name", list(_cases()))
def test_su2_hxv_parity(gpu_ctx, name):
    m, Q, D, site = _cases()[name]
    sym, nq = m.sym, m.sym.nq
    rng = np.random.default_rng(3)
    # two-site pivot
    mps = RandomMPS(m, Q, D, seed=11, profile="gaussian", sigma=[2.0] * nq).canonicalize(site, site + 1)
    L, R = su2_envs(m, mps, site, site + 1)
    V = contract_two_sites(sym, mps.A[site], mps.A[site + 1], m.qloc, m.qloc, nq)
    H = PivotMatrix2(gpu_ctx, sym, L, R, m.W[site], m.W[site + 1], V)
    op = oracle.OraclePivot(2, nq, L, R, V, m.W[site], m.W[site + 1], sym=sym)
    v = rng.standard_normal(V.data.size)
    ref = op.hxv(v)
    assert np.linalg.norm(ref) > 0
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT
    assert H.stats()["n_tasks"] == op.n_tasks
    H.close()
    # one-site pivot
    mps = RandomMPS(m, Q, D, seed=12, profile="gaussian", sigma=[2.0] * nq).canonicalize(site, site)
    L, R = su2_envs(m, mps, site, site)
    H = PivotMatrix1(gpu_ctx, sym, L, R, m.W[site], mps.A[site])
    op = oracle.OraclePivot(1, nq, L, R, mps.A[site], m.W[site], sym=sym)
    v = rng.standard_normal(mps.A[site].data.size)
    ref = op.hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT
    H.close()


@pytest.mark.parametrize("name", list(_cases()))
def test_su2_env_parity(gpu_ctx, name):
    m, Q, D, site = _cases()[name]
    sym, nq = m.sym, m.sym.nq
    mps = RandomMPS(m, Q, D, seed=13, profile="gaussian", sigma=[2.0] * nq).canonicalize(site, site)
    L, R = su2_envs(m, mps, site, site)
    A, W = mps.A[site], m.W[site]
    for side, E in (("L", L), ("R", R)):
        ref = oracle.OracleEnv(side, nq, E, A, W, A, sym=sym).run(E, A, A)
        e = EnvUpdate(gpu_ctx, sym, side, E, A, W, A)
        assert compare_tripods(e.run(E, A, A, "fp64"), ref) < TOL_FP64
        assert compare_tripods(e.run(E, A, A, "bf16x3"), ref) < TOL_SPLIT
        e.close()
