"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py) and
known-answer energies.

* CPU: the oracle re-run on the stored inputs reproduces the stored outputs
  (the oracle cannot drift unnoticed); closed-form ground-state energies of
  small chains pin the MPOs and the dense references.
* GPU: the engine on the stored inputs matches the stored outputs (FP64 1e-12,
  BF16x3 2e-4), and the engine's Lanczos reaches the closed-form energies.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from oracle import ed
from vmps_gb300 import models

from helpers import blocks_from_npz, compare_tripods, mpo_from_npz, rel_err

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PIVOTS = sorted(glob.glob(os.path.join(GOLDEN, "pivot*.npz")))
ENVS = sorted(glob.glob(os.path.join(GOLDEN, "env*.npz")))

E_HEIS_4 = -(3.0 + 2.0 * np.sqrt(3.0)) / 4.0      # open S=1/2 Heisenberg chain, 4 sites
E_HUBB_2 = (4.0 - np.sqrt(4.0 ** 2 + 16.0)) / 2.0   # Hubbard dimer, t=1, U=4, N=2, Sz=0


def _pivot(z):
    kind = int(z["kind"][0])
    L, R, V = blocks_from_npz("L", z), blocks_from_npz("R", z), blocks_from_npz("V", z)
    W = [mpo_from_npz(p, z) for p in ("W", "W2") if p + "_val" in z]
    return kind, L, R, V, W


def _oracle_pivot(kind, L, R, V, W):
    return oracle.OraclePivot(kind, V.nq, L, R, V, *W)


def test_golden_fixtures_present():
    assert len(PIVOTS) >= 4 and len(ENVS) >= 1


@pytest.mark.parametrize("path", PIVOTS, ids=[os.path.basename(p) for p in PIVOTS])
def test_oracle_reproduces_golden_pivot(path):
    z = np.load(path)
    kind, L, R, V, W = _pivot(z)
    assert rel_err(_oracle_pivot(kind, L, R, V, W).hxv(z["v"]), z["out"]) < 1e-13


@pytest.mark.parametrize("path", ENVS, ids=[os.path.basename(p) for p in ENVS])
def test_oracle_reproduces_golden_env(path):
    z = np.load(path)
    for side in ("L", "R"):
        E, A, W = blocks_from_npz(side + "old", z), blocks_from_npz(side + "A", z), mpo_from_npz(side + "W", z)
        got = oracle.OracleEnv(side, E.nq, E, A, W, A).run(E, A, A)
        assert compare_tripods(got, blocks_from_npz(side + "new", z)) < 1e-13


def test_known_heisenberg_chain_4():
    H = models.dense_heisenberg(4)
    assert abs(np.linalg.eigvalsh(H)[0] - E_HEIS_4) < 1e-13
    assert abs(np.linalg.eigvalsh(ed.mpo_to_dense(models.heisenberg_u1(4)))[0] - E_HEIS_4) < 1e-13


def _hubbard_sector(L, N, M):
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == N and sum(bits[0::2]) - sum(bits[1::2]) == M)
    return np.array(mask)


def test_known_hubbard_dimer():
    H = models.dense_hubbard(2, t=1.0, U=4.0)
    assert abs(ed.ground_energy(H, _hubbard_sector(2, 2, 0)) - E_HUBB_2) < 1e-13
    m = models.hubbard_u1xu1(2, t=1.0, U=4.0)
    Hm = ed.permute_to_reference(ed.mpo_to_dense(m), m)
    assert abs(ed.ground_energy(Hm, _hubbard_sector(2, 2, 0)) - E_HUBB_2) < 1e-13


# ---- GPU ---------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("path", PIVOTS, ids=[os.path.basename(p) for p in PIVOTS])
def test_engine_matches_golden_pivot(gpu_ctx, path):
    from vmps_gb300.pivot import PivotMatrix0, PivotMatrix1, PivotMatrix2
    z = np.load(path)
    kind, L, R, V, W = _pivot(z)
    sym = models.heisenberg_u1(2).sym if V.nq == 1 else models.hubbard_u1xu1(2).sym
    H = {0: lambda: PivotMatrix0(gpu_ctx, sym, L, R, V), 1: lambda: PivotMatrix1(gpu_ctx, sym, L, R, W[0], V),
         2: lambda: PivotMatrix2(gpu_ctx, sym, L, R, W[0], W[1], V)}[kind]()
    assert rel_err(H.apply(z["v"], "fp64"), z["out"]) < 1e-12
    assert rel_err(H.apply(z["v"], "bf16x3"), z["out"]) < 2e-4
    H.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", ENVS, ids=[os.path.basename(p) for p in ENVS])
def test_engine_matches_golden_env(gpu_ctx, path):
    from vmps_gb300.pivot import EnvUpdate
    z = np.load(path)
    for side in ("L", "R"):
        E, A, W = blocks_from_npz(side + "old", z), blocks_from_npz(side + "A", z), mpo_from_npz(side + "W", z)
        sym = models.heisenberg_u1(2).sym if E.nq == 1 else models.hubbard_u1xu1(2).sym
        e = EnvUpdate(gpu_ctx, sym, side, E, A, W, A)
        ref = blocks_from_npz(side + "new", z)
        assert compare_tripods(e.run(E, A, A, "fp64"), ref) < 1e-12
        assert compare_tripods(e.run(E, A, A, "bf16x3"), ref) < 2e-4
        e.close()


@pytest.mark.gpu
def test_engine_lanczos_hubbard_dimer_closed_form(gpu_ctx):
    """two-site pivot of the whole Hubbard dimer: its ground state is the exact one"""
    from vmps_gb300.mps import RandomMPS, contract_two_sites
    from vmps_gb300.pivot import PivotMatrix2, left_vacuum, right_target
    m = models.hubbard_u1xu1(2, t=1.0, U=4.0)
    mps = RandomMPS(m, (2, 0), 8, seed=1).canonicalize(0, 1)
    V = contract_two_sites(m.sym, mps.A[0], mps.A[1], m.qloc, m.qloc, 2)
    H = PivotMatrix2(gpu_ctx, m.sym, left_vacuum(m.sym), right_target(m.sym, mps.Qtot), m.W[0], m.W[1], V)
    v0 = np.random.default_rng(2).standard_normal(H.dim)
    e64, _, _ = H.lanczos(v0, "fp64", max_iter=50, tol_eigval=1e-14, tol_state=1e-10)
    es, _, _ = H.lanczos(v0, "bf16x3", max_iter=50, tol_eigval=1e-9, tol_state=1e-6, refine_iters=20)
    assert abs(e64 - E_HUBB_2) < 1e-12
    assert abs(es - E_HUBB_2) < 1e-10
    H.close()


@pytest.mark.gpu
def test_engine_dmrg_heisenberg_4_closed_form(gpu_ctx):
    from vmps_gb300.dmrg import dmrg1
    from vmps_gb300.mps import RandomMPS
    m = models.heisenberg_u1(4)
    # D = 8 gives complete bond bases (the middle bond needs Sz=0 twice); single-site
    # sweeps keep the bases fixed, so smaller D cannot reach the exact state
    mps = RandomMPS(m, (0,), 8, seed=3).canonicalize(0, 0)
    res = dmrg1(gpu_ctx, m, mps, n_sweeps=2, precision="fp64")
    assert abs(res["energies"][-1] - E_HEIS_4) < 1e-12
