"""Parity pinned to the reference's own golden data: the staggered magnetisation
of the L=12 Neel state under the XXZ chain (Jxy = -1, Jz = 0, -1, -2, -4), the
files programs/test_Heisenberg/ref/Mstag_Jxy=-1_Jz=*.dat (31 points, t = 0..6),
committed as tests/golden/mstag_heisenberg_L12.npz by tests/golden/make_mstag.py.

The reference computed them with TDVP (test_Heisenberg.cc:279-310) and printed 6
significant digits.  Exact dynamics deviates from the files by at most 5.2e-5
(at Jz = -4; 4.7e-6 at Jz = 0): the reference's own time-stepping error.  The
tests therefore ask for
  * 1e-4 absolute against the reference's files (every point of all four), and
  * 1e-9 absolute against exact diagonalisation (the path's own accuracy),
with the oracle's HxV on the CPU and with the engine's HxV (FP64) on the GPU, on
a two-site pivot whose complete bond bases span the whole Sz = 0 sector."""
import os

import numpy as np
import pytest

import oracle
from dynamics import L_DYN, exact_mstag, mstag_series, neel_case, neel_vector
from helpers import oracle_envs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mstag_heisenberg_L12.npz")
TOL_REF = 1e-4
TOL_EXACT = 1e-9


def _gold(jz):
    d = np.load(GOLD)
    return d[f"t_Jz{jz}"], d[f"mstag_Jz{jz}"]


def _oracle_apply(op):
    return lambda X: np.stack([op.hxv(X[0]), op.hxv(X[1])])


@pytest.mark.parametrize("jz", [0, -1, -2, -4])
def test_mstag_oracle_matches_reference_files(jz):
    t, ref = _gold(jz)
    model, obs, mps, site, V, comb, neel = neel_case(Jxy=-1.0, Jz=float(jz))
    LH, RH = oracle_envs(model, mps, site, site + 1)
    LM, RM = oracle_envs(obs, mps, site, site + 1)
    opH = oracle.OraclePivot(2, 1, LH, RH, V, model.W[site], model.W[site + 1])
    opM = oracle.OraclePivot(2, 1, LM, RM, V, obs.W[site], obs.W[site + 1])
    psi0 = neel_vector(mps, site, V, comb, neel)
    assert abs(np.linalg.norm(psi0) - 1.0) < 1e-12   # complete bases: the Neel state lies in the pivot space
    got = mstag_series(_oracle_apply(opH), _oracle_apply(opM), psi0, t)
    exact = exact_mstag(L_DYN, -1.0, float(jz), t)
    assert np.max(np.abs(got - exact)) < TOL_EXACT
    assert np.max(np.abs(got - ref)) < TOL_REF, np.max(np.abs(got - ref))


@pytest.mark.gpu
@pytest.mark.parametrize("jz", [0, -1, -2, -4])
def test_mstag_engine_matches_reference_files(gpu_ctx, jz):
    from vmps_gb300.pivot import PivotMatrix2
    from vmps_gb300.workloads import build_envs
    t, ref = _gold(jz)
    model, obs, mps, site, V, comb, neel = neel_case(Jxy=-1.0, Jz=float(jz))
    LH, RH = build_envs(gpu_ctx, model, mps, site, site + 1)
    LM, RM = build_envs(gpu_ctx, obs, mps, site, site + 1)
    H = PivotMatrix2(gpu_ctx, model.sym, LH, RH, model.W[site], model.W[site + 1], V)
    M = PivotMatrix2(gpu_ctx, obs.sym, LM, RM, obs.W[site], obs.W[site + 1], V)
    psi0 = neel_vector(mps, site, V, comb, neel)
    got = mstag_series(lambda X: H.apply_multi(X, "fp64"), lambda X: M.apply_multi(X, "fp64"), psi0, t)
    exact = exact_mstag(L_DYN, -1.0, float(jz), t)
    assert np.max(np.abs(got - exact)) < TOL_EXACT
    assert np.max(np.abs(got - ref)) < TOL_REF, np.max(np.abs(got - ref))
    H.close()
    M.close()
