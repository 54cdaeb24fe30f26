"""3xTF32, the alternative split form: the same three products per K step as
BF16x3 (lo*hi + hi*lo + hi*hi, FP32 accumulation) with TF32 hi/lo operands in FP32
panels, kind::tf32 MMAs.  Against the oracle: HxV (1- and 2-site pivots, U(1) and
SU(2)) within 5e-6 relative and below the BF16x3 error; Lanczos with FP64
refinement to 1e-10 of the oracle's energy."""
import numpy as np
import pytest

import oracle
from vmps_gb300 import _native as N
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import PivotMatrix1, PivotMatrix2

from helpers import pivot1_case, pivot2_case, rel_err
from test_oracle_su2 import su2_envs

pytestmark = pytest.mark.gpu

TOL_TF32 = 5e-6


@pytest.mark.parametrize("kind,L,D,site", [("hubb", 8, 32, 3), ("hubb", 16, 128, 7), ("heis", 16, 64, 7)])
def test_tf32x3_hxv2_parity(gpu_ctx, kind, L, D, site):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case(kind, L=L, D=D, site=site, seed=22, profile="gaussian")
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    op = oracle.OraclePivot(2, model.sym.nq, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(8).standard_normal(V.data.size)
    ref = op.hxv(v)
    e_tf = rel_err(H.apply(v, "tf32x3"), ref)
    e_bf = rel_err(H.apply(v, "bf16x3"), ref)
    assert e_tf < TOL_TF32, e_tf
    assert e_tf < e_bf / 4, (e_tf, e_bf)
    assert np.array_equal(H.apply(v, "tf32x3"), H.apply(v, "tf32x3"))   # deterministic
    H.close()


def test_tf32x3_hxv1_and_su2(gpu_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("hubb", L=8, D=32, site=3, seed=21)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    op = oracle.OraclePivot(1, model.sym.nq, Lenv, Renv, V, W)
    v = np.random.default_rng(7).standard_normal(V.data.size)
    assert rel_err(H.apply(v, "tf32x3"), op.hxv(v)) < TOL_TF32
    H.close()
    m = models.heisenberg_su2(16)
    mps = RandomMPS(m, (1,), 48, seed=11, profile="gaussian", sigma=[2.0]).canonicalize(7, 8)
    L, R = su2_envs(m, mps, 7, 8)
    V = contract_two_sites(m.sym, mps.A[7], mps.A[8], m.qloc, m.qloc, 1)
    H = PivotMatrix2(gpu_ctx, m.sym, L, R, m.W[7], m.W[8], V)
    op = oracle.OraclePivot(2, 1, L, R, V, m.W[7], m.W[8], sym=m.sym)
    v = np.random.default_rng(3).standard_normal(V.data.size)
    assert rel_err(H.apply(v, "tf32x3"), op.hxv(v)) < TOL_TF32
    H.close()


def test_tf32x3_lanczos_and_unsupported_paths(gpu_ctx):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=16, D=128, site=7, seed=22, profile="gaussian")
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    v0 = np.random.default_rng(3).standard_normal(V.data.size)
    e_or, _ = oracle.lanczos_ground(op.hxv, v0)
    e, _, st = H.lanczos(v0, "tf32x3", max_iter=300, tol_eigval=1e-12, tol_state=1e-7, refine_iters=10)
    assert st["hxv_split"] > 0
    assert abs(e - e_or) <= 1e-10 * abs(e_or), (e, e_or)
    with pytest.raises(N.VmpsError):
        H.apply_multi(np.stack([v0, v0]), "tf32x3")
    H.close()
