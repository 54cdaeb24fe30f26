"""Many right-hand sides (config C5's batched HxV) and the Chebyshev recursion.

* vmps_hxv_multi in split precision runs all right-hand sides in one grouped
  HxV; every right-hand side's result equals the single-vector split HxV bit for
  bit (same K order per element), and matches the FP64 HxV and the oracle;
* spectral bounds: the extreme Ritz values equal the dense eigenvalues of the
  effective Hamiltonian on a small pivot;
* Chebyshev moments (polyIter recursion, FP64 moments): FP64 against a dense
  numpy recursion; split precision against FP64, error per moment reported.
"""
import numpy as np
import pytest

import oracle
from vmps_gb300.pivot import PivotMatrix1, PivotMatrix2

from helpers import pivot1_case, pivot2_case, rel_err

pytestmark = pytest.mark.gpu


def _pivot2(gpu_ctx, L=8, D=24, site=3, seed=51):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=L, D=D, site=site, seed=seed)
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    return H, op


@pytest.mark.parametrize("nrhs", [2, 5, 32])
def test_hxv_multi_matches_single(gpu_ctx, nrhs):
    H, op = _pivot2(gpu_ctx)
    X = np.random.default_rng(nrhs).standard_normal((nrhs, H.dim))
    ms = H.apply_multi(X, "bf16x3")
    m64 = H.apply_multi(X, "fp64")
    for k in range(nrhs):
        assert np.array_equal(ms[k], H.apply(X[k], "bf16x3")), k
        assert np.array_equal(m64[k], H.apply(X[k], "fp64")), k
        ref = op.hxv(X[k])
        assert rel_err(m64[k], ref) < 1e-12
        assert rel_err(ms[k], ref) < 2e-4
    H.close()


def test_hxv_multi_single_site_heisenberg(gpu_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=12, D=32, site=5, seed=52)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    X = np.random.default_rng(3).standard_normal((7, H.dim))
    ms = H.apply_multi(X, "bf16x3")
    for k in range(7):
        assert np.array_equal(ms[k], H.apply(X[k], "bf16x3"))
    H.close()


def _dense(op, n):
    M = np.column_stack([op.hxv(np.eye(n)[:, j]) for j in range(n)])
    return 0.5 * (M + M.T)


def test_spectral_bounds_and_chebyshev_moments(gpu_ctx):
    H, op = _pivot2(gpu_ctx, L=6, D=8, site=2, seed=53)
    n = H.dim
    assert n <= 2000
    Hd = _dense(op, n)
    ev = np.linalg.eigvalsh(Hd)
    rng = np.random.default_rng(4)
    lo, hi = H.spectral_bounds(rng.standard_normal(n), iters=min(n - 1, 300))
    assert ev[0] - 1e-9 <= lo <= ev[0] + 1e-8 * max(1, abs(ev[0])), (lo, ev[0])
    assert ev[-1] - 1e-8 * max(1, abs(ev[-1])) <= hi <= ev[-1] + 1e-9, (hi, ev[-1])
    # rescale into [-1, 1] with a 2 % margin
    a = (hi - lo) / (2 * 0.98)
    b = (hi + lo) / 2
    V0 = rng.standard_normal((3, n))
    nmom = 41
    mu64, st64 = H.chebyshev_moments(V0, nmom, a, b, "fp64")
    mus, sts = H.chebyshev_moments(V0, nmom, a, b, "bf16x3")
    assert st64["steps"] == (nmom + 1) // 2 and st64["hxv"] == 3 * st64["steps"]
    Ht = (Hd - b * np.eye(n)) / a
    for k in range(3):
        t0, t1 = V0[k], Ht @ V0[k]
        ref = [t0 @ t0, t1 @ t0]
        tp, tc = t0, t1
        for _ in range(2, nmom):
            tp, tc = tc, 2 * Ht @ tc - tp
            ref.append(tc @ t0)
        ref = np.array(ref)
        scale = np.abs(ref[0])
        assert np.max(np.abs(mu64[k] - ref)) < 1e-11 * scale, np.max(np.abs(mu64[k] - ref))
        # split precision: each moment within 1e-4 of the FP64 one (relative to mu_0)
        assert np.max(np.abs(mus[k] - mu64[k])) < 1e-4 * scale, np.max(np.abs(mus[k] - mu64[k]))
    H.close()


def test_hxv_multi_su2_pivot(gpu_ctx):
    """multi-RHS on an SU(2)xU(1) two-site pivot (CG prefactors in the chain scalars)"""
    from vmps_gb300 import models
    from vmps_gb300.mps import RandomMPS, two_site_layout
    from vmps_gb300.workloads import build_envs
    m = models.hubbard_su2xu1_lattice(8, models.cylinder_bonds(4, 2), U=8.0)
    mps = RandomMPS(m, (1, 8), 48, seed=21).canonicalize(3, 4)
    Lenv, Renv = build_envs(gpu_ctx, m, mps, 3, 4)
    V, _ = two_site_layout(m.sym, m.qloc, m.qloc, mps.dims[3], mps.dims[5], m.sym.nq)
    H = PivotMatrix2(gpu_ctx, m.sym, Lenv, Renv, m.W[3], m.W[4], V)
    X = np.random.default_rng(5).standard_normal((9, H.dim))
    ms = H.apply_multi(X, "bf16x3")
    for k in range(9):
        assert np.array_equal(ms[k], H.apply(X[k], "bf16x3")), k
        assert rel_err(ms[k], H.apply(X[k], "fp64")) < 2e-4
    H.close()
