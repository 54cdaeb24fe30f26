"""Union pivots: start vectors of different quantum-number sectors advanced
together (config C5: c_k|0> for both spin projections in one grouped launch).

* On each part the union's HxV equals that part's own pivot (FP64 to 1e-12 and
  against the oracle; split precision to its own error level), also for many
  right-hand sides in one grouped launch;
* per-part Chebyshev moments of union vectors equal the moments each part's own
  pivot gives (FP64), and the split-precision moments stay within 1e-4 of them."""
import numpy as np
import pytest

import oracle
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import PivotMatrix2
from vmps_gb300.union import UnionPivot2

from helpers import oracle_envs, rel_err

pytestmark = pytest.mark.gpu


def _parts(L=8, D=24, site=3):
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    parts = []
    for Q, seed in (((L - 1, -1), 61), ((L - 1, 1), 62)):
        mps = RandomMPS(model, Q, D, seed=seed).canonicalize(site, site + 1)
        Lenv, Renv = oracle_envs(model, mps, site, site + 1)
        V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, model.sym.nq)
        parts.append((Lenv, Renv, V))
    return model, site, parts


def test_union_hxv_equals_each_part(gpu_ctx):
    model, site, parts = _parts()
    W1, W2 = model.W[site], model.W[site + 1]
    U = UnionPivot2(gpu_ctx, model.sym, W1, W2, parts)
    rng = np.random.default_rng(7)
    x = rng.standard_normal(U.H.dim)
    y64, ysp = U.split(U.H.apply(x, "fp64")), U.split(U.H.apply(x, "bf16x3"))
    X = rng.standard_normal((5, U.H.dim))
    M = [U.split(m) for m in U.H.apply_multi(X, "bf16x3")]
    for p, (Lp, Rp, Vp) in enumerate(parts):
        H = PivotMatrix2(gpu_ctx, model.sym, Lp, Rp, W1, W2, Vp)
        xp = U.split(x)[p]
        ref = oracle.OraclePivot(2, 2, Lp, Rp, Vp, W1, W2).hxv(xp)
        assert rel_err(y64[p], ref) < 1e-12
        assert rel_err(y64[p], H.apply(xp, "fp64")) < 1e-12
        assert rel_err(ysp[p], H.apply(xp, "bf16x3")) < 1e-6
        assert rel_err(ysp[p], ref) < 2e-4
        for k in range(5):
            assert np.array_equal(M[k][p], U.split(U.H.apply(X[k], "bf16x3"))[p])
        H.close()
    U.close()


def test_union_chebyshev_moments_per_part(gpu_ctx):
    model, site, parts = _parts()
    W1, W2 = model.W[site], model.W[site + 1]
    U = UnionPivot2(gpu_ctx, model.sym, W1, W2, parts)
    rng = np.random.default_rng(8)
    nrhs, nmom = 3, 64
    X = rng.standard_normal((nrhs, U.H.dim))
    for p in range(2):   # every part of every vector normalised
        s = slice(U.offsets[p], U.offsets[p + 1])
        X[:, s] /= np.linalg.norm(X[:, s], axis=1, keepdims=True)
    lo, hi = U.H.spectral_bounds(X.sum(axis=0), iters=80)
    a, b = (hi - lo) / 2 / 0.98, (hi + lo) / 2
    mu64, _ = U.chebyshev_moments(X, nmom, a, b, "fp64")
    musp, st = U.chebyshev_moments(X, nmom, a, b, "bf16x3")
    assert mu64.shape == (nrhs, 2, nmom) and st["hxv"] == nrhs * (nmom // 2)
    for p, (Lp, Rp, Vp) in enumerate(parts):
        H = PivotMatrix2(gpu_ctx, model.sym, Lp, Rp, W1, W2, Vp)
        ref, _ = H.chebyshev_moments(U.split(X)[p], nmom, a, b, "fp64")
        assert np.abs(mu64[:, p, :] - ref).max() < 1e-10
        assert np.abs(musp[:, p, :] - ref).max() < 1e-4
        assert np.all(np.abs(ref) <= 1 + 1e-9)   # |T_n| <= 1 on the rescaled spectrum
        H.close()
    # one part alone through the parts entry point equals the plain moments
    one, _ = U.H.chebyshev_moments(X, nmom, a, b, "fp64", parts=[0, U.parts[-1]])
    plain, _ = U.H.chebyshev_moments(X, nmom, a, b, "fp64")
    assert np.array_equal(one[:, 0, :], plain)
    U.close()
