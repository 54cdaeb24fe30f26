"""Autotuned split-precision tiling: every candidate tiling (tile N caps of 256 /
128 per phase, split-K 1 / 2 / 4 of phase 2) gives the oracle's HxV within the
split tolerance, split-K partials are summed in a fixed order (repeat calls give
the same bits), the tuner's choice is cached per sector layout, and the Lanczos
solve runs on a split-K plan (FP32 Krylov vectors take their own partial buffer)."""
import numpy as np
import pytest

import oracle
from vmps_gb300 import _native as N
from vmps_gb300.pivot import PivotMatrix2

from helpers import pivot2_case, rel_err

pytestmark = pytest.mark.gpu

TOL_SPLIT = 2e-4


def test_every_tiling_matches_oracle(gpu_ctx):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=16, D=128, site=7, seed=22, profile="gaussian")
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(8).standard_normal(V.data.size)
    ref = op.hxv(v)
    default = H.apply(v, "bf16x3")
    for c1 in (256, 128):
        for c2 in (256, 128, 64):
            for sk in (1, 2, 4):
                H.set_tiling(c1, c2, sk)
                got = H.apply(v, "bf16x3")
                assert rel_err(got, ref) < TOL_SPLIT, (c1, c2, sk)
                assert np.array_equal(got, H.apply(v, "bf16x3")), (c1, c2, sk)
                if sk == 1 and c2 == 256:
                    # the N cap of phase 1 only moves tile borders of the intermediates
                    assert rel_err(got, default) < TOL_SPLIT
    H.close()


def test_tuner_choice_is_cached_per_layout(gpu_ctx):
    N.lib().vmps_tune_cache_clear()
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=16, D=128, site=7, seed=22, profile="gaussian")
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    info = H.autotune(trials=3)
    assert info["from_cache"] == 0 and info["candidates"] >= 4
    assert info["ms_best"] <= info["ms_default"]
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(9).standard_normal(V.data.size)
    assert rel_err(H.apply(v, "bf16x3"), op.hxv(v)) < TOL_SPLIT
    # the same layout with other values: the cached choice, no timing
    H2 = PivotMatrix2(gpu_ctx, model.sym, Lenv.like(Lenv.data * 0.5), Renv, W1, W2, V)
    info2 = H2.autotune(trials=3)
    assert info2["from_cache"] == 1 and info2["candidates"] == 0
    assert (info2["ncap1"], info2["ncap2"], info2["splitk"]) == (info["ncap1"], info["ncap2"], info["splitk"])
    H.close()
    H2.close()


def test_lanczos_on_a_split_k_plan(gpu_ctx):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=16, D=128, site=7, seed=22, profile="gaussian")
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    v0 = np.random.default_rng(3).standard_normal(V.data.size)
    tol = dict(max_iter=300, tol_eigval=1e-12, tol_state=1e-7)
    e64, _, _ = H.lanczos(v0, "fp64", **tol)
    H.set_tiling(256, 128, 4)
    es, _, st = H.lanczos(v0, "bf16x3", refine_iters=10, **tol)
    assert st["hxv_split"] > 0
    assert abs(es - e64) <= 1e-10 * abs(e64)
    H.close()
