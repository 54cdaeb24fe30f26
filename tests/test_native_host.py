"""Native library on the CPU: exports, host-side task builder and planner
(host-only context, no device work), error channel."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle
from vmps_gb300 import _native as N
from vmps_gb300.blocks import Blocks
from vmps_gb300.pivot import Context, PivotMatrix0, PivotMatrix1, PivotMatrix2, EnvUpdate

from helpers import make_model, oracle_envs, pivot1_case, pivot2_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "vmps_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vmps_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_symbol(native_lib):
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(native_lib, n), n
    assert set(names) == set(N.EXPORTED), set(names) ^ set(N.EXPORTED)


def test_version(native_lib):
    assert b"sm_103a" in native_lib.vmps_version()


@pytest.fixture(scope="module")
def host_ctx(native_lib):
    c = Context(-1)
    yield c
    c.close()


@pytest.mark.parametrize("kind,L,D,site", [("heis", 8, 16, 3), ("heis", 12, 32, 6), ("hubb", 6, 24, 2)])
def test_pivot1_task_count_matches_oracle(host_ctx, kind, L, D, site):
    model, mps, Lenv, Renv, W, V = pivot1_case(kind, L=L, D=D, site=site, seed=3)
    H = PivotMatrix1(host_ctx, model.sym, Lenv, Renv, W, V)
    st = H.stats("fp64")
    op = oracle.OraclePivot(1, model.sym.nq, Lenv, Renv, V, W)
    assert st["n_tasks"] == op.n_tasks
    assert 0 < st["n_chains"] <= st["n_chains_raw"]
    assert st["flops_merged"] <= st["flops_reference"] * (1 + 1e-12)
    assert st["flops_executed"] > 0


@pytest.mark.parametrize("kind,L,D,site", [("hubb", 6, 24, 2), ("heis", 10, 32, 4)])
def test_pivot2_task_count_matches_oracle(host_ctx, kind, L, D, site):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case(kind, L=L, D=D, site=site, seed=4)
    H = PivotMatrix2(host_ctx, model.sym, Lenv, Renv, W1, W2, V)
    st = H.stats("bf16x3")
    op = oracle.OraclePivot(2, model.sym.nq, Lenv, Renv, V, W1, W2)
    assert st["n_tasks"] == op.n_tasks
    # every output block of the two-site layout gets at least one tile
    assert st["n_tiles_phase2"] >= V.n


def test_env_layout_matches_oracle(host_ctx):
    model, Q = make_model("hubb", 6)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 16, seed=2).canonicalize(3, 3)
    Lenv, Renv = oracle_envs(model, mps, 2, 4)
    for side, E, l in (("L", Lenv, 2), ("R", Renv, 4)):
        e = EnvUpdate(host_ctx, model.sym, side, E, mps.A[l], model.W[l], mps.A[l])
        ref = oracle.OracleEnv(side, 2, E, mps.A[l], model.W[l], mps.A[l]).layout
        got = {e.out_layout.key(i): (e.out_layout.rows[i], e.out_layout.cols[i]) for i in range(e.out_layout.n)}
        exp = {ref.key(i): (ref.rows[i], ref.cols[i]) for i in range(ref.n)}
        assert got == exp
        st = e.stats("fp64")
        assert st["n_chains"] > 0


def test_pivot0_plan(host_ctx):
    model, Q = make_model("heis", 8)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 8, seed=7).canonicalize(4, 3)
    Lenv, Renv = oracle_envs(model, mps, 4, 3)
    ent = [(0, q, q, np.zeros((d, d))) for q, d in sorted(mps.dims[4].items())]
    Cb = Blocks.from_entries(1, ent)
    H = PivotMatrix0(host_ctx, model.sym, Lenv, Renv, Cb)
    assert H.stats()["n_chains"] > 0


def test_device_call_on_host_context_is_an_error(host_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=6, D=8, site=2, seed=1)
    H = PivotMatrix1(host_ctx, model.sym, Lenv, Renv, W, V)
    with pytest.raises(N.VmpsError) as ei:
        H.apply(np.zeros(H.dim))
    assert ei.value.code == -1 and "host-only" in str(ei.value)


def test_shape_mismatch_is_reported(host_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=6, D=8, site=2, seed=1)
    # corrupt one L block shape: its chains no longer fit the vector blocks
    bad = Lenv.like(Lenv.data.copy())
    i = int(np.argmax(bad.rows))
    bad.rows = bad.rows.copy()
    bad.rows[i] += 1
    bad.data = np.zeros(int((bad.offset + bad.rows * bad.cols).max()) + 16)
    H = PivotMatrix1(host_ctx, model.sym, bad, Renv, W, V)
    with pytest.raises(N.VmpsError) as ei:
        H.stats()
    assert ei.value.code == -4


def test_invalid_tables_are_rejected(host_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=6, D=8, site=2, seed=1)
    bad = V.like()
    bad.rows = bad.rows.copy()
    bad.rows[0] = 0
    with pytest.raises(N.VmpsError) as ei:
        PivotMatrix1(host_ctx, model.sym, Lenv, Renv, W, bad)
    assert ei.value.code == -1
    # null context / symmetry
    h = C.c_void_p()
    rc = N.lib().vmps_pivot1_create(None, None, None, None, None, None, None, None, C.byref(h))
    assert rc == -1
    assert N.lib().vmps_last_error()


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("mode,ab", [("FIXED_ROWS", 0), ("FIXED_ROWS", 2), ("FIXED_COLS", 1), ("FIXED_COLS", 5),
                                     ("TRIANGULAR", 1), ("TRIANGULAR", 4)])
def test_env_mode_layout_matches_oracle(host_ctx, side, mode, ab):
    model, Q = make_model("hubb", 8)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 24, seed=13).canonicalize(4, 4)
    Lenv, Renv = oracle_envs(model, mps, 3, 5)
    l = 3 if side == "L" else 5
    E = Lenv if side == "L" else Renv
    order = dict(model.basis_order_map(l))
    order.update(model.basis_order_map(l + 1))
    e = EnvUpdate(host_ctx, model.sym, side, E, mps.A[l], model.W[l], mps.A[l], mode=mode, fixed_ab=ab, order=order)
    ref = oracle.OracleEnv(side, 2, E, mps.A[l], model.W[l], mps.A[l], mode=mode, fixed_ab=ab, order=order).layout
    got = {e.out_layout.key(i): (e.out_layout.rows[i], e.out_layout.cols[i]) for i in range(e.out_layout.n)}
    exp = {ref.key(i): (ref.rows[i], ref.cols[i]) for i in range(ref.n)}
    assert got == exp


def test_env_mode_without_order_map_is_rejected(host_ctx):
    model, Q = make_model("heis", 6)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 8, seed=1).canonicalize(3, 3)
    Lenv, _ = oracle_envs(model, mps, 2, 4)
    with pytest.raises(N.VmpsError) as ei:
        EnvUpdate(host_ctx, model.sym, "L", Lenv, mps.A[2], model.W[2], mps.A[2], mode="FIXED_COLS", fixed_ab=0)
    assert ei.value.code == -1
