"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the
same seeded inputs.

Tolerances (relative, Frobenius norm of the whole output vector / Tripod):
  FP64 (DMMA)        : 1e-12   (the spec bar for the plain drop-in form)
  BF16x3 split       : 2e-4    (two bf16 slices per operand ~ 2^-16 per product,
                                FP32 accumulation; the chain has two products)
Energies after FP64 refinement: 1e-10 relative.
"""
import numpy as np
import pytest

import oracle
from vmps_gb300 import _native as N
from vmps_gb300.blocks import Blocks
from vmps_gb300.pivot import (DeviceVector, EnvUpdate, PivotMatrix0, PivotMatrix1, PivotMatrix2, hxv_device,
                              time_hxv)

from helpers import compare_tripods, make_model, oracle_envs, pivot1_case, pivot2_case, rel_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_SPLIT = 2e-4


@pytest.mark.parametrize("kind,L,D,site", [("heis", 8, 16, 3), ("heis", 32, 64, 15), ("hubb", 8, 32, 3),
                                           ("heis", 10, 8, 0), ("heis", 10, 8, 9)])
def test_hxv1_parity(gpu_ctx, kind, L, D, site):
    model, mps, Lenv, Renv, W, V = pivot1_case(kind, L=L, D=D, site=site, seed=21)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    op = oracle.OraclePivot(1, model.sym.nq, Lenv, Renv, V, W)
    rng = np.random.default_rng(7)
    for _ in range(2):
        v = rng.standard_normal(V.data.size)
        ref = op.hxv(v)
        assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
        assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT


@pytest.mark.parametrize("kind,L,D,site,profile", [("hubb", 6, 24, 2, "even"), ("hubb", 16, 128, 7, "gaussian"),
                                                   ("heis", 16, 64, 7, "even")])
def test_hxv2_parity(gpu_ctx, kind, L, D, site, profile):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case(kind, L=L, D=D, site=site, seed=22, profile=profile)
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    op = oracle.OraclePivot(2, model.sym.nq, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(8).standard_normal(V.data.size)
    ref = op.hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT


def test_hxv0_parity(gpu_ctx):
    model, Q = make_model("hubb", 8)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 32, seed=5).canonicalize(4, 3)
    Lenv, Renv = oracle_envs(model, mps, 4, 3)
    ent = [(0, q, q, np.zeros((d, d))) for q, d in sorted(mps.dims[4].items())]
    Cb = Blocks.from_entries(2, ent)
    H = PivotMatrix0(gpu_ctx, model.sym, Lenv, Renv, Cb)
    op = oracle.OraclePivot(0, 2, Lenv, Renv, Cb)
    v = np.random.default_rng(9).standard_normal(Cb.data.size)
    ref = op.hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT


@pytest.mark.parametrize("kind,L,D", [("heis", 12, 32), ("hubb", 10, 48)])
def test_env_parity(gpu_ctx, kind, L, D):
    model, Q = make_model(kind, L)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, D, seed=6, profile="gaussian").canonicalize(L // 2, L // 2)
    Lenv, Renv = oracle_envs(model, mps, L // 2 - 1, L // 2 + 1)
    nq = model.sym.nq
    for side, E, l in (("L", Lenv, L // 2 - 1), ("R", Renv, L // 2 + 1)):
        ref = oracle.OracleEnv(side, nq, E, mps.A[l], model.W[l], mps.A[l]).run(E, mps.A[l], mps.A[l])
        e = EnvUpdate(gpu_ctx, model.sym, side, E, mps.A[l], model.W[l], mps.A[l])
        got = e.run(E, mps.A[l], mps.A[l], "fp64")
        assert compare_tripods(got, ref) < TOL_FP64
        got32 = e.run(E, mps.A[l], mps.A[l], "bf16x3")
        assert compare_tripods(got32, ref) < TOL_SPLIT


def test_env_chain_matches_oracle_chain(gpu_ctx):
    """A whole left sweep of contract_L on the GPU equals the oracle's."""
    from vmps_gb300.pivot import contract_L, left_vacuum
    model, Q = make_model("heis", 16)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 32, seed=3).canonicalize(8, 8)
    E = left_vacuum(model.sym)
    Eo = E
    for l in range(8):
        E = contract_L(gpu_ctx, model.sym, E, mps.A[l], model.W[l], mps.A[l])
        Eo = oracle.contract_L(1, Eo, mps.A[l], model.W[l], mps.A[l])
    assert compare_tripods(E, Eo) < TOL_FP64


def test_device_vectors_and_dot(gpu_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=12, D=32, site=5, seed=2)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    rng = np.random.default_rng(1)
    a, b = rng.standard_normal(H.dim), rng.standard_normal(H.dim)
    da, db = DeviceVector(H, a), DeviceVector(H, b)
    assert abs(da.dot(db) - a @ b) < 1e-12 * np.linalg.norm(a) * np.linalg.norm(b)
    assert np.array_equal(da.download(), a)
    hxv_device(H, da, db, "fp64")
    ref = oracle.OraclePivot(1, 1, Lenv, Renv, V, W).hxv(a)
    assert rel_err(db.download(), ref) < TOL_FP64
    ms, ms2 = time_hxv(H, da, db, "fp64", n_iter=3, use_graph=True)
    assert ms > 0 and ms2 > 0
    assert rel_err(db.download(), ref) < TOL_FP64


def test_host_hxv_after_device_vector_upload(gpu_ctx):
    # regression: a device-vector upload must not leave the host-buffer HxV path
    # with unallocated I/O vectors
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=10, D=16, site=4, seed=2)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    v = np.random.default_rng(4).standard_normal(H.dim)
    dv = DeviceVector(H, v)
    ref = oracle.OraclePivot(1, 1, Lenv, Renv, V, W).hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert np.array_equal(dv.download(), v)
    dv.close()


def test_host_buffer_kinds_give_identical_hxv(gpu_ctx):
    """vmps_hxv reads and writes page-locked buffers through their device mapping
    and pageable ones in place or through a staging copy: every route gives the
    same bits as the device-vector path (pieces of large blocks included)."""
    import ctypes as C

    import torch
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=24, D=1024, site=11, seed=12, profile="gaussian")
    assert max(V.rows * V.cols) > 8192   # blocks larger than one copy piece
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    n = H.dim
    v = np.random.default_rng(9).standard_normal(n)
    ref = oracle.OraclePivot(1, 1, Lenv, Renv, V, W).hxv(v)
    lib = N.lib()
    for prec, code in (("fp64", 0), ("bf16x3", 1)):
        pageable = H.apply(v, prec)
        hin = torch.empty(n, dtype=torch.float64, pin_memory=True)
        hout = torch.zeros(n, dtype=torch.float64, pin_memory=True)
        hin.copy_(torch.from_numpy(v))
        N.check(lib.vmps_hxv(H._h, C.cast(C.c_void_p(hin.data_ptr()), N.f64p),
                             C.cast(C.c_void_p(hout.data_ptr()), N.f64p), code))
        pinned = hout.numpy().copy()
        dv_in, dv_out = DeviceVector(H, v), DeviceVector(H)
        hxv_device(H, dv_in, dv_out, prec)
        dev = dv_out.download()
        dv_in.close()
        dv_out.close()
        assert np.array_equal(pageable, pinned), prec
        assert np.array_equal(pageable, dev), prec
        assert rel_err(pageable, ref) < (TOL_FP64 if prec == "fp64" else TOL_SPLIT)


def test_pipelined_host_hxv_matches_device_path(gpu_ctx):
    """A vector of several 4 MiB chunks goes through the copy/compute pipeline of
    vmps_hxv (phases cut per chunk, transfers on a second stream); every tile is
    computed the same way as in the one-launch device path, so the bits agree."""
    import ctypes as C

    import torch
    from vmps_gb300.workloads import hubbard_two_site
    model, mps, Lenv, Renv, W1, W2, V, info = hubbard_two_site(gpu_ctx, L=32, D=2048, seed=3)
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    n = H.dim
    assert n * 8 >= 2 * (4 << 20)
    v = np.random.default_rng(10).standard_normal(n)
    lib = N.lib()
    dv_in, dv_out = DeviceVector(H, v), DeviceVector(H)
    for prec, code in (("bf16x3", 1), ("fp64", 0)):
        hxv_device(H, dv_in, dv_out, prec)
        dev = dv_out.download()
        pageable = H.apply(v, prec)
        hin = torch.empty(n, dtype=torch.float64, pin_memory=True)
        hout = torch.zeros(n, dtype=torch.float64, pin_memory=True)
        hin.copy_(torch.from_numpy(v))
        N.check(lib.vmps_hxv(H._h, C.cast(C.c_void_p(hin.data_ptr()), N.f64p),
                             C.cast(C.c_void_p(hout.data_ptr()), N.f64p), code))
        assert np.array_equal(pageable, dev), prec
        assert np.array_equal(hout.numpy(), dev), prec
    assert rel_err(H.apply(v, "bf16x3"), H.apply(v, "fp64")) < TOL_SPLIT
    dv_in.close()
    dv_out.close()


def test_nonfinite_input_is_rejected(gpu_ctx):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=8, D=8, site=3, seed=2)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    v = np.zeros(H.dim)
    v[3] = np.nan
    with pytest.raises(N.VmpsError) as ei:
        DeviceVector(H, v)
    assert ei.value.code == -6


def _oracle_ground(op, n):
    Heff = np.column_stack([op.hxv(np.eye(n)[:, j]) for j in range(n)])
    return np.linalg.eigvalsh(0.5 * (Heff + Heff.T))[0]


@pytest.mark.parametrize("case", ["heis1", "hubb2"])
def test_lanczos_energy(gpu_ctx, case, monkeypatch):
    if case == "heis1":
        model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=16, D=16, site=7, seed=31)
        H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
        op = oracle.OraclePivot(1, 1, Lenv, Renv, V, W)
    else:
        model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=8, D=16, site=3, seed=32)
        H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
        op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    n = H.dim
    assert n <= 3000
    e_ref = _oracle_ground(op, n)
    v0 = np.random.default_rng(3).standard_normal(n)
    e64, v64, st64 = H.lanczos(v0, "fp64", max_iter=300, tol_eigval=1e-13, tol_state=1e-9)
    assert abs(e64 - e_ref) < 1e-10 * abs(e_ref), (e64, e_ref, st64)
    es, vs, sts = H.lanczos(v0, "bf16x3", max_iter=300, tol_eigval=1e-9, tol_state=1e-5, refine_iters=30)
    assert abs(es - e_ref) < 1e-10 * abs(e_ref), (es, e_ref, sts)
    # the probe and the FP64 residual of the split Ritz vector at least
    assert sts["hxv_split"] > 0 and sts["hxv_fp64"] >= 2
    # a state tolerance below the split operator's noise takes refinement, by
    # rounds (split runs from the FP64 residual, one FP64 HxV each) or by the
    # Krylov-space correction and closing FP64 steps; both reach the FP64 energy
    # and report the residual of the vector they return
    for mode in ("rounds", "polish"):
        monkeypatch.setenv("VMPS_LANCZOS_REFINE", mode)
        et, vt, stt = H.lanczos(v0, "bf16x3", max_iter=300, tol_eigval=1e-12, tol_state=1e-9, refine_iters=8)
        assert abs(et - e_ref) < 1e-10 * abs(e_ref), (mode, et, e_ref, stt)
        assert stt["refine_iterations"] >= 1 and stt["hxv_fp64"] <= 1 + 8, (mode, stt)
        xt = vt / np.linalg.norm(vt)
        true_res = np.linalg.norm(H.apply(xt, "fp64") - et * xt)
        assert abs(true_res - stt["residual"]) <= 1e-11 + 0.05 * true_res, (mode, true_res, stt)
        if mode == "rounds":
            assert stt["residual"] <= 1e-9, stt
    monkeypatch.setenv("VMPS_LANCZOS_REFINE", "sometimes")
    with pytest.raises(N.VmpsError):
        H.lanczos(v0, "bf16x3", max_iter=300, tol_eigval=1e-12, tol_state=1e-9, refine_iters=8)


def test_lanczos_residual_estimate_and_determinism(gpu_ctx):
    """The device Lanczos reports |beta_m y_m| as the residual: it equals the
    explicit FP64 residual ||H v - E v|| of the returned vector.  Its
    reductions are deterministic, so two runs agree bit for bit.  The split
    run with its refinement rounds reaches the FP64 energy within 1e-10
    relative using at most refine_iters FP64 HxVs after the probe, and reports
    the FP64 residual of the returned vector.
    From a start vector that is already an eigenvector the split run is the
    FP64 run."""
    model, mps, Lenv, Renv, W, V = pivot1_case("hubb", L=10, D=32, site=4, seed=41)
    H = PivotMatrix1(gpu_ctx, model.sym, Lenv, Renv, W, V)
    v0 = np.random.default_rng(7).standard_normal(H.dim)
    e1, x1, st1 = H.lanczos(v0, "fp64", max_iter=200, tol_eigval=1e-12, tol_state=1e-8)
    e2, x2, st2 = H.lanczos(v0, "fp64", max_iter=200, tol_eigval=1e-12, tol_state=1e-8)
    assert e1 == e2 and np.array_equal(x1, x2) and st1["iterations"] == st2["iterations"]
    assert abs(np.linalg.norm(x1) - 1) < 1e-12
    true_res = np.linalg.norm(H.apply(x1, "fp64") - e1 * x1)
    assert abs(true_res - st1["residual"]) <= 1e-11 + 0.05 * true_res, (true_res, st1)
    es, xs, sts = H.lanczos(v0, "bf16x3", max_iter=200, tol_eigval=1e-10, tol_state=1e-6, refine_iters=12)
    assert abs(es - e1) < 1e-10 * abs(e1), (es, e1, sts)
    assert sts["hxv_split"] > 0 and 2 <= sts["hxv_fp64"] <= 1 + 12
    true_res = np.linalg.norm(H.apply(xs, "fp64") - es * xs)
    assert abs(true_res - sts["residual"]) <= 1e-11 + 0.05 * true_res, (true_res, sts)
    # near-converged start: the FP64 probe continues as the FP64 solve
    ec, xc, stc = H.lanczos(x1, "bf16x3", max_iter=200, tol_eigval=1e-12, tol_state=1e-8, refine_iters=12)
    assert stc["hxv_split"] == 0 and abs(ec - e1) < 1e-12 * abs(e1), stc
    H.close()


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("mode,ab", [("FIXED_ROWS", 0), ("FIXED_COLS", 5), ("TRIANGULAR", 1)])
def test_env_mode_parity(gpu_ctx, side, mode, ab):
    model, Q = make_model("hubb", 8)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 24, seed=13).canonicalize(4, 4)
    Lenv, Renv = oracle_envs(model, mps, 3, 5)
    l = 3 if side == "L" else 5
    E = Lenv if side == "L" else Renv
    order = dict(model.basis_order_map(l))
    order.update(model.basis_order_map(l + 1))
    A = mps.A[l]
    ref = oracle.OracleEnv(side, 2, E, A, model.W[l], A, mode=mode, fixed_ab=ab, order=order).run(E, A, A)
    e = EnvUpdate(gpu_ctx, model.sym, side, E, A, model.W[l], A, mode=mode, fixed_ab=ab, order=order)
    assert compare_tripods(e.run(E, A, A, "fp64"), ref) < TOL_FP64
    assert compare_tripods(e.run(E, A, A, "bf16x3"), ref) < TOL_SPLIT


def test_hxv2_parity_hubbard_L64_D1024_middle(gpu_ctx):
    """The C2 configuration's D=1024 stage: the two-site pivot in the middle of the
    L=64 Hubbard chain (U/t=4, half filling, Sz=0, seeded Gaussian-profile MPS, the
    bench's inputs at D=1024) with environments from the oracle.  One FP64 and one
    split HxV against the oracle's HxV, then the ground-state energy of the pivot
    from the engine's Lanczos (FP64, and split precision + FP64 refinement) against
    the oracle's own FP64 Lanczos energy.  Blocks here reach 140-190 rows (two
    M=128 MMA tiles) and the K-class panels of the large sectors appear."""
    from vmps_gb300.mps import RandomMPS, contract_two_sites
    model, Q = make_model("hubb", 64)
    site = 31
    mps = RandomMPS(model, Q, 1024, seed=2, profile="gaussian", sigma=[2.5, 2.5]).canonicalize(site, site + 1)
    Lenv, Renv = oracle_envs(model, mps, site, site + 1)
    V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, model.sym.nq)
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, model.W[site], model.W[site + 1], V)
    op = oracle.OraclePivot(2, model.sym.nq, Lenv, Renv, V, model.W[site], model.W[site + 1])
    v = np.random.default_rng(8).standard_normal(V.data.size)
    ref = op.hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT
    e_or, _ = oracle.lanczos_ground(op.hxv, v, tol=1e-14)
    tol = dict(max_iter=300, tol_eigval=1e-12, tol_state=1e-7)
    e64, x64, _ = H.lanczos(v, "fp64", **tol)
    es, xs, st = H.lanczos(v, "bf16x3", refine_iters=10, **tol)
    assert st["hxv_split"] > 0
    assert abs(e64 - e_or) <= 1e-10 * abs(e_or), (e64, e_or)
    assert abs(es - e_or) <= 1e-10 * abs(e_or), (es, e_or)
    # the split solve's vector, checked with the oracle's operator: Rayleigh quotient and residual
    xs = xs / np.linalg.norm(xs)
    hx = op.hxv(xs)
    rq = float(xs @ hx)
    assert abs(rq - e_or) <= 1e-10 * abs(e_or), (rq, e_or)
    assert np.linalg.norm(hx - rq * xs) <= 1e-6 * abs(e_or)
    H.close()
