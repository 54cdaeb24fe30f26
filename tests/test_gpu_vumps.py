"""VUMPS MpoTransferMatrix on the GPU engine (VUMPS/VumpsMpoTransferMatrix.h:99-212)
against the oracle's restatement (oracle/vumps_cpu.py), and the GMRES environment
solve (VUMPS/VumpsSolver.h:1907-1940) on it."""
import numpy as np
import pytest

from oracle.vumps_cpu import transfer_hxv
from vmps_gb300.vumps import MpoTransferMatrix

from helpers import oracle_envs, rel_err
from vumps_case import transfer_case

pytestmark = pytest.mark.gpu


def _envs(m, mps):
    return oracle_envs(m, mps, 9, 10)


def _positions(order, sym):
    vac = sym.vacuum()
    return sorted(v for (q, i), v in order.items() if tuple(q) == vac)


@pytest.mark.parametrize("direction", ["L", "R"])
def test_transfer_hxv_matches_oracle(gpu_ctx, direction):
    m, mps, (A, W), LR, order, V = transfer_case("heis", direction, envs=_envs)
    rng = np.random.default_rng(11)
    nonzero = 0
    for ab in _positions(order, m.sym):
        T = MpoTransferMatrix(gpu_ctx, m.sym, direction, A, A, W, LR, ab, order, V)
        for _ in range(2):
            v = rng.standard_normal(V.data.size)
            ref = transfer_hxv(direction, m.sym.nq, A, A, W, LR, ab, order, V, v, m.sym.dot_weight)
            if np.linalg.norm(ref) == 0:
                # no cell path returns to slot ab (e.g. an open channel of a two-site term): the
                # reference writes no block, and neither does the engine
                assert not np.any(T.hxv(v, "fp64")) and not np.any(T.hxv(v, "bf16x3"))
                continue
            nonzero += 1
            assert rel_err(T.hxv(v, "fp64"), ref) < 1e-12
            assert rel_err(T.hxv(v, "bf16x3"), ref) < 2e-4
        T.close()
    assert nonzero >= 4   # the IDLE and DONE positions return to themselves


@pytest.mark.parametrize("direction", ["L", "R"])
def test_transfer_solve_linear(gpu_ctx, direction):
    m, mps, (A, W), LR, order, V = transfer_case("heis", direction, envs=_envs)
    ab = _positions(order, m.sym)[0]
    T = MpoTransferMatrix(gpu_ctx, m.sym, direction, A, A, W, LR, ab, order, V)
    b = T.rhs(np.random.default_rng(3).standard_normal(V.data.size), 0.3) * T.slot_mask()
    x, info = T.solve_linear(b, tol=1e-11, dimK=80)
    r = (b - T.hxv(x)) * T.slot_mask()
    assert np.sqrt(T.dot(r, r) / T.dot(b, b)) < 1e-8, info
    T.close()


def test_transfer_su2_linear_and_split_consistent(gpu_ctx):
    """SU(2) cell (the abelian oracle cannot restate it): the operator is linear and
    the split-precision result agrees with FP64"""
    from vmps_gb300.pivot import contract_L, left_vacuum
    m, mps, (A, W), LR, order, _ = transfer_case("su2", "L")
    E = left_vacuum(m.sym)
    for l in range(9):
        E = contract_L(gpu_ctx, m.sym, E, mps.A[l], m.W[l], mps.A[l])
    ab = _positions(order, m.sym)[-1]
    T = MpoTransferMatrix(gpu_ctx, m.sym, "L", A, A, W, LR, ab, order, E)
    rng = np.random.default_rng(5)
    u, v = rng.standard_normal(E.data.size), rng.standard_normal(E.data.size)
    hu, hv, huv = T.hxv(u), T.hxv(v), T.hxv(2.0 * u - 0.5 * v)
    assert np.linalg.norm(hu) > 0
    assert rel_err(huv, 2.0 * hu - 0.5 * hv) < 1e-12
    assert rel_err(T.hxv(u, "bf16x3"), hu) < 2e-4
    T.close()


@pytest.mark.parametrize("direction", ["L", "R"])
@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_transfer_solve_on_the_device(gpu_ctx, direction, precision):
    """vmps_transfer_solve (Krylov vectors on the device, two classical Gram-Schmidt passes,
    Givens rotations on the host; BF16X3: FP64-residual refinement of split corrections)
    reaches the residual the host GMRES reaches on this operator (its attainable floor is
    ~1e-9: the random cell makes 1 - T + |R)(1| ill conditioned) and the same solution"""
    m, mps, (A, W), LR, order, V = transfer_case("heis", direction, envs=_envs)
    ab = _positions(order, m.sym)[0]
    T = MpoTransferMatrix(gpu_ctx, m.sym, direction, A, A, W, LR, ab, order, V)
    b = T.rhs(np.random.default_rng(3).standard_normal(V.data.size), 0.3) * T.slot_mask()
    x_ref, ref = T.solve_linear(b, tol=1e-11, dimK=80)
    x, info = T.solve_device(b, tol=1e-11, dimK=80, precision=precision)
    r = (b - T.hxv(x)) * T.slot_mask()
    res = np.sqrt(T.dot(r, r) / T.dot(b, b))
    assert res < max(1e-8, 3 * ref["residual"]), (info, ref)
    assert info["residual"] == pytest.approx(res, rel=1e-3, abs=1e-13)
    assert info["iterations"] > 0
    if precision == "bf16x3":
        # on this ill-conditioned operator the split corrections stop paying and FP64 finishes
        assert info["outer"] >= 1 and info["fp64_hxv"] >= 2
        assert info["iterations"] >= info["fp64_iterations"] > 0
    d = x - x_ref
    assert np.sqrt(T.dot(d, d) / T.dot(x_ref, x_ref)) < 1e-6
    # a zero right-hand side gives x = 0 and no iteration
    z, zi = T.solve_device(np.zeros_like(b), precision=precision)
    assert not np.any(z) and zi["iterations"] == 0
    T.close()


def test_transfer_solve_on_the_device_su2(gpu_ctx):
    from vmps_gb300.pivot import contract_L, left_vacuum
    m, mps, (A, W), LR, order, _ = transfer_case("su2", "L")
    E = left_vacuum(m.sym)
    for l in range(9):
        E = contract_L(gpu_ctx, m.sym, E, mps.A[l], m.W[l], mps.A[l])
    ab = _positions(order, m.sym)[-1]
    T = MpoTransferMatrix(gpu_ctx, m.sym, "L", A, A, W, LR, ab, order, E)
    b = T.rhs(np.random.default_rng(8).standard_normal(E.data.size), 0.1) * T.slot_mask()
    x_ref, ref = T.solve_linear(b, tol=1e-11, dimK=80)
    for precision in ("fp64", "bf16x3"):
        x, info = T.solve_device(b, tol=1e-11, dimK=80, precision=precision)
        d = x - x_ref
        assert np.sqrt(T.dot(d, d) / T.dot(x_ref, x_ref)) < 1e-6, (precision, info, ref)
        assert info["residual"] < max(1e-8, 3 * ref["residual"])
    T.close()
