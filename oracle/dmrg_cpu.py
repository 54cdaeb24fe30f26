"""ORACLE -- test infrastructure, not product code.

Single-site DMRG sweeps on the CPU oracle: same sweep order, gauge steps and
Lanczos stopping rule as vmps_gb300.dmrg.dmrg1, with the oracle's HxV and
contract_L/R (literal restatements of the reference loops) and a numpy
full-reorthogonalisation Lanczos.  Used as the CPU baseline of the sweep time
and as a checker of the GPU sweep.
"""
from __future__ import annotations

import time

import numpy as np

from . import OracleEnv, OraclePivot


def lanczos_np(hxv, v0, max_iter=100, tol_eigval=1e-12, tol_state=1e-8):
    n = v0.size
    V = np.zeros((min(max_iter, n) + 1, n))
    V[0] = v0 / np.linalg.norm(v0)
    a, b = [], []
    theta_prev = np.inf
    y = np.array([1.0])
    theta = 0.0
    k = 0
    for j in range(min(max_iter, n)):
        w = hxv(V[j])
        for _ in range(2):
            c = V[: j + 1] @ w
            w -= c @ V[: j + 1]
            if _ == 0:
                aj = c[j]
            else:
                aj += c[j]
        a.append(aj)
        bj = np.linalg.norm(w)
        T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
        ev, evec = np.linalg.eigh(T)
        theta, y = ev[0], evec[:, 0]
        k = j + 1
        conv = abs(theta - theta_prev) <= tol_eigval * max(1.0, abs(theta)) and abs(bj * y[-1]) <= tol_state
        theta_prev = theta
        if conv or bj <= 1e-14 * max(1.0, abs(theta)) or j + 1 == min(max_iter, n):
            break
        b.append(bj)
        V[j + 1] = w / bj
    x = y @ V[:k]
    return theta, x / np.linalg.norm(x), k


def dmrg1_cpu(model, mps, n_sweeps=2, max_iter=100, tol_eigval=1e-12, tol_state=1e-8):
    from vmps_gb300.dmrg import _push_left, _push_right
    from vmps_gb300.mps import left_normalize, right_normalize
    from vmps_gb300.pivot import left_vacuum, right_target
    sym, L, nq = model.sym, model.L, model.sym.nq
    envL = [None] * (L + 1)
    envR = [None] * (L + 1)
    envL[0] = left_vacuum(sym)
    envR[L] = right_target(sym, mps.Qtot)
    for l in range(L - 1, 0, -1):
        envR[l] = OracleEnv("R", nq, envR[l + 1], mps.A[l], model.W[l], mps.A[l]).run(envR[l + 1], mps.A[l], mps.A[l])
    energies, times = [], []
    for sweep in range(n_sweeps):
        ts = time.perf_counter()
        order = list(range(L)) + list(range(L - 1, -1, -1))
        for step, l in enumerate(order):
            right = step < L
            op = OraclePivot(1, nq, envL[l], envR[l + 1], mps.A[l], model.W[l])
            E, v, _ = lanczos_np(op.hxv, mps.A[l].data.copy(), max_iter, tol_eigval, tol_state)
            mps.A[l].data[:] = v
            if right and l < L - 1:
                mps.A[l], Rf = left_normalize(mps.A[l], nq)
                _push_right(mps.A[l + 1], Rf)
                envL[l + 1] = OracleEnv("L", nq, envL[l], mps.A[l], model.W[l], mps.A[l]).run(envL[l], mps.A[l], mps.A[l])
            elif not right and l > 0:
                mps.A[l], Lf = right_normalize(mps.A[l], nq)
                _push_left(mps.A[l - 1], Lf)
                envR[l] = OracleEnv("R", nq, envR[l + 1], mps.A[l], model.W[l], mps.A[l]).run(envR[l + 1], mps.A[l],
                                                                                                 mps.A[l])
        times.append(time.perf_counter() - ts)
        energies.append(E)
    return {"energies": energies, "sweep_times": times}


def dmrg2_cpu(model, mps, n_sweeps=2, Dmax=None, max_iter=100, tol_eigval=1e-12, tol_state=1e-8, eps_svd=1e-14):
    """Two-site DMRG on the oracle: the sweep of vmps_gb300.dmrg.dmrg2 (bond order, split_AA2
    truncation, environment updates) with the oracle's two-site HxV and contract_L/R."""
    from vmps_gb300.mps import contract_two_sites, split_two_site
    from vmps_gb300.pivot import left_vacuum, right_target
    sym, L, nq = model.sym, model.L, model.sym.nq
    Dmax = Dmax if Dmax is not None else max(mps.bond_dim(l) for l in range(L + 1))
    qloc = model.qloc

    def env(side, E, A, W):
        return OracleEnv(side, nq, E, A, W, A).run(E, A, A)

    envL = [None] * (L + 1)
    envR = [None] * (L + 1)
    envL[0] = left_vacuum(sym)
    envR[L] = right_target(sym, mps.Qtot)
    for l in range(L - 1, 1, -1):
        envR[l] = env("R", envR[l + 1], mps.A[l], model.W[l])
    energies, times = [], []
    E = None
    for sweep in range(n_sweeps):
        ts = time.perf_counter()
        for move, bonds in (("right", range(L - 1)), ("left", range(L - 2, -1, -1))):
            for l in bonds:
                A1, A2 = mps.A[l], mps.A[l + 1]
                din = {tuple(A1.qin[i]): int(A1.rows[i]) for i in range(A1.n)}
                dout = {tuple(A2.qout[i]): int(A2.cols[i]) for i in range(A2.n)}
                V, comb = contract_two_sites(sym, A1, A2, qloc, qloc, nq, return_basis=True)
                op = OraclePivot(2, nq, envL[l], envR[l + 2], V, model.W[l], model.W[l + 1])
                E, v, _ = lanczos_np(op.hxv, V.data.copy(), max_iter, tol_eigval, tol_state)
                V.data[:] = v
                # the numpy restatement of the split (not the native library's routine)
                A1, A2, _, dmid = split_two_site(V, comb, qloc, qloc, din, dout, nq, Dmax, move=move,
                                                 eps_svd=eps_svd, native=False)
                mps.A[l], mps.A[l + 1] = A1, A2
                mps.dims[l + 1] = dmid
                if move == "right":
                    envL[l + 1] = env("L", envL[l], A1, model.W[l])
                else:
                    envR[l + 1] = env("R", envR[l + 2], A2, model.W[l + 1])
        times.append(time.perf_counter() - ts)
        energies.append(E)
    return {"energies": energies, "sweep_times": times}
