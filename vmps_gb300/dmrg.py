"""Single-site DMRG sweeps over the GB300 engine.

The sweep logic follows DmrgSolver::halfsweep / iteration_one
(solvers/DmrgSolver.h:750-846, :1236-1376) for fixed bond bases:

    for each site l (left-to-right, then right-to-left):
        H = PivotMatrix1(L[l], R[l+1], W[l])            # precalc_blockStructure
        E, A[l] = Lanczos ground state of H              # edgeState, on the device
        QR / LQ gauge step, factor pushed to the next site (Mps::sweepStep, QR branch)
        L[l+1] = contract_L(...) or R[l] = contract_R(...)

HxV, Lanczos and contract_L/R run on the GPU.  The gauge step is a host QR per
QN sector, as in Biped::QR (tensors/Biped.h:901-932).  Bond dimensions stay
fixed (no subspace expansion).

Each sweep's wall time is split like the reference's halfsweep timer
(solvers/DmrgSolver.h:837-845): "lanczos" (the local eigensolver), "precalc"
(the pivot's task lists and plans), "gauge" (QR / LQ and the push to the next
site) and "lr" (contract_L / contract_R).
"""
from __future__ import annotations

import time

import numpy as np

from .mps import left_normalize, right_normalize
from .pivot import EnvUpdate, PivotMatrix1, left_vacuum, right_target


class SweepResult(dict):
    pass


def _push_right(A_next, Rfac):
    """A_next[s](qin, qout) <- R[qin] @ A_next[s](qin, qout)"""
    for i in range(A_next.n):
        q = tuple(A_next.qin[i])
        if q in Rfac:
            A_next.block(i)[...] = Rfac[q] @ A_next.block(i)


def _push_left(A_prev, Lfac):
    for i in range(A_prev.n):
        q = tuple(A_prev.qout[i])
        if q in Lfac:
            A_prev.block(i)[...] = A_prev.block(i) @ Lfac[q]


def dmrg1(ctx, model, mps, n_sweeps=2, precision="fp64", max_iter=100, tol_eigval=1e-12, tol_state=1e-8,
          refine_iters=0, verbose=False):
    """Run n_sweeps full sweeps of single-site DMRG; returns energies and timings.
    `mps` must be right-canonical with the gauge centre on site 0."""
    sym, L = model.sym, model.L
    nq = sym.nq
    envL = [None] * (L + 1)
    envR = [None] * (L + 1)
    envL[0] = left_vacuum(sym)
    envR[L] = right_target(sym, mps.Qtot)
    t0 = time.perf_counter()
    for l in range(L - 1, 0, -1):
        e = EnvUpdate(ctx, sym, "R", envR[l + 1], mps.A[l], model.W[l], mps.A[l])
        envR[l] = e.run(envR[l + 1], mps.A[l], mps.A[l])
        e.close()
    t_init = time.perf_counter() - t0
    energies, sweep_times, timers, hxv = [], [], [], 0
    E = None
    clock = time.perf_counter
    for sweep in range(n_sweeps):
        ts = clock()
        tm = dict(lanczos=0.0, precalc=0.0, gauge=0.0, lr=0.0)
        order = list(range(L)) + list(range(L - 1, -1, -1))
        for step, l in enumerate(order):
            right = step < L
            t = clock()
            H = PivotMatrix1(ctx, sym, envL[l], envR[l + 1], model.W[l], mps.A[l])
            H.prepare("fp64" if refine_iters > 0 else precision)   # the split plan is built if the split phase runs
            t1 = clock()
            E, v, st = H.lanczos(mps.A[l].data, precision, max_iter=max_iter, tol_eigval=tol_eigval,
                                 tol_state=tol_state, refine_iters=refine_iters)
            hxv += st["hxv_fp64"] + st["hxv_split"]
            H.close()
            t2 = clock()
            tm["precalc"] += t1 - t
            tm["lanczos"] += t2 - t1
            mps.A[l].data[:] = v
            if right and l < L - 1:
                mps.A[l], Rf = left_normalize(mps.A[l], nq, sym=mps.sym)
                _push_right(mps.A[l + 1], Rf)
                t3 = clock()
                e = EnvUpdate(ctx, sym, "L", envL[l], mps.A[l], model.W[l], mps.A[l])
                envL[l + 1] = e.run(envL[l], mps.A[l], mps.A[l])
                e.close()
            elif not right and l > 0:
                mps.A[l], Lf = right_normalize(mps.A[l], nq, sym=mps.sym)
                _push_left(mps.A[l - 1], Lf)
                t3 = clock()
                e = EnvUpdate(ctx, sym, "R", envR[l + 1], mps.A[l], model.W[l], mps.A[l])
                envR[l] = e.run(envR[l + 1], mps.A[l], mps.A[l])
                e.close()
            else:
                t3 = clock()
            t4 = clock()
            tm["gauge"] += t3 - t2
            tm["lr"] += t4 - t3
        sweep_times.append(clock() - ts)
        timers.append(tm)
        energies.append(E)
        if verbose:
            print(f"sweep {sweep}: E = {E:.14f}  ({sweep_times[-1]:.2f} s)", flush=True)
    return SweepResult(energies=energies, sweep_times=sweep_times, timers=timers, init_time=t_init, hxv=hxv)
