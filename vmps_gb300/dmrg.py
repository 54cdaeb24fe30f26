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

import contextlib
import os
import time

import numpy as np

from .mps import contract_two_sites, gauge_step, split_two_site
from .pivot import EnvUpdate, PivotMatrix1, PivotMatrix2, left_vacuum, right_target
from .su2 import contract_two_sites_su2, split_two_site_su2


class SweepResult(dict):
    pass


def _count(counts, st):
    """add one Lanczos call's statistics to the running totals"""
    counts["solves"] = counts.get("solves", 0) + 1
    for k in ("hxv_split", "hxv_fp64", "refine_iterations"):
        counts[k] = counts.get(k, 0) + int(st[k])


@contextlib.contextmanager
def _probe_setting(probe):
    """probe=False: split-precision solves skip the FP64 probe (VMPS_LANCZOS_PROBE=off)
    for the duration of the sweeps"""
    if probe:
        yield
        return
    old = os.environ.get("VMPS_LANCZOS_PROBE")
    os.environ["VMPS_LANCZOS_PROBE"] = "off"
    try:
        yield
    finally:
        if old is None:
            del os.environ["VMPS_LANCZOS_PROBE"]
        else:
            os.environ["VMPS_LANCZOS_PROBE"] = old


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
          refine_iters=0, verbose=False, pool=None, probe=True, enrich=0.0, enrich_decay=0.5, Dmax=None):
    """Run n_sweeps full sweeps of single-site DMRG; returns energies and timings.
    `mps` must be right-canonical with the gauge centre on site 0.  The QR / LQ gauge
    steps run on the host cores (`pool`, a hostla.SectorPool; one is made if none is
    given).  The result's `steps` lists every local solve: its energy and its HxV
    counts per precision.  probe=False makes split-precision solves skip the FP64 probe.

    enrich > 0 turns on the subspace expansion of DMRG::BROOM::RICH_SVD (abelian
    symmetries; enrich.py): after each local solve the bond about to be crossed is
    enlarged by alpha * L A W (moving right) or alpha * A W R (moving left) and truncated
    back to at most Dmax states (default: the largest bond dimension of the MPS), with
    alpha = enrich * enrich_decay**sweep.  Bond bases then change during the sweep."""
    if enrich > 0 and model.sym.nonabelian:
        raise ValueError("the subspace expansion is implemented for abelian symmetries")
    with _probe_setting(probe):
        return _dmrg1(ctx, model, mps, n_sweeps, precision, max_iter, tol_eigval, tol_state, refine_iters, verbose,
                      pool, enrich, enrich_decay, Dmax)


def _dmrg1(ctx, model, mps, n_sweeps, precision, max_iter, tol_eigval, tol_state, refine_iters, verbose, pool,
           enrich=0.0, enrich_decay=0.5, Dmax=None):
    sym, L = model.sym, model.L
    nq = sym.nq
    own_pool = pool is None
    if own_pool:
        from .hostla import SectorPool
        pool = SectorPool()
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
    energies, sweep_times, timers, solves, hxv, steps = [], [], [], [], 0, []
    E = None
    clock = time.perf_counter
    if enrich > 0:
        from .enrich import enrich_left, enrich_right
        Dmax = Dmax if Dmax is not None else max(mps.bond_dim(b) for b in range(L + 1))
    for sweep in range(n_sweeps):
        ts = clock()
        tm = dict(lanczos=0.0, precalc=0.0, gauge=0.0, lr=0.0)
        alpha = enrich * enrich_decay ** sweep
        counts = {}
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
            _count(counts, st)
            steps.append((sweep, l, E, st["hxv_split"], st["hxv_fp64"]))
            H.close()
            t2 = clock()
            tm["precalc"] += t1 - t
            tm["lanczos"] += t2 - t1
            mps.A[l].data[:] = v
            if right and l < L - 1:
                if alpha > 0:
                    enrich_right(ctx, model, mps, l, envL[l], alpha, Dmax, pool=pool)
                else:
                    gauge_step(mps.A[l], mps.A[l + 1], nq, "right", sym=mps.sym, pool=pool)
                t3 = clock()
                e = EnvUpdate(ctx, sym, "L", envL[l], mps.A[l], model.W[l], mps.A[l])
                envL[l + 1] = e.run(envL[l], mps.A[l], mps.A[l])
                e.close()
            elif not right and l > 0:
                if alpha > 0:
                    enrich_left(ctx, model, mps, l, envR[l + 1], alpha, Dmax, pool=pool)
                else:
                    gauge_step(mps.A[l], mps.A[l - 1], nq, "left", sym=mps.sym, pool=pool)
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
        solves.append(counts)
        energies.append(E)
        if verbose:
            print(f"sweep {sweep}: E = {E:.14f}  ({sweep_times[-1]:.2f} s)", flush=True)
    if own_pool:
        pool.close()
    return SweepResult(energies=energies, sweep_times=sweep_times, timers=timers, init_time=t_init, hxv=hxv,
                       solves=solves, steps=steps)


def _env(ctx, sym, side, E, A, W):
    e = EnvUpdate(ctx, sym, side, E, A, W, A)
    out = e.run(E, A, A)
    e.close()
    return out


def dmrg2(ctx, model, mps, n_sweeps=2, Dmax=None, precision="fp64", max_iter=100, tol_eigval=1e-12,
          tol_state=1e-8, refine_iters=0, eps_svd=1e-14, pool=None, factor="eigh", verbose=False, window=None,
          probe=True, split_device=True):
    """Two-site DMRG sweeps (DmrgSolver::iteration_two, solvers/DmrgSolver.h:1399-1522): per bond
    (l, l+1) the two-site tensor A[l] A[l+1] (contract_AA2) is the start vector of the Lanczos
    ground state of PivotMatrix2(L[l], R[l+2], W[l], W[l+1]); split_AA2 with a truncated SVD
    (at most Dmax states over all sectors of the middle bond) returns the two sites, the
    orthonormal one feeds contract_L (left-to-right) or contract_R (right-to-left).  Bond
    bases grow and shrink with the SVD.  With SU(2) components the contraction and the
    split are the non-abelian branches (su2.py: coeff_twoSiteGate / coeff_splitAA
    recoupling, multiplets kept by their singular values, host SVD).

    `mps` must be right-canonical with the gauge centre on site 0.  A sweep is a
    left-to-right pass over bonds 0..L-2 followed by a right-to-left pass over L-2..0.
    window=(lo, hi) sweeps bonds lo..hi-1 and back instead (sites < lo left-canonical,
    sites > lo+1 right-canonical), the steps of a full sweep in that part of the chain.
    Timers per sweep as in dmrg1; "gauge" holds the two-site contraction ("contract") and
    the SVD ("split"), whose sectors run on the host cores (`pool`, a hostla.SectorPool; one is made if
    none is given); with split_device (default) the sectors whose Gram matrix has order
    >= 512 run on the GPU in FP64 (vmps_two_site_split_device).  `steps` lists every
    local solve (energy, HxV counts per precision); probe=False makes split-precision
    solves skip the FP64 probe."""
    with _probe_setting(probe):
        return _dmrg2(ctx, model, mps, n_sweeps, Dmax, precision, max_iter, tol_eigval, tol_state, refine_iters,
                      eps_svd, pool, factor, verbose, window, split_device)


def _dmrg2(ctx, model, mps, n_sweeps, Dmax, precision, max_iter, tol_eigval, tol_state, refine_iters, eps_svd,
           pool, factor, verbose, window, split_device):
    sym, L, nq = model.sym, model.L, model.sym.nq
    su2 = sym.nonabelian
    Dmax = Dmax if Dmax is not None else max(mps.bond_dim(l) for l in range(L + 1))
    qloc = model.qloc
    own_pool = pool is None
    if own_pool:
        from .hostla import SectorPool
        pool = SectorPool()
    envL = [None] * (L + 1)
    envR = [None] * (L + 1)
    envL[0] = left_vacuum(sym)
    envR[L] = right_target(sym, mps.Qtot)
    lo, hi = (0, L - 1) if window is None else (int(window[0]), int(window[1]))
    if not 0 <= lo < hi <= L - 1:
        raise ValueError("window must satisfy 0 <= lo < hi <= L-1")
    t0 = time.perf_counter()
    for l in range(lo):
        envL[l + 1] = _env(ctx, sym, "L", envL[l], mps.A[l], model.W[l])
    for l in range(L - 1, lo + 1, -1):
        envR[l] = _env(ctx, sym, "R", envR[l + 1], mps.A[l], model.W[l])
    t_init = time.perf_counter() - t0
    energies, sweep_times, timers, solves, trunc, dims, hxv, steps = [], [], [], [], [], [], 0, []
    E = None
    clock = time.perf_counter
    for sweep in range(n_sweeps):
        ts = clock()
        tm = dict(lanczos=0.0, precalc=0.0, gauge=0.0, lr=0.0, contract=0.0, split=0.0)
        counts = {}
        disc_max = 0.0
        for move, bonds in (("right", range(lo, hi)), ("left", range(hi - 1, lo - 1, -1))):
            for l in bonds:
                t = clock()
                A1, A2 = mps.A[l], mps.A[l + 1]
                din = {tuple(A1.qin[i]): int(A1.rows[i]) for i in range(A1.n)}
                dout = {tuple(A2.qout[i]): int(A2.cols[i]) for i in range(A2.n)}
                if su2:
                    V, comb = contract_two_sites_su2(sym, A1, A2, qloc, qloc, ctx=ctx)
                else:
                    V, comb = contract_two_sites(sym, A1, A2, qloc, qloc, nq, return_basis=True, ctx=ctx)
                t1 = clock()
                H = PivotMatrix2(ctx, sym, envL[l], envR[l + 2], model.W[l], model.W[l + 1], V)
                H.prepare("fp64" if refine_iters > 0 else precision)
                t2 = clock()
                E, v, st = H.lanczos(V.data, precision, max_iter=max_iter, tol_eigval=tol_eigval,
                                     tol_state=tol_state, refine_iters=refine_iters)
                hxv += st["hxv_fp64"] + st["hxv_split"]
                _count(counts, st)
                steps.append((sweep, l, E, st["hxv_split"], st["hxv_fp64"]))
                H.close()
                t3 = clock()
                V.data[:] = v
                if su2:
                    A1, A2, disc, dmid = split_two_site_su2(V, comb, sym, qloc, qloc, din, dout, Dmax, move=move,
                                                            eps_svd=eps_svd)
                else:
                    A1, A2, disc, dmid = split_two_site(V, comb, qloc, qloc, din, dout, nq, Dmax, move=move,
                                                        eps_svd=eps_svd, pool=pool, factor=factor,
                                                        ctx=ctx if split_device else None)
                mps.A[l], mps.A[l + 1] = A1, A2
                mps.dims[l + 1] = dmid
                disc_max = max(disc_max, disc)
                t4 = clock()
                if move == "right":
                    envL[l + 1] = _env(ctx, sym, "L", envL[l], A1, model.W[l])
                else:
                    envR[l + 1] = _env(ctx, sym, "R", envR[l + 2], A2, model.W[l + 1])
                t5 = clock()
                tm["gauge"] += (t1 - t) + (t4 - t3)
                tm["contract"] += t1 - t
                tm["split"] += t4 - t3
                tm["precalc"] += t2 - t1
                tm["lanczos"] += t3 - t2
                tm["lr"] += t5 - t4
        sweep_times.append(clock() - ts)
        timers.append(tm)
        solves.append(counts)
        energies.append(E)
        trunc.append(disc_max)
        dims.append(max(sum(mps.dims[l].values()) for l in range(1, L)))
        if verbose:
            print(f"sweep {sweep}: E = {E:.14f}  D = {dims[-1]}  trunc = {disc_max:.2e}  ({sweep_times[-1]:.2f} s)",
                  flush=True)
    if own_pool:
        pool.close()
    return SweepResult(energies=energies, sweep_times=sweep_times, timers=timers, init_time=t_init, hxv=hxv,
                       solves=solves, truncation=trunc, max_bond_dim=dims, steps=steps)
