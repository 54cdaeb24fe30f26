"""Synthetic frozen-site workloads (seeded) for benchmarks and tests.

A frozen site is the middle of a chain: a random MPS (N(0,1) blocks, QR/LQ
normalised towards the pivot), its left and right environments built with the
engine's own contract_L / contract_R on the GPU, the MPO tensors of the pivot
sites, and the pivot vector layout.  The reference publishes no benchmark data;
these inputs stand in for its benchmark configurations (Heisenberg chain, Hubbard
chain at D=1024 / 4096, SU(2)xU(1) Hubbard cylinder, ...) with their shapes.
"""
from __future__ import annotations

import time

from . import models
import numpy as np

from .mps import RandomMPS, contract_two_sites, two_site_layout
from .pivot import EnvUpdate, left_vacuum, right_target


def build_envs(ctx, model, mps, lo, hi, precision="fp64"):
    """L env at bond lo (sites < lo) and R env at bond hi+1 (sites > hi) on the GPU."""
    sym = model.sym
    Lenv = left_vacuum(sym)
    for l in range(lo):
        e = EnvUpdate(ctx, sym, "L", Lenv, mps.A[l], model.W[l], mps.A[l])
        Lenv = e.run(Lenv, mps.A[l], mps.A[l], precision)
        e.close()
    Renv = right_target(sym, mps.Qtot)
    for l in range(model.L - 1, hi, -1):
        e = EnvUpdate(ctx, sym, "R", Renv, mps.A[l], model.W[l], mps.A[l])
        Renv = e.run(Renv, mps.A[l], mps.A[l], precision)
        e.close()
    return Lenv, Renv


def hubbard_two_site(ctx, L=64, D=4096, U=4.0, seed=2, sigma=2.5, verbose=False, Qtot=None):
    """Hubbard U(1)xU(1) chain, two-site pivot at the middle; total (N, 2Sz) = Qtot,
    half filling with Sz = 0 by default."""
    t0 = time.time()
    model = models.hubbard_u1xu1(L, t=1.0, U=U)
    site = L // 2 - 1
    Qtot = (L, 0) if Qtot is None else tuple(Qtot)
    mps = RandomMPS(model, Qtot, D, seed=seed, profile="gaussian", sigma=[sigma, sigma])
    mps.canonicalize(site, site + 1)
    t1 = time.time()
    Lenv, Renv = build_envs(ctx, model, mps, site, site + 1)
    t2 = time.time()
    V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, model.sym.nq)
    info = dict(model=model.name, L=L, D=D, site=site, seed=seed, sigma=sigma,
                D_left=mps.bond_dim(site), D_right=mps.bond_dim(site + 2),
                sectors_left=len(mps.dims[site]), dim_V=int(V.data.size),
                env_elems=int(Lenv.data.size + Renv.data.size), setup_mps_s=round(t1 - t0, 2), setup_env_s=round(t2 - t1, 2))
    if verbose:
        print("workload", info, flush=True)
    return model, mps, Lenv, Renv, model.W[site], model.W[site + 1], V, info


def heisenberg_two_site(ctx, L=32, D=64, seed=1):
    """Heisenberg U(1) chain, Sz = 0; two-site pivot in the middle (the same return
    values as hubbard_two_site)."""
    model = models.heisenberg_u1(L)
    site = L // 2 - 1
    mps = RandomMPS(model, (0,), D, seed=seed, profile="gaussian", sigma=[4.0]).canonicalize(site, site + 1)
    Lenv, Renv = build_envs(ctx, model, mps, site, site + 1)
    V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, model.sym.nq)
    info = dict(model=model.name, L=L, D=D, site=site, seed=seed, D_left=mps.bond_dim(site),
                sectors_left=len(mps.dims[site]), dim_V=int(V.data.size),
                env_elems=int(Lenv.data.size + Renv.data.size))
    return model, mps, Lenv, Renv, model.W[site], model.W[site + 1], V, info


def heisenberg_one_site(ctx, L=32, D=64, seed=1, site=None):
    """Heisenberg U(1) chain, Sz = 0; one-site pivot (default: the middle)."""
    model = models.heisenberg_u1(L)
    site = L // 2 - 1 if site is None else site
    mps = RandomMPS(model, (0,), D, seed=seed, profile="gaussian", sigma=[4.0]).canonicalize(site, site)
    Lenv, Renv = build_envs(ctx, model, mps, site, site)
    return model, mps, Lenv, Renv, model.W[site], mps.A[site]


def hubbard_su2xu1_cylinder_two_site(ctx, Lx=16, W=4, D=2000, U=8.0, N=None, seed=3, sigma=(3.0, 3.0), verbose=False):
    """Config C3: Hubbard SU(2)xU(1) on a width-W cylinder of Lx rings mapped to an
    L = Lx*W snake (hoppings around the rings and between rings, MPO w = 2W+2), U/t = U,
    N electrons (default 1/8 hole doping), total spin 0; D multiplets per bond from a
    Gaussian sector profile; two-site pivot at the middle.  The pivot vector is seeded
    N(0,1) data in the SU(2) two-site layout (its values do not enter the timings)."""
    t0 = time.time()
    L = Lx * W
    N = int(round(L * 7 / 8)) if N is None else N
    model = models.hubbard_su2xu1_lattice(L, models.cylinder_bonds(Lx, W), U=U)
    site = L // 2 - 1
    mps = RandomMPS(model, (1, N), D, seed=seed, profile="gaussian", sigma=list(sigma))
    mps.canonicalize(site, site + 1)
    t1 = time.time()
    Lenv, Renv = build_envs(ctx, model, mps, site, site + 1)
    t2 = time.time()
    V, _ = two_site_layout(model.sym, model.qloc, model.qloc, mps.dims[site], mps.dims[site + 2], model.sym.nq)
    V.data[:] = np.random.default_rng(seed).standard_normal(V.data.size)
    mid = mps.dims[site + 1]
    info = dict(model=model.name, L=L, width=W, N=N, D_multiplets=sum(mid.values()),
                D_states=sum(q[0] * n for q, n in mid.items()), sectors=len(mid), mpo_w=model.wdim,
                max_sector=max(mid.values()), dim_V=int(V.data.size), seed=seed,
                setup_mps_s=round(t1 - t0, 2), setup_env_s=round(t2 - t1, 2))
    if verbose:
        print("workload", info, flush=True)
    return model, mps, Lenv, Renv, model.W[site], model.W[site + 1], V, info
