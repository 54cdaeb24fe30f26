"""SU(2) end to end on the GPU engine: the spin-1/2 Heisenberg chain with SU(2)
symmetry (reduced W of models.heisenberg_su2, the 9j/6j coefficient families of
the builders, SU(2)-weighted vectors) against U(1) physics, the cross-symmetry
check the reference runs in programs/test_Heisenberg/test_Heisenberg.cc:373-400.

* the dimer: singlet E = -3/4, triplet E = +1/4 (one reduced state each);
* three sites, two-site pivot with one left-normalised site: the S = 1/2 sector
  has the energies {-1, 0};
* ten sites, single-site DMRG with complete multiplet bases: the ground energy
  equals the U(1) exact diagonalisation (FP64, and split precision + FP64 refinement).
"""
import numpy as np
import pytest

from oracle import ed
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import PivotMatrix2, left_vacuum, right_target

pytestmark = pytest.mark.gpu


def _pivot2(ctx, m, mps, site):
    from vmps_gb300.pivot import contract_L, contract_R
    sym = m.sym
    L = left_vacuum(sym)
    for l in range(site):
        L = contract_L(ctx, sym, L, mps.A[l], m.W[l], mps.A[l])
    R = right_target(sym, mps.Qtot)
    for l in range(m.L - 1, site + 1, -1):
        R = contract_R(ctx, sym, R, mps.A[l], m.W[l], mps.A[l])
    V = contract_two_sites(sym, mps.A[site], mps.A[site + 1], m.qloc, m.qloc, sym.nq)
    return PivotMatrix2(ctx, sym, L, R, m.W[site], m.W[site + 1], V)


def _dense(H, prec):
    n = H.dim
    return np.column_stack([H.apply(np.eye(n)[:, j], prec) for j in range(n)])


@pytest.mark.parametrize("qtot,energy", [((1,), -0.75), ((3,), 0.25)])
def test_su2_dimer(gpu_ctx, qtot, energy):
    m = models.heisenberg_su2(2)
    mps = RandomMPS(m, qtot, 4, seed=1).canonicalize(0, 1)
    H = _pivot2(gpu_ctx, m, mps, 0)
    assert H.dim == 1
    v = np.ones(1)
    assert abs(H.apply(v, "fp64")[0] - energy) < 1e-13
    assert abs(H.apply(v, "bf16x3")[0] - energy) < 1e-4 * abs(energy)
    H.close()


def test_su2_three_sites_doublet_sector(gpu_ctx):
    m = models.heisenberg_su2(3)
    mps = RandomMPS(m, (2,), 8, seed=2).canonicalize(1, 2)
    H = _pivot2(gpu_ctx, m, mps, 1)
    ev = np.sort(np.linalg.eigvals(_dense(H, "fp64")).real)
    assert np.allclose(ev, [-1.0, 0.0], atol=1e-12), ev
    H.close()


def _heisenberg_ed(L):
    H = models.dense_heisenberg(L)
    M = np.array([sum(1 if ((s >> (L - 1 - j)) & 1) == 0 else -1 for j in range(L)) for s in range(2 ** L)])
    return ed.ground_energy(H, M == 0)


@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_su2_dmrg_matches_u1_ed(gpu_ctx, precision):
    from vmps_gb300.dmrg import dmrg1
    L = 10
    m = models.heisenberg_su2(L)
    mps = RandomMPS(m, (1,), 64, seed=3).canonicalize(0, 0)
    kw = dict(tol_eigval=1e-9, tol_state=1e-5, refine_iters=40) if precision == "bf16x3" else {}
    res = dmrg1(gpu_ctx, m, mps, n_sweeps=2, precision=precision, **kw)
    e_ed = _heisenberg_ed(L)
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res["energies"], e_ed)


def _hubbard_ed(model_u1, L, N):
    H = ed.permute_to_reference(ed.mpo_to_dense(model_u1), model_u1)
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == N and sum(bits[0::2]) - sum(bits[1::2]) == 0)
    return ed.ground_energy(H, np.array(mask))


@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_su2xu1_hubbard_chain_matches_u1_ed(gpu_ctx, precision):
    """SU(2)xU(1) Hubbard (reduced fermion operators, sign strings) against the U(1)xU(1) ED"""
    from vmps_gb300.dmrg import dmrg1
    L = 4
    m = models.hubbard_su2xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(m, (1, L), 64, seed=7).canonicalize(0, 0)
    kw = dict(tol_eigval=1e-10, tol_state=1e-7, refine_iters=10) if precision == "bf16x3" else {}
    res = dmrg1(gpu_ctx, m, mps, n_sweeps=3, precision=precision, **kw)
    e_ed = _hubbard_ed(models.hubbard_u1xu1(L, 1.0, 4.0), L, L)
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res["energies"], e_ed)


def test_su2xu1_hubbard_ladder_matches_u1_ed(gpu_ctx):
    """the width-2 ladder (range-2 hoppings through a sign string) with SU(2)xU(1); Dmax=128
    so that the even split over the 10 middle sectors keeps every multiplet (8 at most)"""
    from vmps_gb300.dmrg import dmrg1
    L = 6
    bonds = models.cylinder_bonds(3, 2)
    m = models.hubbard_su2xu1_lattice(L, bonds, U=8.0)
    mps = RandomMPS(m, (1, L), 128, seed=8).canonicalize(0, 0)
    res = dmrg1(gpu_ctx, m, mps, n_sweeps=4, precision="fp64")
    e_ed = _hubbard_ed(models.hubbard_u1xu1_lattice(L, bonds, U=8.0), L, L)
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res["energies"], e_ed)
