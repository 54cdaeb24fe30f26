"""End-to-end single-site DMRG on the GPU engine against exact diagonalisation
(the reference's DMRG-vs-ED check, programs/test_Hubbard/test_Hubbard.cc:227-300).
With complete bond bases the variational manifold contains the ground state."""
import numpy as np
import pytest

from oracle import ed
from vmps_gb300 import models
from vmps_gb300.dmrg import dmrg1
from vmps_gb300.mps import RandomMPS

pytestmark = pytest.mark.gpu


def _sector_mask_hubbard(L, N, M):
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == N and sum(bits[0::2]) - sum(bits[1::2]) == M)
    return np.array(mask)


def test_dmrg1_heisenberg_matches_ed(gpu_ctx):
    L = 10
    model = models.heisenberg_u1(L)
    mps = RandomMPS(model, (0,), 64, seed=3).canonicalize(0, 0)
    res = dmrg1(gpu_ctx, model, mps, n_sweeps=2, precision="fp64")
    H = models.dense_heisenberg(L)
    M = np.array([sum(1 if ((s >> (L - 1 - j)) & 1) == 0 else -1 for j in range(L)) for s in range(2 ** L)])
    e_ed = ed.ground_energy(H, M == 0)
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res, e_ed)


def test_dmrg1_hubbard_split_refined_matches_ed(gpu_ctx):
    L = 6
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 512, seed=4).canonicalize(0, 0)
    res = dmrg1(gpu_ctx, model, mps, n_sweeps=2, precision="bf16x3", tol_eigval=1e-9, tol_state=1e-5,
                refine_iters=40)
    e_ed = ed.ground_energy(models.dense_hubbard(L, 1.0, 4.0), _sector_mask_hubbard(L, L, 0))
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res, e_ed)
