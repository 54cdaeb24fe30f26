"""Two-site DMRG with SU(2) symmetry on the engine (vmps_gb300.dmrg.dmrg2 with the
non-abelian contract_AA2 / split_AA2 of su2.py): the ground-state energies of the
SU(2) Heisenberg chain and the SU(2) x U(1) Hubbard chain equal exact diagonalisation
of the same chains with U(1) symmetries (the cross-symmetry check of
programs/test_Heisenberg/test_Heisenberg.cc:373-400), in FP64 and in split precision
with FP64 refinement."""
import numpy as np
import pytest

from oracle import ed
from vmps_gb300 import models
from vmps_gb300.dmrg import dmrg2
from vmps_gb300.mps import RandomMPS

pytestmark = pytest.mark.gpu


def _hubbard_sector(L, N, M):
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == N and sum(bits[0::2]) - sum(bits[1::2]) == M)
    return np.array(mask)


@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_su2_heisenberg_two_site_reaches_ed(gpu_ctx, precision):
    L = 10
    model = models.heisenberg_su2(L)
    mps = RandomMPS(model, (1,), 8, seed=1).canonicalize(0, 0)
    kw = dict(tol_eigval=1e-12, tol_state=1e-8, refine_iters=10) if precision == "bf16x3" else {}
    r = dmrg2(gpu_ctx, model, mps, n_sweeps=3, Dmax=64, precision=precision, **kw)
    e0 = float(np.linalg.eigvalsh(ed.mpo_to_dense(models.heisenberg_u1(L)))[0])
    assert abs(r["energies"][-1] - e0) < 1e-10 * abs(e0), (r["energies"], e0)
    assert max(mps.bond_dim(b) for b in range(L + 1)) > 8   # multiplets grew from D=8


@pytest.mark.parametrize("precision", ["fp64", "bf16x3"])
def test_su2xu1_hubbard_two_site_reaches_ed(gpu_ctx, precision):
    L = 6
    model = models.hubbard_su2xu1_lattice(L, [(i, i + 1, 1.0) for i in range(L - 1)], U=4.0)
    mps = RandomMPS(model, (1, L), 8, seed=1).canonicalize(0, 0)
    kw = dict(tol_eigval=1e-12, tol_state=1e-8, refine_iters=10) if precision == "bf16x3" else {}
    r = dmrg2(gpu_ctx, model, mps, n_sweeps=5, Dmax=64, precision=precision, **kw)
    mu = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    H = ed.permute_to_reference(ed.mpo_to_dense(mu), mu)
    e0 = ed.ground_energy(H, _hubbard_sector(L, L, 0))
    assert abs(r["energies"][-1] - e0) < 1e-10 * abs(e0), (r["energies"], e0)
