"""A two-site unit cell for the VUMPS transfer operator: sites 9 and 10 of a
20-site chain at bond dimension 24, whose bonds 9 and 11 carry the same sectors
with the same dimensions (left-right symmetry of the Hilbert-space counts), so
the cell maps an environment at bond 9 (11) to one with the same layout."""
import numpy as np

from vmps_gb300 import models
from vmps_gb300.blocks import Blocks
from vmps_gb300.mps import RandomMPS


def transfer_case(kind="heis", direction="L", seed=4, envs=None):
    m = models.heisenberg_u1(20) if kind == "heis" else models.heisenberg_su2(20)
    Q = (0,) if kind == "heis" else (1,)
    mps = RandomMPS(m, Q, 24, seed=seed).canonicalize(9, 10)
    assert mps.dims[9] == mps.dims[11]
    Lenv, Renv = envs(m, mps) if envs else (None, None)
    rng = np.random.default_rng(seed + 1)
    ent = [(0, q, q, rng.standard_normal((d, d))) for q, d in sorted(mps.dims[9].items())]
    LR = Blocks.from_entries(m.sym.nq, ent)
    order = m.basis_order_map(9)
    assert order == m.basis_order_map(11)
    cell = ([mps.A[9], mps.A[10]], [m.W[9], m.W[10]])
    return m, mps, cell, LR, order, (Lenv if direction == "L" else Renv)
