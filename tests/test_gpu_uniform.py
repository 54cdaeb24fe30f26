"""Config C4 quantities on the engine (vmps_gb300/uniform.py with the GPU contractions,
transfer operator, GMRES and pivots) against the same steps on the oracle: energy
density and VUMPS gradient norm of a gauge-fixed uniform SU(2) MPS (two-site cell), in
FP64 (1e-10) and in split precision with FP64-refined GMRES."""
import numpy as np
import pytest

from vmps_gb300 import models
from vmps_gb300.uniform import UniformEnvironment, UniformMPS, bond_bases_su2

from test_uniform_mps import oracle_hooks

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nmult,qmax", [(16, 8), (48, 12)])
def test_energy_density_and_gradient_against_oracle(gpu_ctx, nmult, qmax):
    m = models.heisenberg_su2(8)
    u = UniformMPS(m, bond_bases_su2(nmult, qmax), seed=5)
    assert u.gauge()["gauge_err"] < 1e-12
    order, W = m.basis_order_map(4), [m.W[4], m.W[5]]
    env, transfer, apply = oracle_hooks(m.sym)
    ref = UniformEnvironment(None, m, u, W, order, env=env, transfer=transfer, apply=apply)
    ref.left(); ref.right()
    g_ref, _ = ref.gradient()
    for prec, tol_e, tol_g in (("fp64", 1e-10, 1e-10), ("bf16x3", 1e-9, 1e-4)):
        E = UniformEnvironment(gpu_ctx, m, u, W, order, precision=prec, tol=1e-12)
        E.left(); E.right()
        g, _ = E.gradient()
        e, er = E.energy_density(), ref.energy_density()
        assert abs(e - er) < tol_e * abs(er), (prec, e, er)
        assert abs(g - g_ref) < tol_g * g_ref, (prec, g, g_ref)
