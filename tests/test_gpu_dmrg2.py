"""Two-site DMRG on the GPU engine (config C2's algorithm): bond bases grow
from a small random MPS under the truncated SVD; the ground energy matches
exact diagonalisation (DMRG vs ED, programs/test_Hubbard/test_Hubbard.cc:227-300)
in FP64 and in split precision with FP64 refinement, and the GPU sweep agrees
with the same sweep on the CPU oracle."""
import copy

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
def test_dmrg2_hubbard_matches_ed(gpu_ctx, precision):
    L = 6
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 4, seed=5).canonicalize(0, 0)
    kw = dict(tol_eigval=1e-10, tol_state=1e-7, refine_iters=10) if precision == "bf16x3" else {}
    res = dmrg2(gpu_ctx, model, mps, n_sweeps=3, Dmax=64, precision=precision, **kw)
    H = ed.permute_to_reference(ed.mpo_to_dense(model), model)
    e_ed = ed.ground_energy(H, _hubbard_sector(L, L, 0))
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res, e_ed)
    assert res["max_bond_dim"][-1] > 4


def test_dmrg2_heisenberg_gpu_matches_oracle_sweep(gpu_ctx):
    """converged truncated two-site DMRG (D=16 < exact 32): GPU and CPU-oracle sweeps agree"""
    from oracle.dmrg_cpu import dmrg2_cpu
    L = 10
    model = models.heisenberg_u1(L)
    mps = RandomMPS(model, (0,), 8, seed=6).canonicalize(0, 0)
    mps_cpu = copy.deepcopy(mps)
    g = dmrg2(gpu_ctx, model, mps, n_sweeps=4, Dmax=16, precision="fp64")
    c = dmrg2_cpu(model, mps_cpu, n_sweeps=4, Dmax=16)
    assert abs(g["energies"][-1] - c["energies"][-1]) < 1e-10 * abs(c["energies"][-1]), (g, c)
    assert g["max_bond_dim"][-1] == 16 and g["truncation"][-1] > 0


def test_two_site_contraction_on_gpu_matches_host(gpu_ctx):
    """contract_AA2 as one FP64 grouped GEMM against the host products: with the
    products found in the library (vmps_two_site_contract_pairs, the path
    contract_two_sites takes) and with an explicit product list
    (vmps_two_site_contract); both give the same bits."""
    import ctypes as C
    from vmps_gb300 import _native as N
    from vmps_gb300.mps import contract_two_sites
    m = models.hubbard_u1xu1(12)
    mps = RandomMPS(m, (12, 0), 96, seed=9).canonicalize(5, 6)
    A1, A2 = mps.A[5], mps.A[6]
    Vh, comb = contract_two_sites(m.sym, A1, A2, m.qloc, m.qloc, 2, return_basis=True)
    Vg, _ = contract_two_sites(m.sym, A1, A2, m.qloc, m.qloc, 2, return_basis=True, ctx=gpu_ctx)
    assert np.linalg.norm(Vg.data - Vh.data) <= 1e-14 * np.linalg.norm(Vh.data)
    prods = []
    for i in range(A1.n):
        for j in range(A2.n):
            if tuple(A1.qout[i]) != tuple(A2.qin[j]):
                continue
            s13 = comb["index"][(int(A1.leg[i]), int(A2.leg[j]))][0][1]
            k = Vh.find(s13, tuple(A1.qin[i]), tuple(A2.qout[j]))
            if k >= 0:
                prods.append((k, i, j))
    tri = np.ascontiguousarray(np.array(prods, dtype=np.int64).reshape(-1, 3))
    Ve = Vh.like()
    s_, b1, b2, bv = m.sym.c_struct(), A1.c_struct(), A2.c_struct(), Ve.c_struct()
    N.check(N.lib().vmps_two_site_contract(gpu_ctx._h, C.byref(s_), C.byref(b1), A1.data_ptr(), C.byref(b2),
                                           A2.data_ptr(), C.byref(bv), Ve.data_ptr(), len(prods),
                                           tri.ctypes.data_as(N.i64p)))
    assert np.array_equal(Ve.data, Vg.data)


def test_dmrg2_window(gpu_ctx):
    """dmrg2(window=(lo, hi)): the window (0, L-1) is the full sweep (same bits), and
    a window sweep in the middle of a converged MPS (re-centred there) keeps the ED
    energy; bonds outside the window keep their bases"""
    L = 6
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 4, seed=5).canonicalize(0, 0)
    full = dmrg2(gpu_ctx, model, copy.deepcopy(mps), n_sweeps=1, Dmax=64, precision="fp64")
    win = dmrg2(gpu_ctx, model, copy.deepcopy(mps), n_sweeps=1, Dmax=64, precision="fp64", window=(0, L - 1))
    assert full["energies"] == win["energies"]
    with pytest.raises(ValueError):
        dmrg2(gpu_ctx, model, copy.deepcopy(mps), n_sweeps=1, Dmax=64, window=(3, 3))
    conv = copy.deepcopy(mps)
    dmrg2(gpu_ctx, model, conv, n_sweeps=3, Dmax=64, precision="fp64")
    # after full sweeps the centre is on site 0 (right-canonical); move it to sites (2, 3)
    centred = copy.deepcopy(conv).canonicalize(2, 3)
    dims_before = [dict(centred.dims[b]) for b in (1, 5)]
    r = dmrg2(gpu_ctx, model, centred, n_sweeps=1, Dmax=64, precision="bf16x3", tol_eigval=1e-10,
              tol_state=1e-7, refine_iters=10, window=(2, 4))
    H = ed.permute_to_reference(ed.mpo_to_dense(model), model)
    e_ed = ed.ground_energy(H, _hubbard_sector(L, L, 0))
    assert abs(r["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (r, e_ed)
    assert [dict(centred.dims[b]) for b in (1, 5)] == dims_before


def test_converged_sweep_split_equals_fp64_step_by_step(gpu_ctx):
    """A converged two-site sweep (Hubbard L=24, Dmax=256) in both precisions with
    tight tolerances from the same MPS; the split-precision run skips the FP64 probe,
    so every local solve runs split HxVs before its FP64 refinement.  Every one of
    the sweep's local ground-state energies agrees with the FP64 sweep to 1e-10
    relative (the |dE/E| of the metric), and so does the final energy."""
    L = 24
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 256, seed=2, profile="gaussian", sigma=[2.5, 2.5]).canonicalize(0, 0)
    dmrg2(gpu_ctx, model, mps, n_sweeps=4, Dmax=256, precision="bf16x3", refine_iters=10, tol_eigval=1e-12,
          tol_state=1e-8)
    tight = dict(tol_eigval=1e-13, tol_state=1e-10)
    r64 = dmrg2(gpu_ctx, model, copy.deepcopy(mps), n_sweeps=1, Dmax=256, precision="fp64", **tight)
    rsp = dmrg2(gpu_ctx, model, copy.deepcopy(mps), n_sweeps=1, Dmax=256, precision="bf16x3", refine_iters=10,
                probe=False, **tight)
    e64 = np.array([s[2] for s in r64["steps"]])
    esp = np.array([s[2] for s in rsp["steps"]])
    assert sum(s[3] for s in rsp["steps"]) > 0            # split HxVs ran
    assert all(s[3] > 0 for s in rsp["steps"])            # in every local solve
    assert np.max(np.abs(esp - e64) / np.abs(e64)) < 1e-10
    assert abs(rsp["energies"][-1] - r64["energies"][-1]) < 1e-10 * abs(r64["energies"][-1])
