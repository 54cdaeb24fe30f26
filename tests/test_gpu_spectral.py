"""Config C5 end to end on a chain small enough for exact diagonalisation (L=6
Hubbard, pivot bases complete, so the pivot spaces are whole sectors):

* the engine's P c_{k,s}|0> (contract_L / contract_R and the tagged two-site step on
  the GPU) equals the same construction on the oracle and the dense c_{k,s}|0>;
* per-part Chebyshev moments of the union of the two spin sectors, FP64 and split
  precision, equal the dense recursion mu_n = <c_k 0| T_n((H - b)/a) |c_k 0> of the
  full Hamiltonian (the reference's Chebyshev expansion, polyIter,
  DmrgLinearAlgebra.h:550-566), FP64 to 1e-10, split within 1e-4."""
import copy

import numpy as np
import pytest

import oracle
from oracle import ed
from vmps_gb300 import models
from vmps_gb300.dmrg import dmrg2
from vmps_gb300.mps import RandomMPS, two_site_layout
from vmps_gb300.spectral import SpectralPivot, annihilator, standing_wave

from test_spectral import _dense_c, _oracle_apply2, _oracle_env, _relabelled

pytestmark = pytest.mark.gpu


def _ground_state(gpu_ctx, L):
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 64, seed=21).canonicalize(0, 0)
    dmrg2(gpu_ctx, model, mps, n_sweeps=4, Dmax=64, precision="fp64")
    return model, mps


def test_engine_start_vectors_and_union_moments(gpu_ctx):
    L, l = 6, 2
    model, mps = _ground_state(gpu_ctx, L)
    mps = copy.deepcopy(mps)
    mps.canonicalize(l, l + 1)
    assert mps.bond_dim(l) == 16 and mps.bond_dim(l + 2) == 16
    sp = SpectralPivot(gpu_ctx, model, mps, l)
    sp_o = SpectralPivot(None, model, mps, l, env=_oracle_env, apply2=_oracle_apply2)
    _, comb = two_site_layout(model.sym, model.qloc, model.qloc, dict(mps.dims[l]), dict(mps.dims[l + 2]), 2)
    psi = ed.pivot2_isometry(mps, sp.V0, comb, l) @ sp.V0.data
    H = ed.mpo_to_dense(model)
    e0 = float(psi @ H @ psi) / float(psi @ psi)
    ns = [1, 2, 4, 6]
    X, dense = {}, {}
    for spin in ("up", "dn"):
        X[spin] = sp.start_vectors(ns, spin)
        Xo = sp_o.start_vectors(ns, spin)
        assert np.abs(X[spin] - Xo).max() < 1e-12
        dq = annihilator(model, spin)[1]
        Pb = ed.pivot2_isometry(_relabelled(mps, l, dq), sp.sector(spin)[2], comb, l)
        dense[spin] = []
        for i, n in enumerate(ns):
            ref = _dense_c(model, standing_wave(L, n), spin) @ psi
            assert np.linalg.norm(Pb @ X[spin][i] - ref) < 1e-11 * np.linalg.norm(ref)
            dense[spin].append(ref)
    # the union of the two sectors: row i holds momentum ns[i] of both spins
    U = sp.union()
    Xu = U.join([X["up"], X["dn"]])
    lo, hi = U.H.spectral_bounds(np.random.default_rng(3).standard_normal(U.H.dim), iters=120)
    ev = np.linalg.eigvalsh(H)
    assert lo >= ev[0] - 1e-8 and hi <= ev[-1] + 1e-8
    a, b = (hi - lo) / 2 / 0.98, (hi + lo) / 2
    nmom = 60
    mu64, _ = U.chebyshev_moments(Xu, nmom, a, b, "fp64")
    musp, _ = U.chebyshev_moments(Xu, nmom, a, b, "bf16x3")
    Ht = (H - b * np.eye(len(H))) / a
    for p, spin in enumerate(("up", "dn")):
        for i in range(len(ns)):
            t0 = dense[spin][i]
            ref, tp, tc = np.zeros(nmom), None, t0.copy()
            for m in range(nmom):          # T_0 t, T_1 t, ... by the three-term recurrence
                ref[m] = t0 @ tc
                tn = Ht @ tc if m == 0 else 2 * Ht @ tc - tp
                tp, tc = tc, tn
            scale = max(1.0, abs(ref[0]))
            assert np.abs(mu64[i, p] - ref).max() < 1e-10 * scale, (spin, ns[i])
            assert np.abs(musp[i, p] - ref).max() < 1e-4 * scale, (spin, ns[i])
    assert e0 < 0
    U.close()
