"""MPS compression on the engine (vmps_gb300.compress): the two-site fit of sums of
operator-MPS products and the Chebyshev recursion of whole MPS (MpsCompressor::
prodCompress / polyCompress, solvers/MpsCompressor.h:961-1564; polyIter,
DmrgLinearAlgebra.h:550-566), with contract_L / contract_R, the tagged two-site
HxV, the two-site contraction and the split on the GPU:

* on a chain with complete bases (L=6 Hubbard) the fit of 0.7 H psi - 0.3 psi and the
  moments of the MPS recursion equal the dense vectors and the dense recursion (FP64
  to 1e-11 / 1e-10; split precision within 1e-5 of the first moment);
* on a longer chain (L=10, bond dimension 24, no truncation) the engine's fit equals
  the same sweeps run on the oracle's contractions to 1e-10;
* SU(2) and SU(2) x U(1) reduced MPS: the fit of H psi and the moments equal the two-site
  pivot of psi on the oracle when the bases are complete."""
import numpy as np
import pytest

from oracle import ed
from vmps_gb300 import models
from vmps_gb300.compress import Compressor, copy_mps
from vmps_gb300.mps import RandomMPS

from test_compress import _dense, _oracle_apply2, _oracle_env

pytestmark = pytest.mark.gpu


def test_engine_fit_equals_dense(gpu_ctx):
    model = models.hubbard_u1xu1(6, t=1.0, U=4.0)
    psi = RandomMPS(model, (6, 0), 64, seed=3)
    comp = Compressor(gpu_ctx, model)
    H = ed.mpo_to_dense(model)
    phi = copy_mps(psi)
    disc = comp.fit(phi, [(model.W, psi, 0.7), (comp.I, psi, -0.3)], Dmax=256, sweeps=1)
    ref = 0.7 * H @ _dense(psi) - 0.3 * _dense(psi)
    assert disc < 1e-14
    assert np.linalg.norm(_dense(phi) - ref) < 1e-11 * np.linalg.norm(ref)
    assert comp.overlap(phi, phi) == pytest.approx(ref @ ref, rel=1e-11)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("bf16x3", 1e-5)])
def test_engine_mps_chebyshev_equals_dense(gpu_ctx, precision, tol):
    model = models.hubbard_u1xu1(6, t=1.0, U=4.0)
    psi = RandomMPS(model, (6, 0), 64, seed=5)
    H = ed.mpo_to_dense(model)
    x = _dense(psi)
    w = np.linalg.eigvalsh(H)
    a, b = 1.05 * (w[-1] - w[0]) / 2, (w[-1] + w[0]) / 2
    nmom = 10
    comp = Compressor(gpu_ctx, model, precision=precision)
    mu, info = comp.chebyshev_moments(psi, nmom, a, b, Dmax=256, sweeps=1)
    t0, t1 = x, (H @ x - b * x) / a
    ref = [x @ t0, x @ t1]
    for _ in range(2, nmom):
        t0, t1 = t1, 2 * (H @ t1 - b * t1) / a - t0
        ref.append(x @ t1)
    assert np.max(np.abs(mu - ref)) < tol * abs(ref[0])


def test_engine_fit_equals_oracle_sweeps(gpu_ctx):
    L = 10
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    psi = RandomMPS(model, (L, 0), 24, seed=9)
    terms = lambda c: [(model.W, psi, 0.7), (c.I, psi, -0.3)]
    dev = Compressor(gpu_ctx, model)
    host = Compressor(None, model, env=_oracle_env, apply2=_oracle_apply2)
    g, h = copy_mps(psi), copy_mps(psi)
    dev.fit(g, terms(dev), Dmax=10 ** 6, sweeps=2)
    host.fit(h, terms(host), Dmax=10 ** 6, sweeps=2)
    assert [sum(d.values()) for d in g.dims] == [sum(d.values()) for d in h.dims]
    x, y = _dense(g), _dense(h)
    assert np.linalg.norm(x - y) < 1e-10 * np.linalg.norm(y)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("bf16x3", 1e-5)])
def test_engine_charge_changing_start_and_moments(gpu_ctx, precision, tol):
    """c_{k,up}|psi> fitted as an MPS of charge Qtot + dq on the engine, then its MPS
    Chebyshev moments, against dense c_k and the dense recursion"""
    from test_compress import _charged_start
    from test_spectral import _dense_c
    from vmps_gb300.spectral import standing_wave
    model = models.hubbard_u1xu1(6, t=1.0, U=4.0)
    psi = RandomMPS(model, (6, 0), 64, seed=3)
    comp = Compressor(gpu_ctx, model, precision=precision)
    phi, disc = _charged_start(model, psi, "up", 2, comp)
    ref = _dense_c(model, standing_wave(6, 2), "up") @ _dense(psi)
    assert np.linalg.norm(_dense(phi) - ref) < max(1e-11, tol) * np.linalg.norm(ref)
    H = ed.mpo_to_dense(model)
    a, b = 1.01 * np.abs(H).sum(axis=1).max(), 0.0
    mu, _ = comp.chebyshev_moments(phi, 8, a, b, Dmax=256, sweeps=1)
    t0, t1 = ref, H @ ref / a
    mref = [ref @ t0, ref @ t1]
    for _ in range(2, 8):
        t0, t1 = t1, 2 * (H @ t1) / a - t0
        mref.append(ref @ t1)
    assert np.max(np.abs(mu - mref)) < tol * mref[0]


@pytest.mark.parametrize("kind", ["heisenberg_su2", "hubbard_su2xu1"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("bf16x3", 1e-5)])
def test_engine_su2_fit_and_moments_equal_the_complete_pivot(gpu_ctx, kind, precision, tol):
    """SU(2) reduced MPS on the engine (SU(2) environments, tagged SU(2) x U(1) pivots,
    the SU(2) two-site contraction on the GPU): with complete bases the fit of H psi and
    the MPS Chebyshev moments equal the two-site pivot of psi on the oracle"""
    from test_compress import _su2_pivot_reference
    if kind == "heisenberg_su2":
        L, l = 10, 4
        model, Q = models.heisenberg_su2(L), (1,)
        a, b = 8.0, -1.0
    else:
        L, l = 6, 2
        model, Q = models.hubbard_su2xu1_lattice(L, [(i, i + 1, 1.0) for i in range(L - 1)], U=4.0), (1, L)
        a, b = 20.0, 2.0
    psi = RandomMPS(model, Q, 64, seed=7)
    comp = Compressor(gpu_ctx, model, precision=precision)
    v, heff, dot = _su2_pivot_reference(model, psi, l)
    hv = heff(v)
    phi = copy_mps(psi)
    comp.fit(phi, [(model.W, psi, 1.0)], Dmax=1000, sweeps=1)
    assert abs(comp.overlap(phi, phi) - dot(hv, hv)) < max(tol, 1e-10) * dot(hv, hv)
    assert abs(comp.overlap(psi, phi) - dot(v, hv)) < max(tol, 1e-10) * abs(dot(hv, hv)) ** 0.5 * dot(v, v) ** 0.5
    mu, _ = comp.chebyshev_moments(psi, 8, a, b, Dmax=1000, sweeps=1)
    t0, t1 = v, (heff(v) - b * v) / a
    ref = [dot(v, t0), dot(v, t1)]
    for _ in range(2, 8):
        t0, t1 = t1, 2 * (heff(t1) - b * t1) / a - t0
        ref.append(dot(v, t1))
    assert np.max(np.abs(mu - ref)) < tol * abs(ref[0])
