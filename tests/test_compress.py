"""MPS compression (vmps_gb300.compress) on the host: the two-site variational fit of
sums of operator-MPS products and the Chebyshev recursion of whole MPS, run with the
oracle's contract_L / contract_R and two-site HxV in place of the engine's, against
dense vectors and matrices of small chains (MpsCompressor::prodCompress / polyCompress,
solvers/MpsCompressor.h:961-1564; polyIter, DmrgLinearAlgebra.h:550-566)."""
import numpy as np
import pytest

import oracle
from oracle import ed
from vmps_gb300 import models
from vmps_gb300.compress import Compressor, copy_mps, identity_mpo
from vmps_gb300.mps import RandomMPS


def _oracle_env(side, E, Abra, W, Aket):
    return (oracle.contract_L if side == "L" else oracle.contract_R)(W.nq, E, Abra, W, Aket)


def _oracle_apply2(sym, L, R, W1, W2, V, x):
    return oracle.OraclePivot(2, sym.nq, L, R, V, W1, W2).hxv(x)


def _dense(mps):
    """the state in the kron basis of the MPO's local indices, site 0 most significant"""
    return ed.right_isometry(mps, 0)[0]


def _setup(L, D, seed=3):
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    psi = RandomMPS(model, (L, 0), D, seed=seed)
    comp = Compressor(None, model, env=_oracle_env, apply2=_oracle_apply2)
    return model, psi, comp


def test_identity_mpo_and_overlap():
    model, psi, comp = _setup(4, 16)
    for W in comp.I:
        dense = np.zeros((model.d, model.d))
        for i in range(W.nnz):
            assert W.row[i] == 0 and W.col[i] == 0
            dense[W.s1[i], W.s2[i]] += W.val[i]
        assert np.array_equal(dense, np.eye(model.d))
    phi = RandomMPS(model, (4, 0), 16, seed=8)
    assert comp.overlap(phi, psi) == pytest.approx(float(_dense(phi) @ _dense(psi)), rel=1e-12, abs=1e-14)


def test_fit_of_h_psi_is_exact_with_complete_bases():
    """phi = 0.7 H psi - 0.3 psi; bonds free to grow to the complete bases"""
    model, psi, comp = _setup(6, 64)
    H = ed.mpo_to_dense(model)
    phi = copy_mps(psi)
    disc = comp.fit(phi, [(model.W, psi, 0.7), (comp.I, psi, -0.3)], Dmax=256, sweeps=1)
    ref = 0.7 * H @ _dense(psi) - 0.3 * _dense(psi)
    assert disc < 1e-14
    assert np.linalg.norm(_dense(phi) - ref) < 1e-11 * np.linalg.norm(ref)


def test_truncated_fit_improves_on_its_start_and_keeps_dmax():
    """with Dmax below the target's bond dimension the fit is the best MPS of that size
    it finds: its error is below that of the start (psi itself, rescaled) and each
    bond keeps at most Dmax states"""
    model, psi, comp = _setup(6, 64)
    H = ed.mpo_to_dense(model)
    ref = H @ _dense(psi)
    phi = copy_mps(psi)
    disc = comp.fit(phi, [(model.W, psi, 1.0)], Dmax=12, sweeps=3)
    assert disc > 0
    assert max(sum(d.values()) for d in phi.dims) <= 12
    x = _dense(psi)
    start_err = np.linalg.norm(ref - (x @ ref) / (x @ x) * x)
    err = np.linalg.norm(_dense(phi) - ref)
    assert err < 0.5 * start_err
    # the fitted state is the projection of the target onto its own manifold: <phi|ref> = <phi|phi>
    f = _dense(phi)
    assert f @ ref == pytest.approx(f @ f, rel=1e-9)


def test_mps_chebyshev_moments_equal_dense_recursion():
    model, psi, comp = _setup(4, 16)
    H = ed.mpo_to_dense(model)
    x = _dense(psi)
    w = np.linalg.eigvalsh(H)
    a, b = 1.05 * (w[-1] - w[0]) / 2, (w[-1] + w[0]) / 2
    nmom = 8
    mu, info = comp.chebyshev_moments(psi, nmom, a, b, Dmax=64, sweeps=1)
    t0, t1 = x, (H @ x - b * x) / a
    ref = [x @ t0, x @ t1]
    for _ in range(2, nmom):
        t0, t1 = t1, 2 * (H @ t1 - b * t1) / a - t0
        ref.append(x @ t1)
    assert max(info["discarded"]) < 1e-14
    assert np.allclose(mu, ref, rtol=0, atol=1e-10 * abs(ref[0]))


def _dense_mpo(W, d, end_q):
    """the operator of an MPO site list (boundary states: vacuum index 0 on the left,
    end_q index 0 on the right), kron basis, site 0 most significant"""
    L = len(W)
    keys = [set() for _ in range(L + 1)]
    for l, w in enumerate(W):
        for i in range(w.nnz):
            keys[l].add((tuple(w.qin[i]), w.row[i]))
            keys[l + 1].add((tuple(w.qout[i]), w.col[i]))
    idx = [{k: n for n, k in enumerate(sorted(ks))} for ks in keys]
    vac = tuple(0 for _ in end_q)
    T = np.zeros((1, 1, len(idx[0])))
    T[0, 0, idx[0][(vac, 0)]] = 1.0
    for l, w in enumerate(W):
        M = np.zeros((len(idx[l]), len(idx[l + 1]), d, d))
        for i in range(w.nnz):
            M[idx[l][(tuple(w.qin[i]), w.row[i])], idx[l + 1][(tuple(w.qout[i]), w.col[i])], w.s1[i], w.s2[i]] += w.val[i]
        T = np.einsum("xya,abst->xsytb", T, M)
        T = T.reshape(T.shape[0] * d, T.shape[2] * d, M.shape[1])
    return T[:, :, idx[L][(tuple(end_q), 0)]]


def test_mpo_sum_is_the_operator_sum():
    from vmps_gb300.compress import mpo_sum
    from vmps_gb300.spectral import annihilator, annihilator_mpo
    model = models.hubbard_u1xu1(4, t=1.0, U=4.0)
    I = identity_mpo(model)
    S = mpo_sum([model.W, I], [0.7, -0.3], (0, 0))
    assert np.allclose(_dense_mpo(S, model.d, (0, 0)), 0.7 * ed.mpo_to_dense(model) - 0.3 * np.eye(4 ** 4),
                       rtol=0, atol=1e-13)
    # two charge-changing operators with different auxiliary bases
    dq = annihilator(model, "up")[1]
    A1 = annihilator_mpo(model, [1.0, 0.5, 0.0, -2.0], "up")
    A2 = annihilator_mpo(model, [0.0, 1.0, 3.0, 0.0], "up")
    S = mpo_sum([A1, A2], [2.0, -1.0], dq)
    ref = 2.0 * _dense_mpo(A1, model.d, dq) - _dense_mpo(A2, model.d, dq)
    assert np.linalg.norm(ref) > 1
    assert np.allclose(_dense_mpo(S, model.d, dq), ref, rtol=0, atol=1e-13)


def _charged_start(model, psi, spin, n, comp):
    """c_{k,spin}|psi>, k = pi n/(L+1), fitted from a random MPS of the target charge"""
    from vmps_gb300.spectral import annihilator, annihilator_mpo, standing_wave
    dq = annihilator(model, spin)[1]
    W = annihilator_mpo(model, standing_wave(model.L, n), spin)
    Q = tuple(a + b for a, b in zip(psi.Qtot, dq))
    phi = RandomMPS(model, Q, 64, seed=17)
    disc = comp.fit(phi, [(W, psi, 1.0)], Dmax=256, sweeps=2)
    return phi, disc


@pytest.mark.parametrize("spin,n", [("up", 1), ("dn", 4)])
def test_charge_changing_fit_and_its_moments(spin, n):
    """c_{k,s}|psi> as an MPS of charge Qtot + dq (the right boundary of its environments
    carries dq), then the MPS Chebyshev moments in that sector, against dense c_k and the
    dense recursion"""
    from test_spectral import _dense_c
    from vmps_gb300.spectral import standing_wave
    model, psi, comp = _setup(6, 64)
    phi, disc = _charged_start(model, psi, spin, n, comp)
    ref = _dense_c(model, standing_wave(6, n), spin) @ _dense(psi)
    assert disc < 1e-14
    assert np.linalg.norm(_dense(phi) - ref) < 1e-11 * np.linalg.norm(ref)
    H = ed.mpo_to_dense(model)
    a, b = 1.01 * np.abs(H).sum(axis=1).max(), 0.0     # the spectrum lies inside [-a, a] (Gershgorin)
    mu, _ = comp.chebyshev_moments(phi, 6, a, b, Dmax=256, sweeps=1)
    t0, t1 = ref, (H @ ref - b * ref) / a
    mref = [ref @ t0, ref @ t1]
    for _ in range(2, 6):
        t0, t1 = t1, 2 * (H @ t1 - b * t1) / a - t0
        mref.append(ref @ t1)
    assert np.allclose(mu, mref, rtol=0, atol=1e-10 * mref[0])


# ---- SU(2): reduced tensors; checked against the two-site pivot of the same state, whose
# space is the whole sector when the bases are complete (weighted dots, coeff_dot = q)

def _su2_pivot_reference(model, psi, l):
    """(V, Heff(x), dot(x, y)) of psi's two-site pivot (l, l+1) on the oracle"""
    import copy
    from vmps_gb300.pivot import left_vacuum, right_target
    from vmps_gb300.su2 import contract_two_sites_su2
    sym, nq = model.sym, model.sym.nq
    m = copy.deepcopy(psi).canonicalize(l, l + 1)
    Lenv = left_vacuum(sym)
    for j in range(l):
        Lenv = oracle.contract_L(nq, Lenv, m.A[j], model.W[j], m.A[j], sym=sym)
    Renv = right_target(sym, m.Qtot)
    for j in range(model.L - 1, l + 1, -1):
        Renv = oracle.contract_R(nq, Renv, m.A[j], model.W[j], m.A[j], sym=sym)
    V, _ = contract_two_sites_su2(sym, m.A[l], m.A[l + 1], model.qloc, model.qloc)
    piv = oracle.OraclePivot(2, nq, Lenv, Renv, V, model.W[l], model.W[l + 1], sym=sym)
    w = np.concatenate([np.full(int(V.rows[b] * V.cols[b]), sym.dot_weight(tuple(V.qout[b]))) for b in range(V.n)])
    order = np.concatenate([np.arange(V.offset[b], V.offset[b] + V.rows[b] * V.cols[b]) for b in range(V.n)])
    wt = np.zeros(V.data.size)
    wt[order] = w
    return V.data.copy(), piv.hxv, (lambda x, y: float(np.sum(wt * x * y)))


def _su2_compressor(model):
    sym = model.sym
    env = lambda side, E, Abra, W, Aket: (oracle.contract_L if side == "L" else oracle.contract_R)(
        W.nq, E, Abra, W, Aket, sym=sym)
    apply2 = lambda tsym, Le, Re, W1, W2, V, x: oracle.OraclePivot(2, tsym.nq, Le, Re, V, W1, W2, sym=tsym).hxv(x)
    return Compressor(None, model, env=env, apply2=apply2)


@pytest.mark.parametrize("kind", ["heisenberg_su2", "hubbard_su2xu1"])
def test_su2_fit_and_moments_equal_the_complete_pivot(kind):
    if kind == "heisenberg_su2":
        L, l = 10, 4
        model, Q = models.heisenberg_su2(L), (1,)
    else:
        L, l = 6, 2
        model, Q = models.hubbard_su2xu1_lattice(L, [(i, i + 1, 1.0) for i in range(L - 1)], U=4.0), (1, L)
    psi = RandomMPS(model, Q, 64, seed=7)
    comp = _su2_compressor(model)
    v, heff, dot = _su2_pivot_reference(model, psi, l)
    hv = heff(v)
    # the norm and energy of psi, and the fit of H psi
    assert comp.overlap(psi, psi) == pytest.approx(dot(v, v), rel=1e-11)
    phi = copy_mps(psi)
    disc = comp.fit(phi, [(model.W, psi, 1.0)], Dmax=1000, sweeps=1)
    assert disc < 1e-14
    assert comp.overlap(phi, phi) == pytest.approx(dot(hv, hv), rel=1e-10)
    assert comp.overlap(psi, phi) == pytest.approx(dot(v, hv), rel=1e-10)
    # Chebyshev moments of whole MPS against the pivot's recursion
    a, b = (8.0, -1.0) if kind == "heisenberg_su2" else (20.0, 2.0)
    mu, _ = comp.chebyshev_moments(psi, 8, a, b, Dmax=1000, sweeps=1)
    t0, t1 = v, (heff(v) - b * v) / a
    ref = [dot(v, t0), dot(v, t1)]
    for _ in range(2, 8):
        t0, t1 = t1, 2 * (heff(t1) - b * t1) / a - t0
        ref.append(dot(v, t1))
    assert np.allclose(mu, ref, rtol=0, atol=1e-10 * abs(ref[0]))


@pytest.mark.parametrize("kind", ["hubbard_u1xu1", "heisenberg_su2"])
def test_truncated_fit_is_a_projection(kind):
    """with fewer states than the target needs, the fit is the projection of H psi onto the
    fitted MPS's own tangent: <phi|H|psi> = <phi|phi> (<phi|H|psi> by contract_L through
    the chain), every bond keeps at most Dmax states (multiplets for SU(2))"""
    if kind == "heisenberg_su2":
        model = models.heisenberg_su2(12)
        psi = RandomMPS(model, (1,), 32, seed=9)
        comp = _su2_compressor(model)
        Dmax = 6
    else:
        model, psi, comp = _setup(6, 64)
        Dmax = 12
    phi = copy_mps(psi)
    disc = comp.fit(phi, [(model.W, psi, 1.0)], Dmax=Dmax, sweeps=3)
    assert disc > 0
    assert max(sum(d.values()) for d in phi.dims) <= Dmax
    assert comp.matrix_element(phi, model.W, psi) == pytest.approx(comp.overlap(phi, phi), rel=1e-9)


def test_su2_fits_refuse_operators_that_change_the_total_quantum_number():
    model = models.heisenberg_su2(6)
    psi = RandomMPS(model, (1,), 16, seed=1)
    phi = RandomMPS(model, (3,), 16, seed=2)
    comp = _su2_compressor(model)
    with pytest.raises(ValueError):
        comp.fit(phi, [(model.W, psi, 1.0)], Dmax=16, sweeps=1)


def test_mpo_sum_with_su2_vacuum():
    """the summed MPO of H and the identity on an SU(2) chain keeps the vacuum (q = 1)
    boundary states: <psi|(H + 2)|psi> = <psi|H|psi> + 2 <psi|psi>"""
    from vmps_gb300.compress import mpo_sum
    model = models.heisenberg_su2(8)
    psi = RandomMPS(model, (1,), 32, seed=4)
    comp = _su2_compressor(model)
    S = mpo_sum([model.W, comp.I], [1.0, 2.0], (1,), model.sym.vacuum())
    lhs = comp.matrix_element(psi, S, psi)
    rhs = comp.matrix_element(psi, model.W, psi) + 2.0 * comp.overlap(psi, psi)
    assert lhs == pytest.approx(rhs, rel=1e-12)


# ---- the MpsCompressor operations with their stopping rule (|phi - T|^2 <= tol)

def _sz_mpo(model, j):
    from vmps_gb300.models import ChainModel
    sz = np.diag([0.5 * q[1] for q in model.qloc])
    onehot = [1.0 if i == j else 0.0 for i in range(model.L)]
    return ChainModel(model.sym, model.L, model.qloc, {"Sz": (sz, (0, 0))}, [], [("Sz", 1.0)], site_coef=onehot).W


def test_mpo_adjoint_and_product_are_the_dense_operators():
    from vmps_gb300.compress import mpo_adjoint, mpo_product
    from vmps_gb300.spectral import annihilator_mpo
    model = models.hubbard_u1xu1(4, t=1.0, U=4.0)
    H = ed.mpo_to_dense(model)
    S = _sz_mpo(model, 1)
    dS = _dense_mpo(S, model.d, (0, 0))
    assert np.allclose(_dense_mpo(mpo_product(model.W, model.W), model.d, (0, 0)), H @ H, rtol=0, atol=1e-12)
    assert np.allclose(_dense_mpo(mpo_product(model.W, S), model.d, (0, 0)), H @ dS, rtol=0, atol=1e-12)
    assert np.allclose(_dense_mpo(mpo_adjoint(model.W), model.d, (0, 0)), H.T, rtol=0, atol=1e-13)
    with pytest.raises(ValueError):   # two auxiliary states at the end (the finished and the pending operator)
        mpo_product(annihilator_mpo(model, [1.0, 0.0, 0.0, 0.0], "up"), model.W)


def test_state_compress_reports_the_distance():
    model, psi, comp = _setup(6, 64)
    phi, info = comp.state_compress(psi, Dmax=6, tol=0.0, max_sweeps=3)
    d = _dense(phi) - _dense(psi)
    assert info["sweeps"] == 3 and info["discarded"] > 0
    assert info["sqdist"] == pytest.approx(float(d @ d), rel=1e-8)
    assert max(sum(q.values()) for q in phi.dims) <= 6
    # a loose tolerance stops after min_sweeps
    _, info2 = comp.state_compress(psi, Dmax=6, tol=1e9, max_sweeps=5, min_sweeps=2)
    assert info2["sweeps"] == 2


def test_prod_poly_and_lincombo_compress_against_dense():
    model, psi, comp = _setup(6, 64)
    H = ed.mpo_to_dense(model)
    x = _dense(psi)
    # W psi, converged (bases complete) and truncated
    phi, info = comp.prod_compress(model.W, psi, Dmax=1000, tol=1e-18, max_sweeps=2)
    assert info["target_norm2"] == pytest.approx(float((H @ x) @ (H @ x)), rel=1e-11)
    assert np.linalg.norm(_dense(phi) - H @ x) < 1e-10 * np.linalg.norm(H @ x)
    phi, info = comp.prod_compress(model.W, psi, Dmax=10, tol=0.0, max_sweeps=2)
    d = _dense(phi) - H @ x
    assert info["sqdist"] == pytest.approx(float(d @ d), rel=1e-6)
    # H psi1 - b psi2
    psi2 = RandomMPS(model, (6, 0), 64, seed=12)
    y = _dense(psi2)
    phi, info = comp.poly_compress(model.W, psi, 0.7, psi2, Dmax=12, tol=0.0, max_sweeps=2)
    t = H @ x - 0.7 * y
    assert info["target_norm2"] == pytest.approx(float(t @ t), rel=1e-11)
    d = _dense(phi) - t
    assert info["sqdist"] == pytest.approx(float(d @ d), rel=1e-6)
    # 0.5 psi1 + 2 psi2 - psi3
    psi3 = RandomMPS(model, (6, 0), 64, seed=13)
    z = _dense(psi3)
    phi, info = comp.lincombo_compress([psi, psi2, psi3], [0.5, 2.0, -1.0], Dmax=1000, tol=1e-18, max_sweeps=2)
    t = 0.5 * x + 2.0 * y - z
    assert np.linalg.norm(_dense(phi) - t) < 1e-10 * np.linalg.norm(t)
    assert abs(info["sqdist"]) < 1e-9 * float(t @ t)


def test_edge_cases_two_sites_and_one_state():
    """a two-site chain (one two-site step per half sweep) fits exactly; Dmax = 1 keeps one
    state per bond and still returns the projection of the target onto that manifold"""
    model, psi, comp = _setup(2, 16)
    H = ed.mpo_to_dense(model)
    x = _dense(psi)
    phi = copy_mps(psi)
    comp.fit(phi, [(model.W, psi, 1.0)], Dmax=16, sweeps=1)
    assert np.linalg.norm(_dense(phi) - H @ x) < 1e-12 * np.linalg.norm(H @ x)
    model, psi, comp = _setup(6, 64)
    phi = copy_mps(psi)
    disc = comp.fit(phi, [(model.W, psi, 1.0)], Dmax=1, sweeps=2)
    assert disc > 0 and max(sum(d.values()) for d in phi.dims) == 1
    f, t = _dense(phi), ed.mpo_to_dense(model) @ _dense(psi)
    assert f @ t == pytest.approx(f @ f, rel=1e-9)
