"""Pins of the CPU oracle (no GPU): the oracle's HxV / environments against
dense constructions that share no code with it."""
import numpy as np
import pytest

import oracle
from oracle import ed
from vmps_gb300 import models
from vmps_gb300.mps import two_site_layout

from helpers import make_model, pivot1_case, pivot2_case, rel_err


def test_mpo_matches_dense_heisenberg():
    m = models.heisenberg_u1(6)
    H = ed.mpo_to_dense(m)
    Href = models.dense_heisenberg(6)
    assert np.allclose(H, Href, atol=1e-13)


def test_mpo_matches_dense_hubbard():
    m = models.hubbard_u1xu1(3, t=1.0, U=4.0)
    H = ed.permute_to_reference(ed.mpo_to_dense(m), m)
    Href = models.dense_hubbard(3, t=1.0, U=4.0)
    assert np.allclose(H, Href, atol=1e-13)


def test_heisenberg_ground_energy_known_small():
    # two-site XXX: singlet energy -3/4 J
    H = models.dense_heisenberg(2)
    assert abs(np.linalg.eigvalsh(H)[0] + 0.75) < 1e-14


@pytest.mark.parametrize("site", [0, 3, 7])
def test_oracle_hxv1_equals_dense_effective_hamiltonian(site):
    model, mps, Lenv, Renv, W, V = pivot1_case("heis", L=8, D=16, site=site, seed=11)
    H = ed.mpo_to_dense(model)
    P = ed.pivot1_isometry(mps, V, site)
    Heff = P.T @ H @ P
    op = oracle.OraclePivot(1, 1, Lenv, Renv, V, W)
    rng = np.random.default_rng(5)
    for _ in range(3):
        v = rng.standard_normal(V.data.size)
        assert rel_err(op.hxv(v), Heff @ v) < 1e-12


def test_oracle_hxv1_hubbard_dense():
    model, mps, Lenv, Renv, W, V = pivot1_case("hubb", L=4, D=8, site=1, seed=3)
    H = ed.mpo_to_dense(model)
    P = ed.pivot1_isometry(mps, V, 1)
    op = oracle.OraclePivot(1, 2, Lenv, Renv, V, W)
    v = np.random.default_rng(1).standard_normal(V.data.size)
    assert rel_err(op.hxv(v), P.T @ H @ P @ v) < 1e-12


def test_oracle_hxv2_hubbard_dense():
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=4, D=8, site=1, seed=4)
    H = ed.mpo_to_dense(model)
    din = {tuple(mps.A[1].qin[i]): int(mps.A[1].rows[i]) for i in range(mps.A[1].n)}
    dout = {tuple(mps.A[2].qout[i]): int(mps.A[2].cols[i]) for i in range(mps.A[2].n)}
    _, comb = two_site_layout(model.sym, model.qloc, model.qloc, din, dout, 2)
    P = ed.pivot2_isometry(mps, V, comb, 1)
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(2).standard_normal(V.data.size)
    assert rel_err(op.hxv(v), P.T @ H @ P @ v) < 1e-12


def test_oracle_hxv2_heisenberg_dense():
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("heis", L=8, D=16, site=3, seed=9)
    H = ed.mpo_to_dense(model)
    din = {tuple(mps.A[3].qin[i]): int(mps.A[3].rows[i]) for i in range(mps.A[3].n)}
    dout = {tuple(mps.A[4].qout[i]): int(mps.A[4].cols[i]) for i in range(mps.A[4].n)}
    _, comb = two_site_layout(model.sym, model.qloc, model.qloc, din, dout, 1)
    P = ed.pivot2_isometry(mps, V, comb, 3)
    op = oracle.OraclePivot(2, 1, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(3).standard_normal(V.data.size)
    assert rel_err(op.hxv(v), P.T @ H @ P @ v) < 1e-12


def test_oracle_two_site_ground_state_is_exact():
    # with complete bond bases the two-site effective problem contains the ground state
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=4, D=64, site=1, seed=5)
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    n = V.data.size
    Heff = np.column_stack([op.hxv(np.eye(n)[:, j]) for j in range(n)])
    assert np.allclose(Heff, Heff.T, atol=1e-12)
    H = models.dense_hubbard(4, 1.0, 4.0)
    # sector N=4, Sz=0 of the dense reference
    nm = 8
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        N = sum(bits)
        M = sum(bits[0::2]) - sum(bits[1::2])
        mask.append(N == 4 and M == 0)
    e_ed = ed.ground_energy(H, np.array(mask))
    # the random MPS is not orthonormal here in general -> generalized problem; canonical form makes it standard
    e = np.linalg.eigvalsh(Heff)[0]
    assert abs(e - e_ed) < 1e-10 * abs(e_ed)


def test_oracle_pivot0_dense():
    model, Q = make_model("heis", 6)
    from vmps_gb300.mps import RandomMPS
    mps = RandomMPS(model, Q, 8, seed=7).canonicalize(3, 2)   # sites<3 left-, sites>2 right-normalised
    from helpers import oracle_envs
    Lenv, Renv = oracle_envs(model, mps, 3, 2)   # L at bond 3, R at bond 3
    # bond matrix C: diagonal blocks (q,q) of the bond-3 basis
    from vmps_gb300.blocks import Blocks
    ent = [(0, q, q, np.zeros((d, d))) for q, d in sorted(mps.dims[3].items())]
    C = Blocks.from_entries(1, ent)
    H = ed.mpo_to_dense(model)
    UL = ed.left_isometry(mps, 3)
    UR = ed.right_isometry(mps, 3)
    off, cur = {}, 0
    for q, d in sorted(mps.dims[3].items()):
        off[q] = cur
        cur += d
    P = np.zeros((UL.shape[0] * UR.shape[1], C.data.size))
    for b in range(C.n):
        q = tuple(C.qin[b])
        r, c, o = int(C.rows[b]), int(C.cols[b]), int(C.offset[b])
        for j in range(c):
            for i in range(r):
                P[:, o + i + j * r] = np.kron(UL[:, off[q] + i], UR[off[q] + j, :])
    op = oracle.OraclePivot(0, 1, Lenv, Renv, C)
    v = np.random.default_rng(8).standard_normal(C.data.size)
    assert rel_err(op.hxv(v), P.T @ H @ P @ v) < 1e-12


def test_oracle_blas_and_inhouse_agree():
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=6, D=24, site=2, seed=6)
    op = oracle.OraclePivot(2, 2, Lenv, Renv, V, W1, W2)
    v = np.random.default_rng(4).standard_normal(V.data.size)
    a = op.hxv(v)
    lib = oracle.lib()
    lib.oracle_set_blas(b"")
    b = op.hxv(v)
    p = oracle.find_openblas()
    if p:
        lib.oracle_set_blas(p.encode())
    assert rel_err(a, b) < 1e-13


def _env_case(side):
    from helpers import make_model, oracle_envs
    from vmps_gb300.mps import RandomMPS
    model, Q = make_model("hubb", 8)
    mps = RandomMPS(model, Q, 24, seed=13).canonicalize(4, 4)
    Lenv, Renv = oracle_envs(model, mps, 3, 5)
    l = 3 if side == "L" else 5
    E = Lenv if side == "L" else Renv
    # the order map of the auxiliary bond the mode refers to
    return model, mps, E, l


@pytest.mark.parametrize("side", ["L", "R"])
def test_oracle_env_modes_partition_full(side):
    """FIXED_COLS / FIXED_ROWS over all positions partition the W nonzeros, so their
    sum is the FULL contraction; TRIANGULAR(ab) is the sum of FIXED_ROWS (left) or
    FIXED_COLS (right) over the positions it keeps."""
    from helpers import blocks_by_key
    model, mps, E, l = _env_case(side)
    W, A = model.W[l], mps.A[l]
    full = blocks_by_key(oracle.OracleEnv(side, 2, E, A, W, A).run(E, A, A))
    # positions: the incoming (Lold/Rold) and outgoing (Lnew/Rnew) auxiliary bonds
    old_bond, new_bond = (l, l + 1) if side == "L" else (l + 1, l)
    order = dict(model.basis_order_map(old_bond))
    order.update(model.basis_order_map(new_bond))   # same QN/index labels on inner bonds
    npos = len(model.aux[new_bond])
    for mode in ("FIXED_COLS", "FIXED_ROWS"):
        acc = {}
        for ab in range(max(npos, len(model.aux[old_bond]))):
            part = oracle.OracleEnv(side, 2, E, A, W, A, mode=mode, fixed_ab=ab, order=order).run(E, A, A)
            for k, v in blocks_by_key(part).items():
                acc[k] = acc.get(k, 0) + v
        assert set(acc) == set(full)
        for k in full:
            assert np.allclose(acc[k], full[k], atol=1e-12 * max(1.0, np.abs(full[k]).max()))
    # TRIANGULAR keeps a strict subset of FULL
    tri = blocks_by_key(oracle.OracleEnv(side, 2, E, A, W, A, mode="TRIANGULAR", fixed_ab=1, order=order).run(E, A, A))
    assert set(tri) <= set(full)


def test_oracle_dmrg1_heisenberg_matches_ed():
    """single-site DMRG on the oracle with complete bond bases reaches the ED energy"""
    from oracle.dmrg_cpu import dmrg1_cpu
    from vmps_gb300.mps import RandomMPS
    L = 10
    model = models.heisenberg_u1(L)
    mps = RandomMPS(model, (0,), 64, seed=3).canonicalize(0, 0)
    res = dmrg1_cpu(model, mps, n_sweeps=2)
    H = models.dense_heisenberg(L)
    M = np.array([sum(1 if ((s >> (L - 1 - j)) & 1) == 0 else -1 for j in range(L)) for s in range(2 ** L)])
    e_ed = ed.ground_energy(H, M == 0)
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed)


def _hubbard_sector(L, N, M):
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == N and sum(bits[0::2]) - sum(bits[1::2]) == M)
    return np.array(mask)


def test_two_site_split_is_exact_and_orthonormal():
    """split_AA2 without truncation reproduces the two-site tensor; the
    orthonormal site is orthonormal; truncation reports the discarded weight"""
    from vmps_gb300.mps import RandomMPS, contract_two_sites, split_two_site
    m = models.hubbard_u1xu1(8)
    mps = RandomMPS(m, (8, 0), 16, seed=3).canonicalize(3, 4)
    A, B = mps.A[3], mps.A[4]
    V, comb = contract_two_sites(m.sym, A, B, m.qloc, m.qloc, 2, return_basis=True)
    din = {tuple(A.qin[i]): int(A.rows[i]) for i in range(A.n)}
    dout = {tuple(B.qout[i]): int(B.cols[i]) for i in range(B.n)}
    nrm = V.norm()
    for move in ("right", "left"):
        A1, A2, disc, dmid = split_two_site(V, comb, m.qloc, m.qloc, din, dout, 2, Dmax=10 ** 6, move=move)
        assert disc < 1e-14   # eigenvalue round-off of the Gram matrix
        V2 = contract_two_sites(m.sym, A1, A2, m.qloc, m.qloc, 2)
        assert np.linalg.norm(V2.data * nrm - V.data) < 1e-13 * nrm
        O = A1 if move == "right" else A2
        G = {}
        for i in range(O.n):
            q = tuple(O.qout[i]) if move == "right" else tuple(O.qin[i])
            b = O.block(i)
            g = b.T @ b if move == "right" else b @ b.T
            G[q] = G.get(q, 0) + g
        assert max(np.abs(g - np.eye(g.shape[0])).max() for g in G.values()) < 1e-13
    A1, A2, disc, dmid = split_two_site(V, comb, m.qloc, m.qloc, din, dout, 2, Dmax=8, move="right")
    assert sum(dmid.values()) == 8 and 0 < disc < 1
    V2 = contract_two_sites(m.sym, A1, A2, m.qloc, m.qloc, 2)
    assert abs(np.linalg.norm(V2.data) - 1) < 1e-13


def test_oracle_dmrg2_hubbard_matches_ed():
    """two-site DMRG on the oracle grows the bond bases from D=4 to the exact
    state of the L=6 Hubbard chain (DMRG vs ED, programs/test_Hubbard/test_Hubbard.cc:227-300)"""
    from oracle.dmrg_cpu import dmrg2_cpu
    from vmps_gb300.mps import RandomMPS
    L = 6
    model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(model, (L, 0), 4, seed=5).canonicalize(0, 0)
    res = dmrg2_cpu(model, mps, n_sweeps=3, Dmax=64)
    # ED of the MPO (pinned against the fermionic dense Hamiltonian by test_mpo_matches_dense_hubbard)
    H = ed.permute_to_reference(ed.mpo_to_dense(model), model)
    e_ed = ed.ground_energy(H, _hubbard_sector(L, L, 0))
    assert abs(res["energies"][-1] - e_ed) < 1e-10 * abs(e_ed), (res, e_ed)


def test_lattice_mpo_matches_dense_hubbard_cylinder():
    """the long-range lattice MPO (sign strings through intermediate sites) equals the
    second-quantised Hubbard Hamiltonian on a 2x2 cylinder and on the open chain"""
    bonds = models.cylinder_bonds(2, 2)
    m = models.hubbard_u1xu1_lattice(4, bonds, U=8.0)
    H = ed.permute_to_reference(ed.mpo_to_dense(m), m)
    assert np.abs(H - models.dense_hubbard(4, U=8.0, bonds=bonds)).max() < 1e-12
    chain = models.hubbard_u1xu1_lattice(4, [(i, i + 1, 1.0) for i in range(3)], U=4.0)
    assert np.abs(ed.mpo_to_dense(chain) - ed.mpo_to_dense(models.hubbard_u1xu1(4, 1.0, 4.0))).max() < 1e-14
    assert models.hubbard_su2xu1_lattice(64, models.cylinder_bonds(16, 4)).wdim == 10


def test_oracle_lanczos_ground_matches_dense_eigh():
    """the numpy three-term Lanczos of the oracle finds the lowest eigenvalue of a
    dense symmetric matrix to rounding (it is the energy reference of the GPU
    solves at sizes where no dense matrix can be built)"""
    rng = np.random.default_rng(3)
    n = 400
    A = rng.standard_normal((n, n))
    A = (A + A.T) / 2
    e_ref = np.linalg.eigvalsh(A)[0]
    e, steps = oracle.lanczos_ground(lambda v: A @ v, rng.standard_normal(n))
    assert abs(e - e_ref) <= 1e-12 * abs(e_ref), (e, e_ref, steps)
