"""SU(2) in the oracle (CPU): its 6j / 9j symbols against exact rational values,
and its SU(2) HxV (the coeff_HPsi / coeff_tensorProd / coeff_Apair / coeff_buildL /
coeff_buildR families of symmetry/SU2.h:388-519 in the precalc_blockStructure and
contract_L / contract_R loops) pinned by the reference's cross-symmetry check
(programs/test_Heisenberg/test_Heisenberg.cc:373-400): with complete multiplet
bases the SU(2) pivot's spectrum contains the U(1) exact energies."""
import itertools

import numpy as np
import pytest

import oracle
from oracle import ed
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import left_vacuum, right_target


def test_oracle_6j_9j_match_exact_values():
    wig = pytest.importorskip("sympy.physics.wigner")
    from sympy import Rational
    def exact(f, args, **kw):
        try:
            return float(f(*[Rational(a, 2) for a in args], **kw))
        except ValueError:   # arguments that violate a triangle or parity rule: the symbol is 0
            return 0.0

    rng = np.random.default_rng(1)
    checked = nonzero = 0
    for args in itertools.product(range(0, 5), repeat=6):
        if rng.random() > 0.05:
            continue
        e = exact(wig.wigner_6j, args)
        assert abs(oracle.coupling_6j(*args) - e) < 1e-14, (args, e)
        checked += 1
        nonzero += e != 0.0
    # 9j: rows and columns that satisfy the triangle rules (the symbols the builders use)
    tri = [t for t in itertools.product(range(0, 5), repeat=3)
           if (sum(t) % 2 == 0) and abs(t[0] - t[1]) <= t[2] <= t[0] + t[1]]
    n9 = 0
    while n9 < 80:
        r = [tri[i] for i in rng.integers(0, len(tri), size=3)]
        cols = list(zip(*r))
        if not all(c in tri for c in cols):
            continue
        args = [x for row in r for x in row]
        e = exact(wig.wigner_9j, args, prec=40)
        assert abs(oracle.coupling_9j(*args) - e) < 1e-14, (args, e)
        nonzero += e != 0.0
        n9 += 1
    assert checked > 100 and nonzero > 60


def su2_envs(m, mps, lo, hi):
    """oracle environments of an SU(2) (or SU(2)xU(1)) chain: sites < lo and > hi"""
    sym, nq = m.sym, m.sym.nq
    L = left_vacuum(sym)
    for l in range(lo):
        L = oracle.contract_L(nq, L, mps.A[l], m.W[l], mps.A[l], sym=sym)
    R = right_target(sym, mps.Qtot)
    for l in range(m.L - 1, hi, -1):
        R = oracle.contract_R(nq, R, mps.A[l], m.W[l], mps.A[l], sym=sym)
    return L, R


def su2_pivot2(m, mps, site):
    L, R = su2_envs(m, mps, site, site + 1)
    V = contract_two_sites(m.sym, mps.A[site], mps.A[site + 1], m.qloc, m.qloc, m.sym.nq)
    return oracle.OraclePivot(2, m.sym.nq, L, R, V, m.W[site], m.W[site + 1], sym=m.sym), V


def _dense(op, n):
    return np.column_stack([op.hxv(np.eye(n)[:, j]) for j in range(n)])


@pytest.mark.parametrize("qtot,energy", [((1,), -0.75), ((3,), 0.25)])
def test_oracle_su2_dimer(qtot, energy):
    m = models.heisenberg_su2(2)
    mps = RandomMPS(m, qtot, 4, seed=1).canonicalize(0, 1)
    op, V = su2_pivot2(m, mps, 0)
    assert V.data.size == 1
    assert abs(op.hxv(np.ones(1))[0] - energy) < 1e-14


def _heisenberg_ed(L):
    H = models.dense_heisenberg(L)
    M = np.array([sum(1 if ((s >> (L - 1 - j)) & 1) == 0 else -1 for j in range(L)) for s in range(2 ** L)])
    return np.linalg.eigvalsh(H[np.ix_(M == 0, M == 0)])


def test_oracle_su2_heisenberg_pivot2_spectrum():
    """L=8, complete multiplet bases: the S=0 two-site pivot spans every singlet of the
    chain, so its lowest eigenvalue is the chain's ground energy"""
    L = 8
    m = models.heisenberg_su2(L)
    mps = RandomMPS(m, (1,), 64, seed=3).canonicalize(3, 4)
    op, V = su2_pivot2(m, mps, 3)
    ev = np.sort(np.linalg.eigvals(_dense(op, V.data.size)).real)
    e_ed = _heisenberg_ed(L)
    assert abs(ev[0] - e_ed[0]) < 1e-12 * abs(e_ed[0]), (ev[:3], e_ed[:3])


def test_oracle_su2_heisenberg_pivot1_spectrum():
    L = 8
    m = models.heisenberg_su2(L)
    mps = RandomMPS(m, (1,), 64, seed=4).canonicalize(4, 4)
    Lenv, Renv = su2_envs(m, mps, 4, 4)
    V = mps.A[4]
    op = oracle.OraclePivot(1, 1, Lenv, Renv, V, m.W[4], sym=m.sym)
    ev = np.sort(np.linalg.eigvals(_dense(op, V.data.size)).real)
    e_ed = _heisenberg_ed(L)
    assert abs(ev[0] - e_ed[0]) < 1e-12 * abs(e_ed[0]), (ev[:3], e_ed[:3])


def test_oracle_su2xu1_hubbard_pivot2_spectrum():
    """SU(2)xU(1) Hubbard chain L=4 at half filling, complete bases: the singlet two-site
    pivot's lowest eigenvalue is the U(1)xU(1) exact ground energy"""
    L = 4
    m = models.hubbard_su2xu1(L, t=1.0, U=4.0)
    mps = RandomMPS(m, (1, L), 64, seed=7).canonicalize(1, 2)
    op, V = su2_pivot2(m, mps, 1)
    ev = np.sort(np.linalg.eigvals(_dense(op, V.data.size)).real)
    mu1 = models.hubbard_u1xu1(L, 1.0, 4.0)
    H = ed.permute_to_reference(ed.mpo_to_dense(mu1), mu1)
    nm = 2 * L
    mask = []
    for s in range(2 ** nm):
        bits = [(s >> (nm - 1 - j)) & 1 for j in range(nm)]
        mask.append(sum(bits) == L and sum(bits[0::2]) - sum(bits[1::2]) == 0)
    e_ed = ed.ground_energy(H, np.array(mask))
    assert abs(ev[0] - e_ed) < 1e-12 * abs(e_ed), (ev[:3], e_ed)
