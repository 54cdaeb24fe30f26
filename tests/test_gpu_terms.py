"""GPU tests of the two PivotMatrix features beyond a single term: several terms
(PivotMatrix1/2::Terms, summed by HxV, pivot/DmrgPivotMatrix1.h:273-287) and the
excited-state projector (A0proj, Epenalty; :64-68, :304-331), against the
oracle's restatement of the same loops.

Tolerances as in test_gpu_parity: FP64 1e-12, BF16x3 2e-4 relative; energies
1e-10 relative."""
import numpy as np
import pytest

import oracle
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import PivotMatrix1, PivotMatrix2

from helpers import oracle_envs, rel_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_SPLIT = 2e-4


def _two_term_case(L=12, D=48, site=5, two_site=True):
    """two terms with the same bond bases: Hubbard U=4 environments of one seeded MPS
    and Hubbard U=8 environments of another; the pivot vector layout is shared"""
    terms, V = [], None
    for U, seed in ((4.0, 31), (8.0, 32)):
        model = models.hubbard_u1xu1(L, t=1.0, U=U)
        hi = site + 1 if two_site else site
        mps = RandomMPS(model, (L, 0), D, seed=seed, profile="gaussian").canonicalize(site, hi)
        Lenv, Renv = oracle_envs(model, mps, site, hi)
        if two_site:
            terms.append((Lenv, Renv, model.W[site], model.W[site + 1]))
            if V is None:
                V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, 2)
        else:
            terms.append((Lenv, Renv, model.W[site]))
            if V is None:
                V = mps.A[site]
    return model.sym, terms, V


@pytest.mark.parametrize("two_site", [False, True])
def test_two_term_pivot_matches_oracle(gpu_ctx, two_site):
    sym, terms, V = _two_term_case(two_site=two_site)
    cls = PivotMatrix2 if two_site else PivotMatrix1
    H = cls.from_terms(gpu_ctx, sym, terms, V)
    ref_op = oracle.OracleTerms(2 if two_site else 1, 2, terms, V)
    v = np.random.default_rng(4).standard_normal(V.data.size)
    ref = ref_op.hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT
    # each term alone, through the single-term entry point, sums to the same
    parts = [cls(gpu_ctx, sym, *t, V) for t in terms]
    tot = sum(P.apply(v, "fp64") for P in parts)
    assert rel_err(tot, ref) < TOL_FP64
    for P in parts:
        P.close()
    H.close()


def test_projector_hxv_matches_oracle(gpu_ctx):
    sym, terms, V = _two_term_case(two_site=True)
    H = PivotMatrix2.from_terms(gpu_ctx, sym, terms[:1], V)
    rng = np.random.default_rng(5)
    A0 = rng.standard_normal((2, V.data.size))
    A0 /= np.linalg.norm(A0, axis=1, keepdims=True)
    H.set_projector(A0, 7.5)
    ref_op = oracle.OracleTerms(2, 2, terms[:1], V, A0proj=A0, Epenalty=7.5)
    v = rng.standard_normal(V.data.size)
    ref = ref_op.hxv(v)
    assert rel_err(H.apply(v, "fp64"), ref) < TOL_FP64
    assert rel_err(H.apply(v, "bf16x3"), ref) < TOL_SPLIT
    # several right-hand sides in one call: each equals its single-vector HxV
    vs = rng.standard_normal((3, V.data.size))
    for prec, tol in (("fp64", TOL_FP64), ("bf16x3", TOL_SPLIT)):
        outs = H.apply_multi(vs, prec)
        for k in range(3):
            assert rel_err(outs[k], ref_op.hxv(vs[k])) < tol
    # removing the projector gives the plain HxV back
    H.set_projector([], 0.0)
    assert rel_err(H.apply(v, "fp64"), oracle.OracleTerms(2, 2, terms[:1], V).hxv(v)) < TOL_FP64
    H.close()


def test_excited_state_by_projector_equals_ed(gpu_ctx):
    """Heisenberg L=8 with complete bond bases: the two-site pivot in the middle spans
    the whole Sz=0 space, so its ground state is the chain's.  With that state as
    A0proj and a penalty above the spectrum's width, the projected pivot's ground
    state is the first excited state of the sector, as DmrgSolver's excited-state
    runs use it.  Energies from FP64 and from split precision + refinement
    against exact diagonalisation and against the oracle's Lanczos."""
    L = 8
    model = models.heisenberg_u1(L)
    site = 3
    mps = RandomMPS(model, (0,), 64, seed=9).canonicalize(site, site + 1)
    Lenv, Renv = oracle_envs(model, mps, site, site + 1)
    V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, 1)
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, model.W[site], model.W[site + 1], V)
    Hd = models.dense_heisenberg(L)
    M = np.array([sum(1 if ((s >> (L - 1 - j)) & 1) == 0 else -1 for j in range(L)) for s in range(2 ** L)])
    evals = np.linalg.eigvalsh(Hd[np.ix_(M == 0, M == 0)])
    v0 = np.random.default_rng(3).standard_normal(V.data.size)
    tol = dict(max_iter=200, tol_eigval=1e-13, tol_state=1e-8)
    e0, x0, _ = H.lanczos(v0, "fp64", **tol)
    assert abs(e0 - evals[0]) <= 1e-10 * abs(evals[0])
    x0 = x0 / np.linalg.norm(x0)
    Epen = 10.0
    H.set_projector([x0], Epen)
    op = oracle.OracleTerms(2, 1, [(Lenv, Renv, model.W[site], model.W[site + 1])], V, A0proj=[x0], Epenalty=Epen)
    e1_or, _ = oracle.lanczos_ground(op.hxv, v0)
    e1, _, _ = H.lanczos(v0, "fp64", **tol)
    e1s, _, st = H.lanczos(v0, "bf16x3", refine_iters=10, **tol)
    assert abs(e1_or - evals[1]) <= 1e-10 * abs(evals[1]), (e1_or, evals[:2])
    assert abs(e1 - evals[1]) <= 1e-10 * abs(evals[1]), (e1, evals[:2])
    assert abs(e1s - evals[1]) <= 1e-10 * abs(evals[1]), (e1s, evals[:2], st)
    H.close()
