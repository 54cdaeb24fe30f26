"""Make the golden fixtures of tests/golden/ (run from the repository root:
`python tests/golden/make_golden.py`).

Each fixture holds the complete inputs of one small, seeded case of the hot
path -- environments, MPO sites, the PivotVector layout and an input vector --
and the CPU oracle's output for it (the oracle restates the reference loops of
pivot/DmrgPivotMatrix{0,1,2}.h and tensors/DmrgContractions.h).  The tests
re-run the oracle on the stored inputs (pinning the oracle against drift) and
run the GPU engine on them (parity against fixed numbers)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from helpers import blocks_to_npz, mpo_to_npz, oracle_envs, pivot1_case, pivot2_case, make_model  # noqa: E402


def save(name, arrays):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print("wrote", name, sum(a.nbytes for a in arrays.values()), "bytes")


def pivot1(name, kind, L, D, site, seed):
    model, mps, Lenv, Renv, W, V = pivot1_case(kind, L=L, D=D, site=site, seed=seed)
    v = np.random.default_rng(seed + 100).standard_normal(V.data.size)
    out = oracle.OraclePivot(1, model.sym.nq, Lenv, Renv, V, W).hxv(v)
    a = {"kind": np.array([1]), "v": v, "out": out}
    blocks_to_npz("L", Lenv, a); blocks_to_npz("R", Renv, a); blocks_to_npz("V", V, a); mpo_to_npz("W", W, a)
    save(name, a)


def pivot2(name, kind, L, D, site, seed, profile):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case(kind, L=L, D=D, site=site, seed=seed, profile=profile)
    v = np.random.default_rng(seed + 100).standard_normal(V.data.size)
    out = oracle.OraclePivot(2, model.sym.nq, Lenv, Renv, V, W1, W2).hxv(v)
    a = {"kind": np.array([2]), "v": v, "out": out}
    blocks_to_npz("L", Lenv, a); blocks_to_npz("R", Renv, a); blocks_to_npz("V", V, a)
    mpo_to_npz("W", W1, a); mpo_to_npz("W2", W2, a)
    save(name, a)


def pivot0(name, seed):
    from vmps_gb300.blocks import Blocks
    from vmps_gb300.mps import RandomMPS
    model, Q = make_model("hubb", 8)
    mps = RandomMPS(model, Q, 32, seed=seed).canonicalize(4, 3)
    Lenv, Renv = oracle_envs(model, mps, 4, 3)
    C = Blocks.from_entries(2, [(0, q, q, np.zeros((d, d))) for q, d in sorted(mps.dims[4].items())])
    v = np.random.default_rng(seed + 100).standard_normal(C.data.size)
    out = oracle.OraclePivot(0, 2, Lenv, Renv, C).hxv(v)
    a = {"kind": np.array([0]), "v": v, "out": out}
    blocks_to_npz("L", Lenv, a); blocks_to_npz("R", Renv, a); blocks_to_npz("V", C, a)
    save(name, a)


def env(name, kind, L, D, seed):
    from vmps_gb300.mps import RandomMPS
    model, Q = make_model(kind, L)
    mps = RandomMPS(model, Q, D, seed=seed, profile="gaussian").canonicalize(L // 2, L // 2)
    Lenv, Renv = oracle_envs(model, mps, L // 2 - 1, L // 2 + 1)
    nq = model.sym.nq
    a = {}
    for side, E, l in (("L", Lenv, L // 2 - 1), ("R", Renv, L // 2 + 1)):
        res = oracle.OracleEnv(side, nq, E, mps.A[l], model.W[l], mps.A[l]).run(E, mps.A[l], mps.A[l])
        blocks_to_npz(side + "old", E, a); blocks_to_npz(side + "A", mps.A[l], a)
        mpo_to_npz(side + "W", model.W[l], a); blocks_to_npz(side + "new", res, a)
    save(name, a)


if __name__ == "__main__":
    oracle.build()
    pivot1("pivot1_heisenberg_L8_D16", "heis", 8, 16, 3, 21)
    pivot1("pivot1_hubbard_L8_D32", "hubb", 8, 32, 3, 21)
    pivot2("pivot2_hubbard_L6_D24", "hubb", 6, 24, 2, 22, "even")
    pivot0("pivot0_hubbard_L8_D32", 5)
    env("env_hubbard_L10_D48", "hubb", 10, 48, 6)
