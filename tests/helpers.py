"""Workload builders shared by the tests (small sizes, seeded)."""
from __future__ import annotations

import numpy as np

import oracle
from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites
from vmps_gb300.pivot import left_vacuum, right_target


def make_model(kind, L):
    if kind == "heis":
        return models.heisenberg_u1(L), (0,)
    if kind == "hubb":
        return models.hubbard_u1xu1(L, t=1.0, U=4.0), (L, 0)
    raise ValueError(kind)


def oracle_envs(model, mps, lo, hi):
    """L env at bond lo (sites < lo) and R env at bond hi+1 (sites > hi), by the oracle."""
    sym = model.sym
    nq = sym.nq
    Lenv = left_vacuum(sym)
    for l in range(lo):
        Lenv = oracle.contract_L(nq, Lenv, mps.A[l], model.W[l], mps.A[l])
    Renv = right_target(sym, mps.Qtot)
    for l in range(model.L - 1, hi, -1):
        Renv = oracle.contract_R(nq, Renv, mps.A[l], model.W[l], mps.A[l])
    return Lenv, Renv


def pivot1_case(kind="heis", L=8, D=16, site=3, seed=1, profile="even"):
    model, Q = make_model(kind, L)
    mps = RandomMPS(model, Q, D, seed=seed, profile=profile).canonicalize(site, site)
    Lenv, Renv = oracle_envs(model, mps, site, site)
    return model, mps, Lenv, Renv, model.W[site], mps.A[site]


def pivot2_case(kind="hubb", L=6, D=16, site=2, seed=2, profile="even"):
    model, Q = make_model(kind, L)
    mps = RandomMPS(model, Q, D, seed=seed, profile=profile).canonicalize(site, site + 1)
    Lenv, Renv = oracle_envs(model, mps, site, site + 1)
    V = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, model.sym.nq)
    return model, mps, Lenv, Renv, model.W[site], model.W[site + 1], V


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def blocks_by_key(B):
    return {B.key(i): B.block(i) for i in range(B.n)}


def compare_tripods(A, B):
    """max relative difference of two block tables compared by block keys."""
    ka, kb = blocks_by_key(A), blocks_by_key(B)
    assert set(ka) == set(kb), (set(ka) ^ set(kb))
    num = sum(float(np.sum((ka[k] - kb[k]) ** 2)) for k in ka)
    den = sum(float(np.sum(kb[k] ** 2)) for k in kb)
    return np.sqrt(num / max(den, 1e-300))


# ---- golden fixtures: block tables and MPO sites as flat npz arrays -----------
def blocks_to_npz(prefix, B, out):
    out[prefix + "_nq"] = np.array([B.nq])
    for name in ("qin", "qout", "leg", "rows", "cols", "offset", "data"):
        out[prefix + "_" + name] = getattr(B, name)
    if B.qmid is not None:
        out[prefix + "_qmid"] = B.qmid


def blocks_from_npz(prefix, z):
    from vmps_gb300.blocks import Blocks
    nq = int(z[prefix + "_nq"][0])
    qmid = z[prefix + "_qmid"] if prefix + "_qmid" in z else None
    return Blocks(nq, z[prefix + "_qin"], z[prefix + "_qout"], z[prefix + "_leg"], z[prefix + "_rows"],
                  z[prefix + "_cols"], data=z[prefix + "_data"], qmid=qmid, offset=z[prefix + "_offset"])


def mpo_to_npz(prefix, W, out):
    a = W.arrays()
    out[prefix + "_nq"] = np.array([W.nq])
    for name in ("s1", "s2", "k", "qin", "qout", "row", "col", "val", "qloc", "qop"):
        out[prefix + "_" + name] = a[name]


def mpo_from_npz(prefix, z):
    from vmps_gb300.blocks import MpoSite
    nq = int(z[prefix + "_nq"][0])
    W = MpoSite(nq, [tuple(q) for q in z[prefix + "_qloc"]], [tuple(q) for q in z[prefix + "_qop"]])
    for i in range(len(z[prefix + "_val"])):
        W.add(int(z[prefix + "_s1"][i]), int(z[prefix + "_s2"][i]), int(z[prefix + "_k"][i]),
              tuple(z[prefix + "_qin"][i]), tuple(z[prefix + "_qout"][i]), int(z[prefix + "_row"][i]),
              int(z[prefix + "_col"][i]), float(z[prefix + "_val"][i]))
    return W
