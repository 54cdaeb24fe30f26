"""ORACLE -- test infrastructure, not product code.

Dense pins for small chains:
* the full Hamiltonian contracted from an MPO, compared with an independent
  second-quantised construction (vmps_gb300.models.dense_*);
* the dense effective Hamiltonian P^T H P of a pivot (P = isometry from the
  pivot tensor to the full Hilbert space, built from the MPS tensors), which
  HxV must reproduce (the reference's ED-vs-DMRG check,
  programs/test_Hubbard/test_Hubbard.cc:227-300, applied to one HxV);
* exact ground-state energies.
"""
from __future__ import annotations

import numpy as np


def mpo_to_dense(model):
    """H = W[0] W[1] ... W[L-1] contracted over the auxiliary legs (boundary aux
    dimension 1 on both ends).  Basis: kron over sites, site 0 most significant."""
    d = model.d
    T = model.dense_W(0)[0]            # [a_out, s1, s2]
    T = np.transpose(T, (1, 2, 0))     # [s1, s2, a]
    for l in range(1, model.L):
        W = model.dense_W(l)           # [a_in, a_out, s1, s2]
        T = np.einsum("xya,abst->xsytb", T, W)
        n = T.shape[0] * d
        T = T.reshape(n, n, W.shape[1])
    return T[:, :, 0]


def local_perm(model):
    """Map MPO local index -> index in the dense reference construction."""
    if model.d == 4:
        return [0, 2, 1, 3]   # |0>,|up>,|dn>,|updn>  ->  Fock |n_up n_dn> = 0,2,1,3
    return list(range(model.d))


def permute_to_reference(H, model):
    """Reorder a kron-basis operator from MPO local indices to the dense
    reference construction's local indices."""
    p = np.array(local_perm(model))
    L = model.L
    idx = np.zeros(model.d ** L, dtype=np.int64)
    for n in range(model.d ** L):
        digits = np.unravel_index(n, [model.d] * L)
        idx[n] = np.ravel_multi_index([p[x] for x in digits], [model.d] * L)
    Hr = np.zeros_like(H)
    Hr[np.ix_(idx, idx)] = H
    return Hr


def _sector_offsets(dims):
    off, cur = {}, 0
    for q in sorted(dims):
        off[q] = cur
        cur += dims[q]
    return off, cur


def left_isometry(mps, l):
    """U (d^l x D_l): columns = left basis states of bond l, ordered by sorted QN sectors."""
    U = {(): np.ones((1, 1))}   # sector QN -> matrix (d^l x dim)
    vac = tuple(0 for _ in mps.Qtot)
    cur = {vac: np.ones((1, 1))}
    for site in range(l):
        A = mps.A[site]
        d = len(mps.qloc)
        nxt = {}
        rows_before = next(iter(cur.values())).shape[0]
        for i in range(A.n):
            qin, qout, s = tuple(A.qin[i]), tuple(A.qout[i]), int(A.leg[i])
            if qin not in cur:
                continue
            M = np.kron(cur[qin], np.eye(d)[:, [s]])     # (rows*d) x din, picks local state s as least significant
            contrib = M @ A.block(i)
            if qout in nxt:
                nxt[qout] = nxt[qout] + contrib
            else:
                nxt[qout] = contrib
        cur = nxt
        del rows_before
    off, tot = _sector_offsets(mps.dims[l])
    n = next(iter(cur.values())).shape[0]
    out = np.zeros((n, tot))
    for q, M in cur.items():
        out[:, off[q]:off[q] + M.shape[1]] = M
    del U
    return out


def right_isometry(mps, l):
    """V (D_l x d^(L-l)): rows = right basis states of bond l (sorted QN sectors)."""
    cur = {tuple(mps.Qtot): np.ones((1, 1))}
    d = len(mps.qloc)
    for site in range(mps.L - 1, l - 1, -1):
        A = mps.A[site]
        nxt = {}
        for i in range(A.n):
            qin, qout, s = tuple(A.qin[i]), tuple(A.qout[i]), int(A.leg[i])
            if qout not in cur:
                continue
            M = np.kron(np.eye(d)[[s], :], cur[qout])     # dout x (d * cols), local state most significant
            contrib = A.block(i) @ M
            nxt[qin] = nxt[qin] + contrib if qin in nxt else contrib
        cur = nxt
    off, tot = _sector_offsets(mps.dims[l])
    n = next(iter(cur.values())).shape[1]
    out = np.zeros((tot, n))
    for q, M in cur.items():
        out[off[q]:off[q] + M.shape[0], :] = M
    return out


def pivot1_isometry(mps, V, l):
    """P (d^L x dim V): maps the compact 1-site pivot tensor at site l to the full space."""
    UL = left_isometry(mps, l)
    UR = right_isometry(mps, l + 1)
    offL, _ = _sector_offsets(mps.dims[l])
    offR, _ = _sector_offsets(mps.dims[l + 1])
    d = len(mps.qloc)
    P = np.zeros((UL.shape[0] * d * UR.shape[1], V.data.size))
    for b in range(V.n):
        qin, qout, s = tuple(V.qin[b]), tuple(V.qout[b]), int(V.leg[b])
        r, c, o = int(V.rows[b]), int(V.cols[b]), int(V.offset[b])
        es = np.zeros(d); es[s] = 1.0
        for j in range(c):
            for i in range(r):
                P[:, o + i + j * r] = np.kron(np.kron(UL[:, offL[qin] + i], es), UR[offR[qout] + j, :])
    return P


def pivot2_isometry(mps, V, comb, l):
    """P for a 2-site pivot on sites l, l+1 with combined local index s1s3."""
    UL = left_isometry(mps, l)
    UR = right_isometry(mps, l + 2)
    offL, _ = _sector_offsets(mps.dims[l])
    offR, _ = _sector_offsets(mps.dims[l + 2])
    d = len(mps.qloc)
    inv = {}
    for (s1, s3), lst in comb["index"].items():
        for _, s13 in lst:
            inv[s13] = (s1, s3)
    P = np.zeros((UL.shape[0] * d * d * UR.shape[1], V.data.size))
    for b in range(V.n):
        qin, qout, s13 = tuple(V.qin[b]), tuple(V.qout[b]), int(V.leg[b])
        s1, s3 = inv[s13]
        e = np.zeros(d * d); e[s1 * d + s3] = 1.0
        r, c, o = int(V.rows[b]), int(V.cols[b]), int(V.offset[b])
        for j in range(c):
            for i in range(r):
                P[:, o + i + j * r] = np.kron(np.kron(UL[:, offL[qin] + i], e), UR[offR[qout] + j, :])
    return P


def ground_energy(H, sector_mask=None):
    if sector_mask is not None:
        H = H[np.ix_(sector_mask, sector_mask)]
    return float(np.linalg.eigvalsh(H)[0])
