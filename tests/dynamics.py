"""Real-time evolution on a two-site pivot with complete bond bases (test
infrastructure for the reference's golden dynamics data).

With complete bond bases the two-site pivot of an L-site chain spans the whole
symmetry sector, so exp(-i H t) applied to a pivot vector is exact dynamics, and
only HxV is needed: a Krylov (Lanczos) propagator with complex coefficients
calls the operator on the real and imaginary parts.  The observable is an MPO
(here the staggered magnetisation) applied through its own pivot.

This is the shape of the reference's dynamics check
(programs/test_Heisenberg/test_Heisenberg.cc:279-310: Neel state, L = 12,
TDVPPropagator::t_step with LanczosPropagator, M_stag = (1/L) sum_l (-1)^l <S^z_l>).
"""
from __future__ import annotations

import numpy as np

from vmps_gb300 import models
from vmps_gb300.mps import RandomMPS, contract_two_sites

L_DYN = 12


def neel_case(L=L_DYN, Jxy=-1.0, Jz=0.0, seed=11):
    """(model, observable MPO, mps, site, V layout, comb, neel config): complete bond
    bases (D = 2^(L/2)), centre on the two middle sites"""
    model = models.heisenberg_u1(L, Jxy=Jxy, Jz=Jz)
    obs = models.spin_half_local_sum(L, [(-1) ** l / L for l in range(L)])
    site = L // 2 - 1
    mps = RandomMPS(model, (0,), 2 ** (L // 2), seed=seed).canonicalize(site, site + 1)
    V, comb = contract_two_sites(model.sym, mps.A[site], mps.A[site + 1], model.qloc, model.qloc, 1,
                                 return_basis=True)
    neel = [l % 2 for l in range(L)]   # s = 0 (up) on even sites: M_stag(0) = +1/2
    return model, obs, mps, site, V, comb, neel


def neel_vector(mps, site, V, comb, neel):
    """The Neel product state in the pivot's coordinates: V[s s'](a, b) = l_a r_b on the
    block of the Neel configuration of the two pivot sites, where l (r) is the row
    (column) of the left (right) isometry for the Neel configuration of the sites left
    (right) of the pivot."""
    A = mps.A
    left = {(0,): np.ones(1)}
    for l in range(site):
        nxt = {}
        for i in range(A[l].n):
            if A[l].leg[i] != neel[l] or tuple(A[l].qin[i]) not in left:
                continue
            q = tuple(A[l].qout[i])
            nxt[q] = nxt.get(q, 0) + left[tuple(A[l].qin[i])] @ A[l].block(i)
        left = nxt
    right = {tuple(mps.Qtot): np.ones(1)}
    for l in range(len(A) - 1, site + 1, -1):
        nxt = {}
        for i in range(A[l].n):
            if A[l].leg[i] != neel[l] or tuple(A[l].qout[i]) not in right:
                continue
            q = tuple(A[l].qin[i])
            nxt[q] = nxt.get(q, 0) + A[l].block(i) @ right[tuple(A[l].qout[i])]
        right = nxt
    v = np.zeros(V.data.size)
    out = V.like(v)
    (qn, s13), = comb["index"][(neel[site], neel[site + 1])]
    for k in range(out.n):
        if out.leg[k] == s13 and tuple(out.qin[k]) in left and tuple(out.qout[k]) in right:
            out.block(k)[...] = np.outer(left[tuple(out.qin[k])], right[tuple(out.qout[k])])
    return out.data.copy()


def krylov_step(apply2, psi, dt, m=30):
    """psi(t + dt) = exp(-i H dt) psi by an m-step Lanczos propagator with full
    reorthogonalisation; apply2(X) applies H to the rows of a real 2 x n array (the
    real and imaginary parts)."""
    nrm = np.linalg.norm(psi)
    Q = np.zeros((m + 1, psi.size), dtype=np.complex128)
    Q[0] = psi / nrm
    a, b = np.zeros(m), np.zeros(m)
    k = m
    for j in range(m):
        q = Q[j]
        hq = apply2(np.stack([q.real, q.imag]))
        w = hq[0] + 1j * hq[1]
        a[j] = float(np.real(np.vdot(q, w)))
        w = w - Q[:j + 1].T @ (Q[:j + 1].conj() @ w)
        w = w - Q[:j + 1].T @ (Q[:j + 1].conj() @ w)
        b[j] = np.linalg.norm(w)
        if b[j] < 1e-14 * max(1.0, abs(a[j])):
            k = j + 1
            break
        Q[j + 1] = w / b[j]
    T = np.diag(a[:k]) + np.diag(b[:k - 1], 1) + np.diag(b[:k - 1], -1)
    e, U = np.linalg.eigh(T)
    c = U @ (np.exp(-1j * e * dt) * U[0])
    return nrm * (Q[:k].T @ c)


def mstag_series(apply_h, apply_m, psi0, times):
    """M_stag(t) = <psi(t)| M |psi(t)> at the given, evenly spaced times (t_0 = 0);
    apply_h / apply_m apply H and the observable to the rows of a real 2 x n array"""
    dt = times[1] - times[0]
    psi = psi0.astype(np.complex128)
    out = []
    for i, _ in enumerate(times):
        if i:
            psi = krylov_step(apply_h, psi, dt)
        mp = apply_m(np.stack([psi.real, psi.imag]))
        out.append(float(psi.real @ mp[0] + psi.imag @ mp[1]) / float(np.vdot(psi, psi).real))
    return np.array(out)


def exact_mstag(L, Jxy, Jz, times):
    """exact diagonalisation of the Sz = 0 sector (bit l set = spin up on site l)"""
    states = [s for s in range(1 << L) if bin(s).count("1") == L // 2]
    idx = {s: i for i, s in enumerate(states)}
    n = len(states)
    H = np.zeros((n, n))
    for i, s in enumerate(states):
        for l in range(L - 1):
            a, b = (s >> l) & 1, (s >> (l + 1)) & 1
            H[i, i] += Jz * (a - 0.5) * (b - 0.5)
            if a != b:
                H[idx[s ^ (1 << l) ^ (1 << (l + 1))], i] += 0.5 * Jxy
    neel = sum(1 << l for l in range(0, L, 2))
    stag = np.array([sum((-1) ** l * (((s >> l) & 1) - 0.5) for l in range(L)) / L for s in states])
    e, U = np.linalg.eigh(H)
    c = U[idx[neel]]
    return np.array([float(np.sum(np.abs(U @ (np.exp(-1j * e * t) * c)) ** 2 * stag)) for t in times])
