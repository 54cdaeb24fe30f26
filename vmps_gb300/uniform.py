"""Infinite-MPS quantities of config C4 on the engine: a uniform MPS with a one-site
unit cell in the mixed gauge, its MPO environments, the energy density and the
VUMPS gradient.

* Gauge fixing (Umps: AL, AR, C with AL C = C AR = AC): left fixed point of
  C A = AL C' by repeated QR per outgoing multiplet (the diagonal of each R made
  positive, so the fixed point is unique), right fixed point of A C = C' AR by LQ
  with the SU(2) weights, then C = C_L C_R normalised with the multiplet weights.
* Environments (VumpsSolver::build_L / build_R, VUMPS/VumpsSolver.h:790-878): the
  MPO's auxiliary slots in the order of its basis (IDLE, OPEN..., DONE here); the
  left environment starts from the identity at IDLE; every later slot b is
  Y_b = contract_L(L, AL, W, AL) restricted to output slot b (FIXED_COLS, make_YL of
  VUMPS/VumpsContractions.h:228-258); the slot whose W entry is the identity (DONE)
  solves (1 - T_L + |R)(1|) L_b = Y_b - (Y_b|R) 1 by GMRES on the engine's transfer
  operator (vumps.MpoTransferMatrix), with |R) = C C^dagger; the right environment
  the same from DONE down to IDLE with AR and (L| = C^dagger C.
* Energy density e_L = (Y_DONE|R) (contract_LR, DmrgContractions.h:994-1020; unit
  cell of one site), e_R = (L|Y_IDLE).
* Gradient B = H_AC(AC) - AL H_C(C) (H_AC = PivotMatrix1(L, R, W), H_C =
  PivotMatrix0(L, R)); its norm with the PivotVector weights.

`precision` applies to the GMRES (split precision: FP64-refined, vumps.MpoTransferMatrix.
solve_linear_refined) and to the pivot applications; the slot contractions run in FP64.
`env(side, mode, fixed_ab, order, E, Abra, W, Aket)`, `transfer(side, A, W, LR, ab,
order, V, b)` (solves the linear system, returns (x, info)) and `apply(kind, L, R, W, V,
x)` are the contraction, the GMRES solve and the pivot application; by default the
engine's, so that the same steps can run on another implementation.
"""
from __future__ import annotations

import numpy as np

from .blocks import Blocks, Symmetry
from .mps import left_normalize, random_site, right_normalize
from .pivot import EnvUpdate, PivotMatrix0, PivotMatrix1
from .vumps import MpoTransferMatrix


def _deg(sym: Symmetry, q) -> float:
    d = 1.0
    for x, k in zip(q, sym.kinds):
        if k == "SU2":
            d *= x
    return d


def bond_bases_su2(nmult: int, qmax: int, q0: float = 3.0, sigma: float = None) -> list:
    """bond bases [{(q,): multiplets}] of a two-site unit cell of spin 1/2: integer spins
    (q odd) at bond 0, half-integer spins (q even) at bond 1, q <= qmax, nmult multiplets
    per bond, a Gaussian profile about q0; every multiplet is reached from the other
    bond's neighbours (d_q <= d'_{q-1} + d'_{q+1}, so the per-sector QR / LQ of the gauge
    fixing have full rank)"""
    sigma = sigma if sigma is not None else qmax / 3.0
    out = []
    for parity in (1, 0):
        qs = [q for q in range(1, qmax + 1) if q % 2 == parity]
        w = np.exp(-0.5 * ((np.array(qs) - q0) / sigma) ** 2)
        n = np.maximum(1, np.round(w / w.sum() * nmult)).astype(int)
        while n.sum() > nmult:
            n[int(np.argmax(n))] -= 1
        while n.sum() < nmult:
            n[int(np.argmax(w))] += 1
        out.append({(q,): int(c) for q, c in zip(qs, n)})
    # consistency between the two bonds: cap each sector by its neighbours on the other bond
    for _ in range(4 * qmax):
        changed = False
        for b in (0, 1):
            other = out[1 - b]
            for (q,), c in list(out[b].items()):
                cap = other.get((q - 1,), 0) + other.get((q + 1,), 0)
                if c > cap:
                    out[b][(q,)] = cap
                    changed = True
            out[b] = {k: v for k, v in out[b].items() if v > 0}
        if not changed:
            break
    return out


def _fix_left(AL: Blocks, R: dict):
    """positive diagonal of each R; the same signs on AL's columns"""
    for q, Rq in R.items():
        s = np.where(np.diag(Rq) < 0, -1.0, 1.0)
        R[q] = s[:, None] * Rq
        for i in range(AL.n):
            if tuple(AL.qout[i]) == q:
                AL.block(i)[...] = AL.block(i) * s[None, :]


def _fix_right(AR: Blocks, Lf: dict):
    """positive diagonal of each L; the same signs on AR's rows"""
    for q, Lq in Lf.items():
        s = np.where(np.diag(Lq) < 0, -1.0, 1.0)
        Lf[q] = Lq * s[None, :]
        for i in range(AR.n):
            if tuple(AR.qin[i]) == q:
                AR.block(i)[...] = s[:, None] * AR.block(i)


def _norm(sym, C: dict) -> float:
    return float(np.sqrt(sum(_deg(sym, q) * np.sum(M * M) for q, M in C.items())))


class UniformMPS:
    """uniform MPS with an n-site unit cell (site l between bonds l and l+1, bond n =
    bond 0) in the mixed gauge: AL[l], AR[l], C[l] (at bond l), AC[l] = AL[l] C[l+1]"""

    def __init__(self, model, dims: list, seed: int = 1):
        self.model, self.sym = model, model.sym
        self.dims = [dict(d) for d in dims]
        self.n = len(self.dims)
        rng = np.random.default_rng(seed)
        sym = self.sym if self.sym.nonabelian else None
        self.A = [random_site(model.qloc, self.dims[l], self.dims[(l + 1) % self.n], self.sym.nq, rng, sym)
                  for l in range(self.n)]

    def gauge(self, tol=1e-13, max_iter=2000):
        """left: C[l] A[l] = AL[l] C[l+1] around the cell until C[0] is stationary; right:
        A[l] C[l+1] = C[l] AR[l]; then C[l] = C_L[l] C_R[l] normalised, AC[l] = AL[l] C[l+1].
        Returns the iteration counts and the largest |AL C - C AR|."""
        sym, nq, n = self.sym, self.sym.nq, self.n
        s2 = sym if sym.nonabelian else None
        C = {q: np.eye(m) for q, m in self.dims[0].items()}
        CL, AL = [None] * n, [None] * n
        itl = 0
        for itl in range(1, max_iter + 1):
            C0 = C
            for l in range(n):
                CL[l] = C
                AL[l], R = left_normalize(self.A[l], nq, carry=C, sym=s2)
                _fix_left(AL[l], R)
                nr = _norm(sym, R)
                C = {q: M / nr for q, M in R.items()}
            d = _norm(sym, {q: C[q] - C0[q] for q in C})
            if d < tol:
                break
        CR, AR = [None] * n, [None] * n
        C = {q: np.eye(m) for q, m in self.dims[0].items()}
        itr = 0
        for itr in range(1, max_iter + 1):
            C0 = C
            for l in range(n - 1, -1, -1):
                CR[(l + 1) % n] = C
                AR[l], Lf = right_normalize(self.A[l], nq, carry=C, sym=s2)
                _fix_right(AR[l], Lf)
                nl = _norm(sym, Lf)
                C = {q: M / nl for q, M in Lf.items()}
            d = _norm(sym, {q: C[q] - C0[q] for q in C})
            if d < tol:
                break
        self.AL, self.AR = AL, AR
        self.C = []
        for l in range(n):
            M = {q: CL[l][q] @ CR[l][q] for q in self.dims[l]}
            nc = _norm(sym, M)
            self.C.append({q: X / nc for q, X in M.items()})
        self.AC = []
        for l in range(n):
            AC = AL[l].like(AL[l].data.copy())
            Cn = self.C[(l + 1) % n]
            for i in range(AC.n):
                AC.block(i)[...] = AL[l].block(i) @ Cn[tuple(AL[l].qout[i])]
            self.AC.append(AC)
        # the mixed-gauge condition AL[l] C[l+1] = C[l] AR[l]
        err = 0.0
        for l in range(n):
            for i in range(AL[l].n):
                q1, q2 = tuple(AL[l].qin[i]), tuple(AL[l].qout[i])
                j = AR[l].find(int(AL[l].leg[i]), q1, q2)
                if j >= 0:
                    err = max(err, float(np.abs(AL[l].block(i) @ self.C[(l + 1) % n][q2] -
                                                self.C[l][q1] @ AR[l].block(j)).max()))
        return {"left": itl, "right": itr, "gauge_err": err}

    def C_blocks(self, l: int) -> Blocks:
        """C[l] as a PivotVector of PivotMatrix0 (blocks (q, q))"""
        return Blocks.from_entries(self.sym.nq, [(0, q, q, self.C[l][q]) for q in sorted(self.C[l])])


class UniformEnvironment:
    """environments, energy density and gradient of a gauge-fixed UniformMPS with the
    bulk MPO sites W[l] of the cell (auxiliary basis `order`: basis_order_map of a bulk
    bond, the same at every bond of the cell)"""

    def __init__(self, ctx, model, u: UniformMPS, W: list, order: dict, precision="fp64", tol=1e-12, dimK=100,
                 env=None, transfer=None, apply=None, solver="device"):
        """solver: "device" runs GMRES on the GPU (vmps_transfer_solve), "host" the host loop
        of MpoTransferMatrix.solve_linear[_refined] over device operator applications"""
        self.ctx, self.model, self.u, self.W, self.order = ctx, model, u, list(W), order
        self.sym = model.sym
        self.precision, self.tol, self.dimK = precision, tol, dimK
        if solver not in ("device", "host"):
            raise ValueError("solver: 'device' or 'host'")
        self.solver = solver
        self.env = env or self._engine_env
        self.transfer = transfer or self._engine_transfer
        self.apply = apply or self._engine_apply
        self.inv = {v: k for k, v in order.items()}
        self.vac = self.sym.vacuum()
        vac_slots = sorted(v for (q, _), v in order.items() if tuple(q) == self.vac)
        self.first, self.last = vac_slots[0], vac_slots[-1]        # IDLE and DONE positions
        self.info = {}

    # ---- engine defaults
    def _engine_env(self, side, mode, fixed_ab, order, E, Abra, W, Aket):
        # a few contractions per environment: FP64 always, so that the energy density is FP64
        # whatever the precision of the GMRES and the pivots
        e = EnvUpdate(self.ctx, self.sym, side, E, Abra, W, Aket, mode=mode, fixed_ab=fixed_ab, order=order)
        try:
            return e.run(E, Abra, Aket, "fp64")
        finally:
            e.close()

    def _engine_transfer(self, side, A, W, LR, ab, order, V, b):
        T = MpoTransferMatrix(self.ctx, self.sym, side, A, A, W, LR, ab, order, V)
        try:
            if self.solver == "device":
                return T.solve_device(b, tol=self.tol, dimK=self.dimK, precision=self.precision)
            if self.precision == "fp64":
                return T.solve_linear(b, tol=self.tol, dimK=self.dimK)
            return T.solve_linear_refined(b, tol=self.tol, dimK=self.dimK)
        finally:
            T.close()

    def _engine_apply(self, kind, L, R, W, V, x):
        H = PivotMatrix1(self.ctx, self.sym, L, R, W, V) if kind == 1 else PivotMatrix0(self.ctx, self.sym, L, R, V)
        try:
            return H.apply(x, self.precision)
        finally:
            H.close()

    # ---- helpers
    def _identity(self, slot, bond=0) -> Blocks:
        q0, a = self.inv[slot]
        return Blocks.from_entries(self.sym.nq, [(a, q, q, tuple(q0), np.eye(n))
                                                 for q, n in sorted(self.u.dims[bond].items())], tripod=True)

    def _into(self, V: Blocks, Y: Blocks) -> np.ndarray:
        x = np.zeros(V.data.size)
        for i in range(Y.n):
            k = V.find(*Y.key(i))
            if k >= 0:
                o, r, c = int(V.offset[k]), int(V.rows[k]), int(V.cols[k])
                x[o:o + r * c] = Y.data[Y.offset[i]:Y.offset[i] + r * c]
        return x

    def _contract_LR(self, Y: Blocks, slot, LR: dict) -> float:
        """(Y|LR) over the vacuum-mid blocks of one slot with multiplet weights (contract_LR)"""
        q0, a = self.inv[slot]
        s = 0.0
        for i in range(Y.n):
            if tuple(Y.qmid[i]) == tuple(q0) and int(Y.leg[i]) == a and tuple(Y.qin[i]) == tuple(Y.qout[i]):
                q = tuple(Y.qin[i])
                if q in LR:
                    s += float(np.trace(Y.block(i) @ LR[q])) * _deg(self.sym, q)
        return s

    @staticmethod
    def _merge(parts: list) -> Blocks:
        ent = []
        for P in parts:
            for i in range(P.n):
                leg, qin, qout, qmid = P.key(i)
                ent.append((leg, qin, qout, qmid, P.block(i).copy()))
        return Blocks.from_entries(parts[0].nq, ent, tripod=True)

    def _blocks_of(self, M: dict) -> Blocks:
        return Blocks.from_entries(self.sym.nq, [(0, q, q, M[q]) for q in sorted(M)])

    def _cell(self, side, mode_last, b, E, A):
        """E through the cell (left: sites 0..n-1, right: n-1..0), the last contraction
        restricted to slot b (the others FULL: E holds only the slots already built)"""
        n = self.u.n
        sites = range(n) if side == "L" else range(n - 1, -1, -1)
        for k, l in enumerate(sites):
            mode = mode_last if k == n - 1 else "FULL"
            E = self.env(side, mode, b, self.order, E, A[l], self.W[l], A[l])
        return E

    def _solve(self, side, Y, slot, LR, A):
        e = self._contract_LR(Y, slot, LR)
        V = self._identity(slot).like()
        T = MpoTransferMatrix.__new__(MpoTransferMatrix)   # the right-hand side helper only
        T.sym, T.V, T.ab_key = self.sym, V, self.inv[slot]
        rhs = MpoTransferMatrix.rhs(T, self._into(V, Y), e)
        x, info = self.transfer(side, A, self.W, self._blocks_of(LR), slot, self.order, V, rhs)
        return e, V.like(x), info

    # ---- the environments at bond 0
    def left(self):
        u = self.u
        R = {q: M @ M.T for q, M in u.C[0].items()}
        parts = [self._identity(self.first)]
        for b in range(self.first + 1, self.last + 1):
            Y = self._cell("L", "FIXED_COLS", b, self._merge(parts), u.AL)
            if b != self.last:
                parts.append(Y)
                continue
            self.eL, X, self.info["gmres_left"] = self._solve("L", Y, b, R, u.AL)
            parts.append(X)
        self.L = self._merge(parts)
        return self.L

    def right(self):
        u = self.u
        Lf = {q: M.T @ M for q, M in u.C[0].items()}
        parts = [self._identity(self.last)]
        for a in range(self.last - 1, self.first - 1, -1):
            Y = self._cell("R", "FIXED_ROWS", a, self._merge(parts), u.AR)
            if a != self.first:
                parts.append(Y)
                continue
            self.eR, X, self.info["gmres_right"] = self._solve("R", Y, a, Lf, u.AR)
            parts.append(X)
        self.R = self._merge(parts)
        return self.R

    def energy_density(self) -> float:
        """the energy per site, (e_L + e_R) / 2 over the cell length"""
        return 0.5 * (self.eL + self.eR) / self.u.n

    def gradient(self):
        """VUMPS gradient over the cell: sqrt(sum_l |B_l|^2), B_l = H_AC(AC[l]) - AL[l] H_C(C[l+1]),
        with the PivotVector weights; environments at every bond from those at bond 0"""
        u, n = self.u, self.u.n
        Ls = [self.L]
        for l in range(n - 1):
            Ls.append(self.env("L", "FULL", 0, self.order, Ls[-1], u.AL[l], self.W[l], u.AL[l]))
        Rs = [None] * (n + 1)
        Rs[n] = self.R
        for l in range(n - 1, 0, -1):
            Rs[l] = self.env("R", "FULL", 0, self.order, Rs[l + 1], u.AR[l], self.W[l], u.AR[l])
        Rs[0] = self.R
        tot = 0.0
        parts = []
        for l in range(n):
            AC = u.AC[l]
            hac = self.apply(1, Ls[l], Rs[l + 1], self.W[l], AC, AC.data)
            m = (l + 1) % n
            Cb = u.C_blocks(m)
            hc = self.apply(0, Ls[m] if m < n else Ls[0], Rs[m] if m > 0 else Rs[n], None, Cb, Cb.data)
            HC = {tuple(Cb.qin[i]): hc[Cb.offset[i]:Cb.offset[i] + Cb.rows[i] * Cb.cols[i]].reshape(
                Cb.cols[i], Cb.rows[i]).T for i in range(Cb.n)}
            w = np.zeros(AC.data.size)
            alhc = np.zeros(AC.data.size)
            for i in range(AC.n):
                o, r, c = int(AC.offset[i]), int(AC.rows[i]), int(AC.cols[i])
                q = tuple(AC.qout[i])
                alhc[o:o + r * c] = (u.AL[l].block(i) @ HC[q]).T.ravel()
                w[o:o + r * c] = self.sym.dot_weight(q)
            B = hac - alhc
            nb = float(np.sum(w * B * B))
            parts.append(float(np.sqrt(nb)))
            tot += nb
        return float(np.sqrt(tot)), parts
