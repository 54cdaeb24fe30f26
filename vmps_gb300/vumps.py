"""VUMPS environment operator on the GB300 engine.

``MpoTransferMatrix`` mirrors the reference's MpoTransferMatrix /
MpoTransferVector pair (VUMPS/VumpsMpoTransferMatrix.h:14-330): ``hxv`` is
HxV(MpoTransferMatrix, Vin, Vout) (:99-212), the cell chain of contract_L or
contract_R with FIXED_ROWS / FIXED_COLS masks plus the |R)(1| projector via
contract_LR, evaluated by the native library with the contractions on the GPU.
``dot`` is the transfer-vector inner product (:258-275) and ``solve_linear``
the GMRES solve of VumpsSolver::solve_linear (VUMPS/VumpsSolver.h:1907-1940),
b = Y - LRdotY * 1 on slot ab (MpoTransferVector's constructor, :53-66).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .blocks import Blocks, Symmetry


class MpoTransferMatrix:
    def __init__(self, ctx, sym: Symmetry, direction: str, Abra: list, Aket: list, W: list, LReigen: Blocks,
                 ab: int, order: dict, V: Blocks):
        """direction 'L' (1 - T_L + |R)(1|) or 'R'; Abra/Aket/W: the unit cell's site tensors;
        order: basis_order_map {(aux QN, index in sector): position}; V: the Tripod layout of the vectors."""
        self.sym, self.V = sym, V
        self.ab = ab
        inv = {v: k for k, v in order.items()}
        self.ab_key = inv[ab]            # basis_order[ab] = (QN, index)
        n = len(W)
        self._keep = (Abra, Aket, W, LReigen, V)
        bra = [a.c_struct() for a in Abra]
        ket = [a.c_struct() for a in Aket]
        wst = [w.c_struct() for w in W]
        BP = C.POINTER(N.vmps_blocks)
        pbra = (BP * n)(*[C.pointer(b) for b in bra])
        pket = (BP * n)(*[C.pointer(b) for b in ket])
        pw = (C.POINTER(N.vmps_mpo_site) * n)(*[C.pointer(w) for w in wst])
        dbra = (N.f64p * n)(*[a.data.ctypes.data_as(N.f64p) for a in Abra])
        dket = (N.f64p * n)(*[a.data.ctypes.data_as(N.f64p) for a in Aket])
        items = sorted(order.items())
        qn = np.ascontiguousarray(np.array([list(k[0]) for k, _ in items], dtype=np.int32).reshape(-1, sym.nq))
        idx = np.ascontiguousarray([k[1] for k, _ in items], dtype=np.int32)
        val = np.ascontiguousarray([v for _, v in items], dtype=np.int64)
        s, lr, vb = sym.c_struct(), LReigen.c_struct(), V.c_struct()
        self._h = C.c_void_p()
        N.check(N.lib().vmps_transfer_create(
            ctx._h, C.byref(s), N.ENV_LEFT if direction == "L" else N.ENV_RIGHT, n, pbra, dbra, pket, dket, pw,
            C.byref(lr), LReigen.data.ctypes.data_as(N.f64p), ab, len(val), qn.ctypes.data_as(N.i32p),
            idx.ctypes.data_as(N.i32p), val.ctypes.data_as(N.i64p), C.byref(vb), C.byref(self._h)))

    def hxv(self, vin: np.ndarray, precision="fp64") -> np.ndarray:
        vin = np.ascontiguousarray(vin, dtype=np.float64)
        out = np.zeros_like(vin)
        N.check(N.lib().vmps_transfer_hxv(self._h, vin.ctypes.data_as(N.f64p), out.ctypes.data_as(N.f64p),
                                          1 if precision == "bf16x3" else 0))
        return out

    # ---- the transfer-vector space: blocks of mid QN ab.first at slot ab.second
    def slot_mask(self) -> np.ndarray:
        if getattr(self, "_mask", None) is None:
            V, (q, a) = self.V, self.ab_key
            m = np.zeros(V.data.size, dtype=bool)
            for i in range(V.n):
                if tuple(V.qmid[i]) == tuple(q) and V.leg[i] == a:
                    m[V.offset[i]:V.offset[i] + V.rows[i] * V.cols[i]] = True
            self._mask = m
        return self._mask

    def weights(self) -> np.ndarray:
        """coeff_dot(out) per element (VumpsMpoTransferMatrix.h:258-275)"""
        if getattr(self, "_w", None) is None:
            V = self.V
            w = np.zeros(V.data.size)
            for i in range(V.n):
                w[V.offset[i]:V.offset[i] + V.rows[i] * V.cols[i]] = self.sym.dot_weight(tuple(V.qout[i]))
            self._w = w
        return self._w

    def dot(self, a: np.ndarray, b: np.ndarray) -> float:
        m = self.slot_mask()
        return float(np.sum((a * b * self.weights())[m]))

    def rhs(self, Y: np.ndarray, LRdotY: float) -> np.ndarray:
        """MpoTransferVector(Y, ab, LRdotY): Y - LRdotY * 1 on the slot-ab blocks"""
        V, (q, a) = self.V, self.ab_key
        b = np.array(Y, dtype=np.float64)
        for i in range(V.n):
            if tuple(V.qmid[i]) == tuple(q) and V.leg[i] == a:
                blk = b[V.offset[i]:V.offset[i] + V.rows[i] * V.cols[i]].reshape(V.cols[i], V.rows[i]).T
                blk -= LRdotY * np.eye(V.rows[i], V.cols[i])
                b[V.offset[i]:V.offset[i] + V.rows[i] * V.cols[i]] = blk.T.ravel()
        return b

    def solve_linear(self, b: np.ndarray, x0: np.ndarray | None = None, tol=1e-10, dimK=200, max_restarts=20,
                     precision="fp64"):
        """GMRES (restarted, modified Gram-Schmidt with the weighted dot) for H x = b; returns (x, info)."""
        m = self.slot_mask()
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        nb = np.sqrt(self.dot(b, b))
        if nb == 0:
            return x, {"iterations": 0, "residual": 0.0}
        its = 0
        for _ in range(max_restarts):
            r = (b - self.hxv(x, precision)) * m
            beta = np.sqrt(self.dot(r, r))
            if beta <= tol * nb:
                return x, {"iterations": its, "residual": beta / nb}
            Q = [r / beta]
            Hh = np.zeros((dimK + 1, dimK))
            k = 0
            for k in range(dimK):
                w = self.hxv(Q[k], precision) * m
                its += 1
                for j in range(k + 1):
                    Hh[j, k] = self.dot(Q[j], w)
                    w = w - Hh[j, k] * Q[j]
                Hh[k + 1, k] = np.sqrt(self.dot(w, w))
                if not np.all(np.isfinite(Hh[:k + 2, k])):
                    raise FloatingPointError("GMRES: the operator produced non-finite values")
                e1 = np.zeros(k + 2); e1[0] = beta
                y, *_ = np.linalg.lstsq(Hh[:k + 2, :k + 1], e1, rcond=None)
                res = np.linalg.norm(Hh[:k + 2, :k + 1] @ y - e1)
                if Hh[k + 1, k] <= 1e-14 * beta or res <= tol * nb:
                    break
                Q.append(w / Hh[k + 1, k])
            x = x + sum(yi * qi for yi, qi in zip(y, Q))
        r = (b - self.hxv(x, precision)) * m
        return x, {"iterations": its, "residual": np.sqrt(self.dot(r, r)) / nb}

    def solve_device(self, b: np.ndarray, tol=1e-10, dimK=200, max_restarts=20, precision="fp64", inner_tol=1e-4,
                     max_outer=10):
        """The same solves on the device (vmps_transfer_solve): Krylov vectors in device
        memory, the Hessenberg matrix on the host.  precision "fp64": GMRES with the FP64
        operator (solve_linear); "bf16x3": FP64-residual refinement with split-precision
        GMRES corrections (solve_linear_refined), FP64 GMRES finishing when a round does not
        halve the residual.  Returns (x, info)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        st = N.vmps_gmres_stats()
        N.check(N.lib().vmps_transfer_solve(self._h, b.ctypes.data_as(N.f64p), x.ctypes.data_as(N.f64p), float(tol),
                                            int(dimK), int(max_restarts), 1 if precision == "bf16x3" else 0,
                                            float(inner_tol), int(max_outer), C.byref(st)))
        return x, st.as_dict()

    def solve_linear_refined(self, b: np.ndarray, tol=1e-10, inner_tol=1e-4, dimK=200, max_outer=10):
        """Mixed-precision iterative refinement: the residual r = b - H x with the FP64
        operator, the correction H d = r by GMRES with the split-precision operator to
        inner_tol, x += d; each round gains about the split operator's accuracy.
        Returns (x, info) with the FP64 residual."""
        m = self.slot_mask()
        x = np.zeros_like(b)
        nb = np.sqrt(self.dot(b, b))
        info = {"outer": 0, "split_iterations": 0, "fp64_hxv": 0, "residual": 0.0}
        if nb == 0:
            return x, info
        for outer in range(max_outer):
            r = (b - self.hxv(x, "fp64")) * m
            info["fp64_hxv"] += 1
            res = np.sqrt(self.dot(r, r)) / nb
            info["residual"] = res
            if res <= tol:
                break
            d, inner = self.solve_linear(r, tol=inner_tol, dimK=dimK, max_restarts=2, precision="bf16x3")
            info["split_iterations"] += inner["iterations"]
            info["outer"] = outer + 1
            x = x + d
        return x, info

    def close(self):
        if getattr(self, "_h", None):
            N.lib().vmps_transfer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
