"""Reference-facing API: PivotMatrix1/2/0, HxV, contract_L / contract_R.

Mirrors the operator interface of VMPS for the effective-Hamiltonian path:

    HxV(const PivotMatrix1&, const PivotVector& Vin, PivotVector& Vout)   pivot/DmrgPivotMatrix1.h:123-129
    HxV(const PivotMatrix2&, ...)                                         pivot/DmrgPivotMatrix2.h:78-83
    HxV(const PivotMatrix0&, ...)                                         pivot/DmrgPivotMatrix0.h:31-96
    contract_L(Lold, Abra, W, Aket, qloc, qOp, Lnew)                      tensors/DmrgContractions.h:34-158
    contract_R(Rold, Abra, W, Aket, qloc, qOp, Rnew)                      tensors/DmrgContractions.h:179-311

A ``PivotVector`` is a ``Blocks`` table with leg = physical (or combined
two-site) index.  Every compute call goes through the native library; errors
come back as ``VmpsError`` with the library's message (the reference itself
asserts).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .blocks import Blocks, MpoSite, Symmetry

PREC = {"fp64": N.PREC_FP64, "bf16x3": N.PREC_BF16X3, "tf32x3": N.PREC_TF32X3}


def _prec(p):
    return PREC[p] if isinstance(p, str) else int(p)


class Context:
    """One CUDA stream on one device."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        self.device = device
        N.check(N.lib().vmps_ctx_create(device, C.byref(self._h)))

    def close(self):
        if self._h:
            N.lib().vmps_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Pivot:
    def __init__(self, ctx: Context, sym: Symmetry, V: Blocks):
        self.ctx = ctx
        self.sym = sym
        self.layout = V.like()
        self._h = C.c_void_p()

    def close(self):
        if self._h:
            N.lib().vmps_pivot_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def dim(self) -> int:
        n = C.c_int64()
        N.check(N.lib().vmps_pivot_dim(self._h, C.byref(n)))
        return n.value

    def chains(self):
        """(idx, coef, n_tasks): the pivot's task list, idx rows (out, x, y, z)"""
        n, nt = C.c_int64(), C.c_int64()
        N.check(N.lib().vmps_pivot_chains(self._h, 0, C.byref(n), None, None, C.byref(nt)))
        idx = np.zeros((max(n.value, 1), 4), dtype=np.int64)
        coef = np.zeros(max(n.value, 1))
        if n.value:
            N.check(N.lib().vmps_pivot_chains(self._h, n.value, C.byref(n), idx.ctypes.data_as(N.i64p),
                                              coef.ctypes.data_as(N.f64p), C.byref(nt)))
        return idx[:n.value], coef[:n.value], nt.value

    def stats(self, precision="fp64") -> dict:
        s = N.vmps_plan_stats()
        N.check(N.lib().vmps_pivot_stats(self._h, _prec(precision), C.byref(s)))
        return s.as_dict()

    def prepare(self, precision="fp64", fp64_too=False):
        """Build the device work lists of `precision` now instead of at the first
        HxV (and the FP64 ones as well when the FP64 refinement will need them)."""
        self.stats(precision)
        if fp64_too and _prec(precision) != _prec("fp64"):
            self.stats("fp64")

    def apply(self, vin: np.ndarray, precision="fp64", out: np.ndarray | None = None) -> np.ndarray:
        """Vout = H * Vin on compact host arrays (host->device->host inside)."""
        vin = np.ascontiguousarray(vin, dtype=np.float64)
        if vin.size != self.dim:
            raise ValueError(f"vector has {vin.size} elements, layout needs {self.dim}")
        if out is None:
            out = np.empty_like(vin)
        N.check(N.lib().vmps_hxv(self._h, vin.ctypes.data_as(N.f64p), out.ctypes.data_as(N.f64p), _prec(precision)))
        return out

    def apply_multi(self, vin: np.ndarray, precision="fp64") -> np.ndarray:
        """H applied to the rows of vin (nrhs x dim) in one call; split precision runs
        all right-hand sides in one grouped HxV."""
        vin = np.ascontiguousarray(np.atleast_2d(vin), dtype=np.float64)
        if vin.shape[1] != self.dim:
            raise ValueError(f"vectors have {vin.shape[1]} elements, layout needs {self.dim}")
        out = np.empty_like(vin)
        N.check(N.lib().vmps_hxv_multi(self._h, vin.ctypes.data_as(N.f64p), out.ctypes.data_as(N.f64p),
                                       vin.shape[0], _prec(precision)))
        return out

    def spectral_bounds(self, v0: np.ndarray, iters=80):
        """(E_min, E_max): extreme Ritz values after `iters` FP64 Lanczos steps."""
        v = np.ascontiguousarray(v0, dtype=np.float64)
        lo, hi = C.c_double(), C.c_double()
        N.check(N.lib().vmps_spectral_bounds(self._h, v.ctypes.data_as(N.f64p), iters, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def chebyshev_moments(self, v0: np.ndarray, nmom: int, a: float, b: float, precision="fp64", parts=None):
        """Moments mu[k, n] = <v0_k| T_n((H - b)/a) |v0_k> of the rows of v0 (nrhs x dim),
        advanced together on the device; returns (mu, stats).  parts: block-index
        boundaries [0, b1, ..., nblocks] of the vector layout (a union pivot's sectors);
        mu is then nrhs x nparts x nmom, the moments of each part of each row."""
        v0 = np.ascontiguousarray(np.atleast_2d(v0), dtype=np.float64)
        if v0.shape[1] != self.dim:
            raise ValueError(f"vectors have {v0.shape[1]} elements, layout needs {self.dim}")
        st = N.vmps_cheb_stats()
        if parts is None:
            mu = np.empty((v0.shape[0], nmom))
            N.check(N.lib().vmps_chebyshev_moments(self._h, v0.ctypes.data_as(N.f64p), v0.shape[0], nmom, float(a),
                                                   float(b), _prec(precision), mu.ctypes.data_as(N.f64p),
                                                   C.byref(st)))
        else:
            pb = np.ascontiguousarray(parts, dtype=np.int64)
            mu = np.empty((v0.shape[0], len(pb) - 1, nmom))
            N.check(N.lib().vmps_chebyshev_moments_parts(self._h, v0.ctypes.data_as(N.f64p), v0.shape[0], nmom,
                                                         float(a), float(b), _prec(precision), len(pb) - 1,
                                                         pb.ctypes.data_as(N.i64p), mu.ctypes.data_as(N.f64p),
                                                         C.byref(st)))
        return mu, st.as_dict()

    def autotune(self, trials=5) -> dict:
        """Choose the split-precision tiling (tile N caps, split-K) of this pivot by
        timing the candidates on it (vmps_pivot_autotune); cached per sector layout."""
        info = N.vmps_tune_info()
        N.check(N.lib().vmps_pivot_autotune(self._h, int(trials), C.byref(info)))
        return info.as_dict()

    def set_tiling(self, ncap1=256, ncap2=256, splitk=1):
        """Fix the split-precision tiling (tile N caps of the two phases, split-K of
        phase 2) without tuning."""
        N.check(N.lib().vmps_pivot_set_tiling(self._h, int(ncap1), int(ncap2), int(splitk)))

    def set_projector(self, A0proj, Epenalty: float):
        """Excited-state projector (PivotMatrix1/2::A0proj, Epenalty): every later HxV
        adds Epenalty * <A0_n|Vin> * A0_n for each vector A0_n (compact layout of this
        pivot; a list of vectors or an nproj x dim array).  An empty list removes it."""
        A0 = np.ascontiguousarray(np.reshape(np.asarray(A0proj, dtype=np.float64), (-1, self.dim)))
        self._A0 = A0
        N.check(N.lib().vmps_pivot_set_penalty(self._h, A0.shape[0], A0.ctypes.data_as(N.f64p), float(Epenalty)))

    def lanczos(self, v0: np.ndarray, precision="fp64", max_iter=200, tol_eigval=1e-12, tol_state=1e-8,
                refine_iters=0):
        """Ground state by full-reorthogonalisation Lanczos on the device."""
        v = np.array(v0, dtype=np.float64, copy=True)
        e = C.c_double()
        st = N.vmps_lanczos_stats()
        N.check(N.lib().vmps_lanczos_ground(self._h, v.ctypes.data_as(N.f64p), _prec(precision), max_iter,
                                            tol_eigval, tol_state, refine_iters, C.byref(e), C.byref(st)))
        return e.value, v, st.as_dict()


def _term_arrays(terms, nmpo):
    """ctypes arrays of the per-term tables of a multi-term pivot"""
    n = len(terms)
    keep = []
    Lt, Ld = (C.POINTER(N.vmps_blocks) * n)(), (N.f64p * n)()
    Rt, Rd = (C.POINTER(N.vmps_blocks) * n)(), (N.f64p * n)()
    Ws = [(C.POINTER(N.vmps_mpo_site) * n)() for _ in range(nmpo)]
    for t, term in enumerate(terms):
        L, R, mpos = term[0], term[1], term[2:]
        lb, rb = L.c_struct(), R.c_struct()
        ws = [W.c_struct() for W in mpos]
        keep += [lb, rb] + ws
        Lt[t], Ld[t] = C.pointer(lb), L.data_ptr()
        Rt[t], Rd[t] = C.pointer(rb), R.data_ptr()
        for i in range(nmpo):
            Ws[i][t] = C.pointer(ws[i])
    return Lt, Ld, Rt, Rd, Ws, keep


class PivotMatrix1(_Pivot):
    """1-site effective Hamiltonian (pivot/DmrgPivotMatrix1.h:46-121)."""

    def __init__(self, ctx, sym, L: Blocks, R: Blocks, W: MpoSite, V: Blocks, _terms=None):
        super().__init__(ctx, sym, V)
        s, vb = sym.c_struct(), V.c_struct()
        if _terms is not None:
            Lt, Ld, Rt, Rd, (Wt,), keep = _term_arrays(_terms, 1)
            N.check(N.lib().vmps_pivot1_create_terms(ctx._h, C.byref(s), len(_terms), Lt, Ld, Rt, Rd, Wt,
                                                     C.byref(vb), C.byref(self._h)))
            return
        lb, rb, wb = L.c_struct(), R.c_struct(), W.c_struct()
        N.check(N.lib().vmps_pivot1_create(ctx._h, C.byref(s), C.byref(lb), L.data_ptr(), C.byref(rb), R.data_ptr(),
                                           C.byref(wb), C.byref(vb), C.byref(self._h)))

    @classmethod
    def from_terms(cls, ctx, sym, terms, V: Blocks):
        """PivotMatrix1 with several terms (PivotMatrix1::Terms): `terms` is a list of
        (L, R, W); HxV returns the sum over the terms."""
        return cls(ctx, sym, None, None, None, V, _terms=list(terms))


class PivotMatrix2(_Pivot):
    """2-site effective Hamiltonian (pivot/DmrgPivotMatrix2.h:29-76)."""

    def __init__(self, ctx, sym, L: Blocks, R: Blocks, W12: MpoSite, W34: MpoSite, V: Blocks, _terms=None):
        super().__init__(ctx, sym, V)
        s, vb = sym.c_struct(), V.c_struct()
        if _terms is not None:
            Lt, Ld, Rt, Rd, (W1t, W2t), keep = _term_arrays(_terms, 2)
            N.check(N.lib().vmps_pivot2_create_terms(ctx._h, C.byref(s), len(_terms), Lt, Ld, Rt, Rd, W1t, W2t,
                                                     C.byref(vb), C.byref(self._h)))
            return
        lb, rb = L.c_struct(), R.c_struct()
        w1, w2 = W12.c_struct(), W34.c_struct()
        N.check(N.lib().vmps_pivot2_create(ctx._h, C.byref(s), C.byref(lb), L.data_ptr(), C.byref(rb), R.data_ptr(),
                                           C.byref(w1), C.byref(w2), C.byref(vb), C.byref(self._h)))

    @classmethod
    def from_terms(cls, ctx, sym, terms, V: Blocks):
        """PivotMatrix2 with several terms: `terms` is a list of (L, R, W12, W34)."""
        return cls(ctx, sym, None, None, None, None, V, _terms=list(terms))


class PivotMatrix0(_Pivot):
    """0-site (bond) effective Hamiltonian (pivot/DmrgPivotMatrix0.h:10-26)."""

    def __init__(self, ctx, sym, L: Blocks, R: Blocks, V: Blocks):
        super().__init__(ctx, sym, V)
        s, lb, rb, vb = sym.c_struct(), L.c_struct(), R.c_struct(), V.c_struct()
        N.check(N.lib().vmps_pivot0_create(ctx._h, C.byref(s), C.byref(lb), L.data_ptr(), C.byref(rb), R.data_ptr(),
                                           C.byref(vb), C.byref(self._h)))


def HxV(H: _Pivot, Vin: Blocks, Vout: Blocks | None = None, precision="fp64") -> Blocks:
    """Vout = H * Vin; Vout takes Vin's block layout (``Vout = Vin`` then OxV)."""
    out = H.apply(Vin.data, precision)
    if Vout is None:
        return Vin.like(out)
    Vout.data = out
    return Vout


class DeviceVector:
    """A PivotVector resident on the device (Lanczos / benchmark use)."""

    def __init__(self, H: _Pivot, host: np.ndarray | None = None):
        self.H = H
        self._h = C.c_void_p()
        N.check(N.lib().vmps_dvec_create(H._h, C.byref(self._h)))
        if host is not None:
            try:
                self.upload(host)
            except Exception:
                self.close()
                raise

    def upload(self, host):
        host = np.ascontiguousarray(host, dtype=np.float64)
        N.check(N.lib().vmps_dvec_upload(self._h, host.ctypes.data_as(N.f64p)))

    def download(self) -> np.ndarray:
        out = np.empty(self.H.dim)
        N.check(N.lib().vmps_dvec_download(self._h, out.ctypes.data_as(N.f64p)))
        return out

    def dot(self, other) -> float:
        r = C.c_double()
        N.check(N.lib().vmps_dvec_dot(self._h, other._h, C.byref(r)))
        return r.value

    def close(self):
        if self._h:
            N.lib().vmps_dvec_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hxv_device(H: _Pivot, vin: DeviceVector, vout: DeviceVector, precision="fp64"):
    N.check(N.lib().vmps_hxv_device(H._h, vin._h, vout._h, _prec(precision)))


def time_hxv(H: _Pivot, vin: DeviceVector, vout: DeviceVector, precision="fp64", n_iter=10, use_graph=True):
    """(ms per HxV, ms of the second grouped-GEMM phase) from CUDA events."""
    ms, ms2 = C.c_double(), C.c_double()
    N.check(N.lib().vmps_hxv_time(H._h, vin._h, vout._h, _prec(precision), n_iter, int(use_graph), C.byref(ms),
                                  C.byref(ms2)))
    return ms.value, ms2.value


class EnvUpdate:
    """Prepared contract_L / contract_R for fixed block layouts."""

    def __init__(self, ctx: Context, sym: Symmetry, side: str, Eold: Blocks, Abra: Blocks, W: MpoSite, Aket: Blocks,
                 mode: str = "FULL", fixed_ab: int = 0, order: dict | None = None):
        """mode: CONTRACT_LR_MODE (FULL, TRIANGULAR, FIXED_ROWS, FIXED_COLS); order: basis_order_map
        {(aux QN, index inside the sector): position in the full auxiliary basis}."""
        self.ctx, self.sym = ctx, sym
        self._h = C.c_void_p()
        s, eb, bb, kb, wb = sym.c_struct(), Eold.c_struct(), Abra.c_struct(), Aket.c_struct(), W.c_struct()
        sd = N.ENV_LEFT if side == "L" else N.ENV_RIGHT
        items = sorted((order or {}).items())
        qn = np.ascontiguousarray(np.array([list(k[0]) for k, _ in items], dtype=np.int32).reshape(-1, sym.nq))
        idx = np.ascontiguousarray([k[1] for k, _ in items], dtype=np.int32)
        val = np.ascontiguousarray([v for _, v in items], dtype=np.int64)
        N.check(N.lib().vmps_env_create_mode(ctx._h, C.byref(s), sd, N.ENV_MODES[mode], fixed_ab, len(val),
                                             qn.ctypes.data_as(N.i32p), idx.ctypes.data_as(N.i32p),
                                             val.ctypes.data_as(N.i64p), C.byref(eb), C.byref(bb), C.byref(wb),
                                             C.byref(kb), C.byref(self._h)))
        nb, tot = C.c_int64(), C.c_int64()
        N.check(N.lib().vmps_env_layout(self._h, C.byref(nb), C.byref(tot)))
        nq, n = sym.nq, nb.value
        qin = np.zeros((n, nq), np.int32); qout = np.zeros((n, nq), np.int32); qmid = np.zeros((n, nq), np.int32)
        leg = np.zeros(n, np.int32); rows = np.zeros(n, np.int64); cols = np.zeros(n, np.int64)
        off = np.zeros(n, np.int64)
        N.check(N.lib().vmps_env_layout_get(self._h, qin.ctypes.data_as(N.i32p), qout.ctypes.data_as(N.i32p),
                                            qmid.ctypes.data_as(N.i32p), leg.ctypes.data_as(N.i32p),
                                            rows.ctypes.data_as(N.i64p), cols.ctypes.data_as(N.i64p),
                                            off.ctypes.data_as(N.i64p)))
        self.out_layout = Blocks(nq, qin, qout, leg, rows, cols, qmid=qmid, offset=off)

    def stats(self, precision="fp64") -> dict:
        s = N.vmps_plan_stats()
        N.check(N.lib().vmps_env_stats(self._h, _prec(precision), C.byref(s)))
        return s.as_dict()

    def run(self, Eold: Blocks, Abra: Blocks, Aket: Blocks, precision="fp64") -> Blocks:
        out = self.out_layout.like()
        N.check(N.lib().vmps_env_run(self._h, Eold.data_ptr(), Abra.data_ptr(), Aket.data_ptr(), out.data_ptr(),
                                     _prec(precision)))
        return out

    def close(self):
        if self._h:
            N.lib().vmps_env_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def contract_L(ctx, sym, Lold: Blocks, Abra: Blocks, W: MpoSite, Aket: Blocks, precision="fp64") -> Blocks:
    e = EnvUpdate(ctx, sym, "L", Lold, Abra, W, Aket)
    try:
        return e.run(Lold, Abra, Aket, precision)
    finally:
        e.close()


def contract_R(ctx, sym, Rold: Blocks, Abra: Blocks, W: MpoSite, Aket: Blocks, precision="fp64") -> Blocks:
    e = EnvUpdate(ctx, sym, "R", Rold, Abra, W, Aket)
    try:
        return e.run(Rold, Abra, Aket, precision)
    finally:
        e.close()


def left_vacuum(sym: Symmetry) -> Blocks:
    """Tripod::setVacuum: one 1x1 block {vac, vac, vac} = 1 (tensors/Multipede.h:123)."""
    v = sym.vacuum()
    return Blocks.from_entries(sym.nq, [(0, v, v, v, np.ones((1, 1)))], tripod=True)


def right_target(sym: Symmetry, Qtot) -> Blocks:
    """Tripod::setTarget({Qtot, Qtot, vac}) (tensors/Multipede.h:129)."""
    v = sym.vacuum()
    return Blocks.from_entries(sym.nq, [(0, tuple(Qtot), tuple(Qtot), v, np.ones((1, 1)))], tripod=True)
