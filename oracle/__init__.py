"""ORACLE -- test infrastructure, not product code.

CPU restatement of the VMPS effective-Hamiltonian path (oracle.cpp) and the
dense exact-diagonalisation pins (ed.py).  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this
package, as the checker.  The GPU engine never imports it.

Symmetries: U(1) and SU(2) components and their products (set_symmetry).

Parity status: the reference (header-only C++ over Eigen, Boost, GSL and the
TNWorkers TOOLS/ALGS headers) cannot be compiled in this environment, and it
ships no numeric golden vectors for this path.  The restatement is therefore
pinned against the reference's own test mechanisms, restated: exact
diagonalisation of small chains (programs/test_Hubbard/test_Hubbard.cc:227-300),
the dense effective Hamiltonian P^T H P of small systems, and
variance / Hermiticity properties (programs/test_Heisenberg/test_Heisenberg.cc:189-192).
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")

_lib = None
_blas_kind = "inhouse"


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(SRC) > os.path.getmtime(LIB):
        tmp = LIB + ".tmp"
        subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp, "-ldl"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def find_openblas():
    """OpenBLAS shared library bundled with the numpy wheel, if any."""
    try:
        d = os.path.dirname(np.__file__)
    except Exception:
        return None
    for pat in ("../numpy.libs/libscipy_openblas*.so*", "../numpy.libs/libopenblas*.so*", ".libs/libopenblas*.so*"):
        hits = sorted(glob.glob(os.path.join(d, pat)))
        if hits:
            return hits[0]
    return None


def lib(use_blas=True):
    global _lib, _blas_kind
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.oracle_pivot_create.restype = C.c_void_p
        _lib.oracle_env_create.restype = C.c_void_p
        _lib.oracle_pivot_tasks.restype = C.c_int64
        _lib.oracle_env_nblocks.restype = C.c_int64
        _lib.oracle_max_threads.restype = C.c_int
        for f in ("oracle_hxv", "oracle_pivot_destroy", "oracle_env_run", "oracle_env_destroy",
                  "oracle_env_layout", "oracle_pivot_tasks", "oracle_env_nblocks"):
            getattr(_lib, f).argtypes = None
        _lib.oracle_set_blas.argtypes = [C.c_char_p]
        _lib.oracle_set_threads.argtypes = [C.c_int]
        _lib.oracle_set_symmetry.argtypes = [C.c_int, C.POINTER(C.c_int32)]
        _lib.oracle_coupling_6j.restype = C.c_double
        _lib.oracle_coupling_6j.argtypes = [C.c_int] * 6
        _lib.oracle_coupling_9j.restype = C.c_double
        _lib.oracle_coupling_9j.argtypes = [C.c_int] * 9
        if use_blas:
            p = find_openblas()
            if p and _lib.oracle_set_blas(p.encode()) > 0:
                _blas_kind = "openblas:" + os.path.basename(p)
    return _lib


def blas_kind():
    lib()
    return _blas_kind


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return lib().oracle_max_threads()


def set_symmetry(nq, kinds=None):
    """QN component kinds of the oracle objects created next: a sequence of "U1" /
    "SU2" (or a vmps_gb300 Symmetry); None means U(1) for every component."""
    if kinds is not None and hasattr(kinds, "kinds"):
        kinds = kinds.kinds
    k = np.zeros(4, dtype=np.int32)
    for i, name in enumerate(kinds or ()):
        k[i] = 1 if name == "SU2" else 0
    lib().oracle_set_symmetry(int(nq), k.ctypes.data_as(C.POINTER(C.c_int32)))


def coupling_6j(*two_j):
    """the oracle's 6j symbol; arguments are 2j"""
    return lib().oracle_coupling_6j(*[int(x) for x in two_j])


def coupling_9j(*two_j):
    """the oracle's 9j symbol; arguments are 2j"""
    return lib().oracle_coupling_9j(*[int(x) for x in two_j])


def _p(a, t=C.c_int32):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def _tab(B, mid=True):
    args = [C.c_int64(B.n), _p(B.qin), _p(B.qout)]
    if mid:
        args.append(_p(B.qmid))
    args += [_p(B.leg), _p(B.rows, C.c_int64), _p(B.cols, C.c_int64), _p(B.offset, C.c_int64)]
    return args


def _mpo(W):
    if W is None:
        return [C.c_int64(0)] + [None] * 8 + [C.c_int(0), None, C.c_int(0), None]
    a = W.arrays()
    return [C.c_int64(W.nnz), _p(a["s1"]), _p(a["s2"]), _p(a["k"]), _p(a["qin"]), _p(a["qout"]), _p(a["row"]),
            _p(a["col"]), _p(a["val"], C.c_double), C.c_int(len(W.qloc)), _p(a["qloc"]), C.c_int(len(W.qop)),
            _p(a["qop"])]


class OraclePivot:
    """kind 1: PivotMatrix1 (W), kind 2: PivotMatrix2 (W, W34), kind 0: PivotMatrix0."""

    def __init__(self, kind, nq, L, R, V, W=None, W34=None, sym=None):
        self.V = V
        self._keep = (L, R, V, W, W34)
        set_symmetry(nq, sym)
        args = [C.c_int(kind), C.c_int(nq)] + _tab(L) + [_p(L.data, C.c_double)] + _tab(R) + \
               [_p(R.data, C.c_double)] + _tab(V, mid=False) + _mpo(W) + _mpo(W34)
        self._h = C.c_void_p(lib().oracle_pivot_create(*args))

    @property
    def n_tasks(self):
        return lib().oracle_pivot_tasks(self._h)

    def hxv(self, vin):
        vin = np.ascontiguousarray(vin, dtype=np.float64)
        out = np.zeros_like(vin)
        lib().oracle_hxv(self._h, _p(vin, C.c_double), _p(out, C.c_double))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_pivot_destroy(self._h)
            self._h = None


def order_arrays(nq, order):
    """basis_order_map {(QN tuple, index in sector): position} as flat arrays"""
    items = sorted(order.items())
    qn = np.array([list(k[0]) for k, _ in items], dtype=np.int32).reshape(-1, nq) if items else np.zeros((0, nq), np.int32)
    idx = np.array([k[1] for k, _ in items], dtype=np.int32)
    val = np.array([v for _, v in items], dtype=np.int64)
    return np.ascontiguousarray(qn), idx, val


MODES = {"FULL": 0, "TRIANGULAR": 1, "FIXED_ROWS": 2, "FIXED_COLS": 3}


class OracleEnv:
    """contract_L (side 'L') / contract_R (side 'R'), with CONTRACT_LR_MODE."""

    def __init__(self, side, nq, E, B, W, K, mode="FULL", fixed_ab=0, order=None, sym=None):
        from vmps_gb300.blocks import Blocks
        set_symmetry(nq, sym)
        qn, idx, val = order_arrays(nq, order or {})
        self._keep = (E, B, W, K, qn, idx, val)
        args = [C.c_int(0 if side == "L" else 1), C.c_int(nq)] + _tab(E) + _tab(B, mid=False) + \
               _tab(K, mid=False) + _mpo(W)[:] + [C.c_int(MODES[mode]), C.c_int64(fixed_ab), C.c_int64(len(val)),
                                                  _p(qn), _p(idx), _p(val, C.c_int64)]
        self._h = C.c_void_p(lib().oracle_env_create(*args))
        n = lib().oracle_env_nblocks(self._h)
        qin = np.zeros((n, nq), np.int32); qout = np.zeros((n, nq), np.int32); qmid = np.zeros((n, nq), np.int32)
        leg = np.zeros(n, np.int32); rows = np.zeros(n, np.int64); cols = np.zeros(n, np.int64)
        off = np.zeros(n, np.int64)
        lib().oracle_env_layout(self._h, _p(qin), _p(qout), _p(qmid), _p(leg), _p(rows, C.c_int64),
                                _p(cols, C.c_int64), _p(off, C.c_int64))
        self.layout = Blocks(nq, qin, qout, leg, rows, cols, qmid=qmid, offset=off)

    def run(self, E, B, K):
        out = self.layout.like()
        lib().oracle_env_run(self._h, _p(E.data, C.c_double), _p(B.data, C.c_double), _p(K.data, C.c_double),
                             _p(out.data, C.c_double))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_env_destroy(self._h)
            self._h = None


def contract_L(nq, Lold, Abra, W, Aket, sym=None):
    return OracleEnv("L", nq, Lold, Abra, W, Aket, sym=sym).run(Lold, Abra, Aket)


def contract_R(nq, Rold, Abra, W, Aket, sym=None):
    return OracleEnv("R", nq, Rold, Abra, W, Aket, sym=sym).run(Rold, Abra, Aket)


def lanczos_ground(hxv, v0, tol=1e-14, max_iter=600, patience=4):
    """Lowest eigenvalue of the symmetric operator `hxv` (a function on flat FP64
    vectors) by plain three-term Lanczos from v0, in numpy.  Without
    reorthogonalisation the basis loses orthogonality once a Ritz value converges,
    which only adds copies of converged values; the lowest Ritz value itself is
    accurate to rounding.  Stops when it changes by less than tol * |E| for
    `patience` consecutive steps.  Returns (E, steps).  Three vectors of memory,
    so it runs at any pivot size the oracle handles; the tridiagonal problem is
    solved with numpy.linalg.eigvalsh."""
    q = np.array(v0, dtype=np.float64, copy=True)
    q /= np.linalg.norm(q)
    q_prev = np.zeros_like(q)
    alpha, beta = [], []
    b = 0.0
    e_old, calm = None, 0
    for j in range(max_iter):
        w = hxv(q)
        a = float(q @ w)
        w -= a * q + b * q_prev
        alpha.append(a)
        b = float(np.linalg.norm(w))
        T = np.diag(alpha) + np.diag(beta, 1) + np.diag(beta, -1)
        e = float(np.linalg.eigvalsh(T)[0])
        if e_old is not None and abs(e - e_old) <= tol * abs(e):
            calm += 1
            if calm >= patience:
                return e, j + 1
        else:
            calm = 0
        e_old = e
        if b == 0.0:
            return e, j + 1
        beta.append(b)
        q_prev, q = q, w / b
    return e_old, max_iter


class OracleTerms:
    """PivotMatrix1/2 with several terms and the excited-state projector, as
    HxV(PivotMatrix1) evaluates them (pivot/DmrgPivotMatrix1.h:273-287 and
    :304-331): the sum of the terms' OxV, then for every projector vector A0_n
    Vout += Epenalty * overlap * A0_n with overlap = sum over blocks of
    tr(A0_n^dagger Vin), the plain Frobenius product of the compact arrays.
    terms: list of (L, R, W) for kind 1 or (L, R, W12, W34) for kind 2."""

    def __init__(self, kind, nq, terms, V, A0proj=(), Epenalty=0.0, sym=None):
        self.ops = [OraclePivot(kind, nq, t[0], t[1], V, *t[2:], sym=sym) for t in terms]
        self.A0 = [np.asarray(a, dtype=np.float64) for a in A0proj]
        self.E = float(Epenalty)

    def hxv(self, vin):
        out = self.ops[0].hxv(vin)
        for op in self.ops[1:]:
            out += op.hxv(vin)
        for a in self.A0:
            out += self.E * float(a @ vin) * a
        return out


def dot_weights(V, sym):
    """sqrt(coeff_dot(qout)) per element of a PivotVector layout (SU(2) components: the
    multiplet dimension q; pivot/DmrgPivotVector.h:296-339 weights every block's
    Frobenius product by it).  Scaling a vector by these turns the weighted dot into
    a plain one, which makes the SU(2) HxV symmetric for a plain Lanczos."""
    kinds = getattr(sym, "kinds", ())
    w = np.ones(V.data.size)
    for i in range(V.n):
        q = 1.0
        for k, name in enumerate(kinds):
            if name == "SU2":
                q *= float(V.qout[i][k])
        o, n = int(V.offset[i]), int(V.rows[i] * V.cols[i])
        w[o:o + n] = np.sqrt(q)
    return w
