"""Host dense linear algebra of the sweep (the truncated SVD of split_AA2 and the
QR gauge steps): LAPACK through numpy, one sector per host thread.

GB300's FP64 rate makes small dense SVDs (sectors of tens to hundreds of rows)
cheaper on the Grace cores than on the GPU.  numpy's bundled OpenBLAS would
otherwise thread each small call; `SectorPool` pins it to one thread per call
and runs the sectors concurrently (LAPACK releases the GIL), restoring the
previous thread count afterwards.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

_blas = None


def _openblas_paths():
    """Shared-library files of numpy's bundled OpenBLAS."""
    d = os.path.dirname(np.__file__)
    return sorted(glob.glob(os.path.join(d, "..", "numpy.libs", "*openblas*.so*")) +
                  glob.glob(os.path.join(d, ".libs", "*openblas*.so*")))


_native_lapack = None


def native_lapack() -> bool:
    """Bind numpy's ILP64 LAPACK to the native library's host routines (the
    two-site split); False when no bundled OpenBLAS exports them."""
    global _native_lapack
    if _native_lapack is None:
        from . import _native as N
        _native_lapack = False
        for path in _openblas_paths():
            if N.lib().vmps_hostla_load(os.path.abspath(path).encode()) == 0:
                _native_lapack = True
                break
    return _native_lapack


def _openblas_controls():
    """(set_num_threads, get_num_threads) of numpy's bundled OpenBLAS, or None."""
    global _blas
    if _blas is not None:
        return _blas or None
    _blas = False
    for path in _openblas_paths():
        try:
            lib = C.CDLL(path)
        except OSError:
            continue
        for suffix in ("64_", "_64_", ""):
            for pre in ("scipy_openblas", "openblas"):
                try:
                    setf = getattr(lib, f"{pre}_set_num_threads{suffix}")
                    getf = getattr(lib, f"{pre}_get_num_threads{suffix}")
                except AttributeError:
                    continue
                setf.argtypes = [C.c_int]
                getf.restype = C.c_int
                _blas = (setf, getf)
                return _blas
    return None


class SectorPool:
    """Thread pool for independent per-sector LAPACK calls (map(f, items)).  While
    the pool is open, numpy's OpenBLAS runs one thread per call (set once: changing
    OpenBLAS's thread count is not free); close() restores the previous count."""

    def __init__(self, threads: int | None = None):
        self.threads = max(1, threads or min(16, os.cpu_count() or 1))
        self._ex = ThreadPoolExecutor(self.threads) if self.threads > 1 else None
        self._ctl = _openblas_controls() if self._ex is not None else None
        self._prev = None
        if self._ctl:
            self._prev = self._ctl[1]()
            self._ctl[0](1)

    def map(self, f, items):
        items = list(items)
        if self._ex is None or len(items) < 2:
            return [f(x) for x in items]
        # largest sectors first so the pool drains evenly
        order = sorted(range(len(items)), key=lambda i: -getattr(items[i], "size", 0))
        out = [None] * len(items)
        for i, r in zip(order, self._ex.map(lambda i: f(items[i]), order)):
            out[i] = r
        return out

    def close(self):
        if self._ex is not None:
            self._ex.shutdown()
            self._ex = None
        if self._ctl and self._prev is not None:
            self._ctl[0](self._prev)
            self._prev = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
