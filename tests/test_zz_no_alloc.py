"""GPU test of vmps_chain_fp64_noalloc, the entry point for callers that cannot
allocate device memory (see include/vmps_gb300.h).  Its result must equal what
the regular HxV(PivotMatrix0) path computes for the same single-block product,
on two calls in a row that reuse the library's fixed scratch array.  This file
is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from vmps_gb300 import _native as N
from vmps_gb300.blocks import Blocks, Symmetry
from vmps_gb300.pivot import Context, PivotMatrix0

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _dev(torch, a):
    """column-major copy of a numpy matrix in device memory (test-side allocation)"""
    return torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()


def _noalloc(X, xr, xc, tx, Y, yr, yc, Z, zr, zc, tz, alpha, out):
    return N.lib().vmps_chain_fp64_noalloc(C.c_void_p(X.data_ptr()), xr, xc, tx, C.c_void_p(Y.data_ptr()), yr, yc,
                                          C.c_void_p(Z.data_ptr()), zr, zc, tz, alpha, C.c_void_p(out.data_ptr()),
                                          None)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_chain_matches_pivot0_hxv(native_lib):
    torch = pytest.importorskip("torch")
    ctx = Context(0)
    rng = np.random.default_rng(11)
    m, n = 300, 200
    sym = Symmetry(("U1",))
    v = (0,)
    for call in range(2):   # two calls in a row share the scratch array
        X = rng.standard_normal((m, m))
        Y = rng.standard_normal((m, n))
        Z = rng.standard_normal((n, n))
        # regular path: HxV(PivotMatrix0) with one L block, one R block, one C block
        L = Blocks.from_entries(1, [(0, v, v, v, X)], tripod=True)
        R = Blocks.from_entries(1, [(0, v, v, v, Z)], tripod=True)
        Cb = Blocks.from_entries(1, [(0, v, v, Y)])
        H = PivotMatrix0(ctx, sym, L, R, Cb)
        ref = H.apply(Cb.data, "fp64").reshape((m, n), order="F")
        H.close()
        dX, dY, dZ = _dev(torch, X), _dev(torch, Y), _dev(torch, Z)
        dO = torch.zeros(m * n, dtype=torch.float64, device="cuda")
        rc = _noalloc(dX, m, m, 0, dY, m, n, dZ, n, n, 0, 1.0, dO)
        assert rc == 0, N.lib().vmps_last_error()
        torch.cuda.synchronize()
        got = dO.cpu().numpy().reshape((m, n), order="F")
        assert _rel(got, ref) < TOL_FP64, (call, _rel(got, ref))
    ctx.close()


def test_noalloc_transposes_and_scale(native_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    m, k, n, p = 97, 130, 61, 45
    X = rng.standard_normal((k, m))   # op(X) = X^T
    Y = rng.standard_normal((k, n))
    Z = rng.standard_normal((p, n))   # op(Z) = Z^T
    dX, dY, dZ = _dev(torch, X), _dev(torch, Y), _dev(torch, Z)
    dO = torch.zeros(m * p, dtype=torch.float64, device="cuda")
    for alpha in (1.0, -0.375):
        assert _noalloc(dX, k, m, 1, dY, k, n, dZ, p, n, 1, alpha, dO) == 0, N.lib().vmps_last_error()
        torch.cuda.synchronize()
        got = dO.cpu().numpy().reshape((m, p), order="F")
        assert _rel(got, alpha * (X.T @ Y @ Z.T)) < TOL_FP64


def test_noalloc_rejects_oversized_intermediate(native_lib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    # op(X) * Y would be 2048 x 1024 = 2^21 elements > 2^20: refused before any launch
    rc = _noalloc(buf, 2048, 4, 0, buf, 4, 1024, buf, 1024, 4, 0, 1.0, buf)
    assert rc == -1
    assert b"scratch" in N.lib().vmps_last_error()
    # shapes that do not chain
    rc = _noalloc(buf, 4, 3, 0, buf, 4, 2, buf, 2, 2, 0, 1.0, buf)
    assert rc == -4
