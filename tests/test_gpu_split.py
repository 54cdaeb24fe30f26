"""The two-site split with its large sectors on the GPU in FP64
(vmps_two_site_split_device: cuBLAS dsyrk for the Gram matrix, cuSOLVER dsyevd for
its eigensystem, cuBLAS dgemm for the non-orthonormal factor) against the host
routine (LAPACK) on the same two-site tensors: the same middle bond basis and
block layout, the kept singular spectrum and discarded weight to 1e-12, the same
truncated two-site tensor to 1e-12 (eigenvector signs may differ), orthonormal
factors.  The device threshold is lowered so that most sectors take the device
path, and left at its default for the D=1024 case.  The cuts keep singular values
well above the Gram matrices' resolution (about 1e-8 of the largest value: the
Gram matrix squares them), with a gap at the cut: states below that resolution
are determined by rounding alone, in either routine."""
import numpy as np
import pytest

from vmps_gb300.hostla import SectorPool, native_lapack
from vmps_gb300.mps import split_two_site

from test_hostla import _case, _product

pytestmark = pytest.mark.gpu


def _compare(a, b, move, dmax):
    assert a[3] == b[3] and sum(b[3].values()) <= dmax
    assert abs(a[2] - b[2]) <= 1e-12 * max(a[2], 1e-300) + 1e-15
    for X, Y in ((a[0], b[0]), (a[1], b[1])):
        for f in ("leg", "qin", "qout", "rows", "cols", "offset"):
            assert np.array_equal(getattr(X, f), getattr(Y, f)), f
    pa, pb = _product(a[0], a[1]), _product(b[0], b[1])
    assert pa.keys() == pb.keys()
    scale = max(np.abs(pa[k]).max() for k in pa)
    assert max(np.abs(pa[k] - pb[k]).max() for k in pa) < 1e-12 * scale
    Q = b[0] if move == "right" else b[1]
    for qm in b[3]:
        blks = [Q.block(i) for i in range(Q.n) if tuple((Q.qout if move == "right" else Q.qin)[i]) == qm]
        M = np.vstack(blks) if move == "right" else np.hstack(blks)
        G = M.T @ M if move == "right" else M @ M.T
        assert np.abs(G - np.eye(len(G))).max() < 1e-12


@pytest.mark.parametrize("move", ["right", "left"])
@pytest.mark.parametrize("kind,L,D,l,gmin,dmax", [("hubbard", 12, 256, 5, "16", 200),
                                                  ("heisenberg", 24, 1024, 11, "512", 301)])
def test_device_split_matches_host(gpu_ctx, monkeypatch, move, kind, L, D, l, gmin, dmax):
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    model, V, comb, din, dout = _case(L, D, l, seed=3, kind=kind, sigma=1.0)
    monkeypatch.setenv("VMPS_SPLIT_GPU_MIN", gmin)
    monkeypatch.setenv("VMPS_SPLIT_DEVICE", "all")   # every sector of order >= gmin on the device
    pool = SectorPool(4)
    try:
        nq = model.sym.nq
        a = split_two_site(V, comb, model.qloc, model.qloc, din, dout, nq, dmax, move=move, pool=pool)
        b = split_two_site(V, comb, model.qloc, model.qloc, din, dout, nq, dmax, move=move, pool=pool, ctx=gpu_ctx)
        c = split_two_site(V, comb, model.qloc, model.qloc, din, dout, nq, dmax, move=move, pool=pool, ctx=gpu_ctx)
    finally:
        pool.close()
    _compare(a, b, move, dmax)
    # deterministic: a second device split gives the same bits
    assert np.array_equal(b[0].data, c[0].data) and np.array_equal(b[1].data, c[1].data)
