"""Native two-site split (vmps_two_site_split) against the numpy restatement of
split_AA2 / Biped::truncateSVD (tensors/DmrgContractions.h:2461-2631,
tensors/Biped.h:744-932): same middle bond basis, same block layout, the same
two-site tensor after truncation, orthonormal factors.  Host code only."""
import numpy as np
import pytest

from vmps_gb300 import models
from vmps_gb300.hostla import SectorPool, native_lapack
from vmps_gb300.mps import RandomMPS, contract_two_sites, split_two_site

VMPS_E_ARG = -1   # include/vmps_gb300.h


def _case(L, D, l, seed, kind="hubbard", sigma=1.5):
    if kind == "hubbard":
        model = models.hubbard_u1xu1(L, t=1.0, U=4.0)
        mps = RandomMPS(model, (L, 0), D, seed=seed, profile="gaussian", sigma=[2.5, 2.5]).canonicalize(l, l)
    else:   # spin-1/2 chain: few, large sectors (Gram matrices of order 256 and more at D=512)
        model = models.heisenberg_u1(L)
        mps = RandomMPS(model, (0,), D, seed=seed, profile="gaussian", sigma=[sigma]).canonicalize(l, l)
    A1, A2 = mps.A[l], mps.A[l + 1]
    din = {tuple(A1.qin[i]): int(A1.rows[i]) for i in range(A1.n)}
    dout = {tuple(A2.qout[i]): int(A2.cols[i]) for i in range(A2.n)}
    V, comb = contract_two_sites(model.sym, A1, A2, model.qloc, model.qloc, model.sym.nq, return_basis=True)
    return model, V, comb, din, dout


def _product(A1, A2):
    out = {}
    for i in range(A1.n):
        for j in range(A2.n):
            if tuple(A1.qout[i]) == tuple(A2.qin[j]):
                k = (int(A1.leg[i]), int(A2.leg[j]), tuple(A1.qin[i]), tuple(A2.qout[j]))
                out[k] = out.get(k, 0) + A1.block(i) @ A2.block(j)
    return out


@pytest.mark.parametrize("move", ["right", "left"])
@pytest.mark.parametrize("dmax", [24, 64])
@pytest.mark.parametrize("threads", [1, 4])
def test_native_split_matches_numpy(move, dmax, threads):
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    model, V, comb, din, dout = _case(10, 64, 4, seed=5)
    pool = SectorPool(threads)
    try:
        a = split_two_site(V, comb, model.qloc, model.qloc, din, dout, 2, dmax, move=move, pool=pool, native=False)
        b = split_two_site(V, comb, model.qloc, model.qloc, din, dout, 2, dmax, move=move, pool=pool, native=True)
    finally:
        pool.close()
    assert a[3] == b[3] and sum(b[3].values()) <= dmax
    assert abs(a[2] - b[2]) < 1e-13
    for X, Y in ((a[0], b[0]), (a[1], b[1])):
        for f in ("leg", "qin", "qout", "rows", "cols", "offset"):
            assert np.array_equal(getattr(X, f), getattr(Y, f)), f
    pa, pb = _product(a[0], a[1]), _product(b[0], b[1])
    assert pa.keys() == pb.keys()
    assert max(np.abs(pa[k] - pb[k]).max() for k in pa) < 1e-12
    # the orthonormal factor of the sweep direction
    Q = b[0] if move == "right" else b[1]
    for qm in b[3]:
        blks = [Q.block(i) for i in range(Q.n) if tuple((Q.qout if move == "right" else Q.qin)[i]) == qm]
        M = np.vstack(blks) if move == "right" else np.hstack(blks)
        G = M.T @ M if move == "right" else M @ M.T
        assert np.abs(G - np.eye(len(G))).max() < 1e-12


@pytest.mark.parametrize("move", ["right", "left"])
@pytest.mark.parametrize("D,sigma,least", [(512, 1.5, 256), (1024, 1.0, 512)])
def test_native_split_large_sectors(move, D, sigma, least):
    """Sectors of Gram order >= 256 take the tridiagonal path (kept eigenvectors
    only); the result matches the numpy restatement."""
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    model, V, comb, din, dout = _case(24, D, 11, seed=3, kind="heisenberg", sigma=sigma)
    rows = {}
    for s1, q1 in enumerate(model.qloc):
        for q, d in din.items():
            qm = tuple(a + b for a, b in zip(q, q1))
            rows[qm] = rows.get(qm, 0) + d
    cols = {}
    for s3, q3 in enumerate(model.qloc):
        for q, d in dout.items():
            qm = tuple(a - b for a, b in zip(q, q3))
            cols[qm] = cols.get(qm, 0) + d
    order = max(rows.values()) if move == "right" else max(cols.values())
    assert order >= least
    pool = SectorPool(4)
    try:
        for dmax in (D // 4, (3 * D) // 5):
            a = split_two_site(V, comb, model.qloc, model.qloc, din, dout, 1, dmax, move=move, pool=pool,
                               native=False)
            b = split_two_site(V, comb, model.qloc, model.qloc, din, dout, 1, dmax, move=move, pool=pool,
                               native=True)
            assert a[3] == b[3] and abs(a[2] - b[2]) < 1e-13
            pa, pb = _product(a[0], a[1]), _product(b[0], b[1])
            scale = max(np.abs(pa[k]).max() for k in pa)
            # the kept subspace is determined to eps * |G| / (gap at the cut)
            assert max(np.abs(pa[k] - pb[k]).max() for k in pa) < 1e-9 * scale
    finally:
        pool.close()


def test_native_split_rejects_bad_leg():
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    from vmps_gb300 import _native as N
    model, V, comb, din, dout = _case(6, 16, 2, seed=1)
    bad = dict(comb)
    bad["n"] = 1
    bad["index"] = {k: [(q, 0) for q, _ in v] for k, v in comb["index"].items()}
    V.leg[:] = 3
    with pytest.raises(N.VmpsError):
        split_two_site(V, bad, model.qloc, model.qloc, din, dout, 2, 16, native=True)


@pytest.mark.parametrize("move", ["right", "left"])
@pytest.mark.parametrize("kind", ["hubbard", "su2"])
def test_native_gauge_step_matches_numpy(move, kind):
    """vmps_gauge_step (QR / LQ per sector and the neighbour's factor) against
    left/right_normalize with the factor pushed by numpy"""
    import copy
    from vmps_gb300.dmrg import _push_left, _push_right
    from vmps_gb300.mps import gauge_step, left_normalize, right_normalize
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    if kind == "hubbard":
        model = models.hubbard_u1xu1(10, t=1.0, U=4.0)
        mps = RandomMPS(model, (10, 0), 64, seed=4, profile="gaussian", sigma=[2.5, 2.5]).canonicalize(4, 4)
    else:
        model = models.heisenberg_su2(10)
        mps = RandomMPS(model, (1,), 24, seed=4).canonicalize(4, 4)
    nq, sym = model.sym.nq, mps.sym
    l = 4
    nb = l + 1 if move == "right" else l - 1
    A, N = copy.deepcopy(mps.A[l]), copy.deepcopy(mps.A[nb])
    if move == "right":
        Q, R = left_normalize(A, nq, sym=sym)
        _push_right(N, R)
    else:
        Q, Lf = right_normalize(A, nq, sym=sym)
        _push_left(N, Lf)
    A2, N2 = copy.deepcopy(mps.A[l]), copy.deepcopy(mps.A[nb])
    pool = SectorPool(4)
    try:
        gauge_step(A2, N2, nq, move, sym=sym, pool=pool)
    finally:
        pool.close()
    assert np.abs(Q.data - A2.data).max() < 1e-13
    assert np.abs(N.data - N2.data).max() < 1e-12 * np.abs(N.data).max()


def test_native_split_edge_cases():
    """Dmax = 0 keeps nothing; a two-site tensor without blocks gives empty sites;
    a sector with a quantum number out of the packed range is refused (host
    threads report the error to the caller instead of ending the process)"""
    from vmps_gb300 import _native as N
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    model, V, comb, din, dout = _case(8, 32, 3, seed=2)
    a = split_two_site(V, comb, model.qloc, model.qloc, din, dout, 2, 0, native=False)
    b = split_two_site(V, comb, model.qloc, model.qloc, din, dout, 2, 0, native=True)
    assert a[3] == b[3] == {} and b[0].n == 0 and b[1].n == 0
    empty = V.like()
    empty.data[:] = 0
    e = split_two_site(empty, comb, model.qloc, model.qloc, din, dout, 2, 16, native=True)
    assert e[3] == {} and e[2] == 0.0
    big = {(q[0] + 40000, q[1]): d for q, d in din.items()}
    with pytest.raises(N.VmpsError):
        split_two_site(V, comb, model.qloc, model.qloc, big, dout, 2, 16, native=True)


def test_host_routines_refuse_bad_tables():
    """malformed tables or arguments come back as VMPS_E_ARG (-1), nothing is read"""
    import ctypes as C
    from vmps_gb300 import _native as N
    from vmps_gb300.blocks import Blocks
    if not native_lapack():
        pytest.skip("numpy's bundled OpenBLAS exports no ILP64 LAPACK")
    lib = N.lib()
    A = Blocks(1, [[0]], [[1]], [0], [3], [2])
    bad = Blocks(1, [[0]], [[1]], [0], [3], [2])
    bad.rows[0] = 0                      # non-positive shape
    ab, bb = A.c_struct(), bad.c_struct()
    rc = lib.vmps_gauge_step(1, 1, C.byref(bb), bad.data_ptr(), C.cast(None, N.f64p), C.byref(ab), A.data_ptr(), 1)
    assert rc == VMPS_E_ARG
    nul = N.vmps_blocks()
    nul.nblocks = 1                       # arrays left null
    rc = lib.vmps_gauge_step(1, 1, C.byref(nul), A.data_ptr(), C.cast(None, N.f64p), C.byref(ab), A.data_ptr(), 1)
    assert rc == VMPS_E_ARG
    args = N.vmps_split_args()
    q = np.zeros(1, np.int32)
    pair = np.zeros(1, np.int32)
    args.nq, args.n1, args.n3, args.n13 = 1, 1, 1, 1
    args.qloc1 = args.qloc3 = q.ctypes.data_as(N.i32p)
    args.pair1 = args.pair3 = pair.ctypes.data_as(N.i32p)
    args.nin = 1                          # a left basis without its arrays
    args.dmax, args.threads = 4, 1
    h = C.c_void_p()
    rc = lib.vmps_two_site_split(C.byref(args), C.byref(ab), A.data_ptr(), C.byref(h))
    assert rc == VMPS_E_ARG and not h.value


@pytest.mark.parametrize("kind,D,l", [("hubbard", 256, 5), ("heisenberg", 64, 6), ("su2", 32, 6)])
def test_two_site_layout_matches_direct_loop(kind, D, l):
    """two_site_layout (pairs made once per merged QN) gives the table of the direct
    loop over (s1s3, sorted qin, fused qout), block for block"""
    from vmps_gb300.mps import combined_basis, two_site_layout
    if kind == "hubbard":
        model, Q = models.hubbard_u1xu1(12, t=1.0, U=4.0), (12, 0)
    elif kind == "heisenberg":
        model, Q = models.heisenberg_u1(14), (0,)
    else:
        model, Q = models.heisenberg_su2(14), (1,)
    mps = RandomMPS(model, Q, D, seed=2)
    din, dout = mps.dims[l], mps.dims[l + 2]
    V, comb = two_site_layout(model.sym, model.qloc, model.qloc, din, dout, model.sym.nq)
    assert comb == combined_basis(model.sym, model.qloc, model.qloc)
    ent = []
    for s13, qm in enumerate(comb["q_of"]):
        for qin in sorted(din):
            for qout in model.sym.fuse(qin, qm):
                if qout in dout:
                    ent.append((s13, qin, qout, din[qin], dout[qout]))
    assert V.n == len(ent) > 0
    for i, (s13, qin, qout, r, c) in enumerate(ent):
        assert (int(V.leg[i]), tuple(V.qin[i]), tuple(V.qout[i]), int(V.rows[i]), int(V.cols[i])) == \
            (s13, qin, qout, r, c)
