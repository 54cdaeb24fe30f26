"""The oracle's VUMPS transfer operator (oracle/vumps_cpu.py) on the CPU: it is
linear, and with a zero cell (T = 0) it reduces to Vin + contract_LR(ab, Vin, LR) * 1
on the slot-ab blocks (VUMPS/VumpsMpoTransferMatrix.h:168-210)."""
import numpy as np

from oracle.vumps_cpu import transfer_hxv

from helpers import oracle_envs
from vumps_case import transfer_case


def _case(direction):
    return transfer_case("heis", direction, envs=lambda m, mps: oracle_envs(m, mps, 9, 10))


def test_oracle_transfer_is_linear():
    for direction in ("L", "R"):
        m, mps, (A, W), LR, order, V = _case(direction)
        rng = np.random.default_rng(1)
        u, v = rng.standard_normal(V.data.size), rng.standard_normal(V.data.size)
        f = lambda x: transfer_hxv(direction, 1, A, A, W, LR, 0, order, V, x, m.sym.dot_weight)
        assert np.allclose(f(3 * u - v), 3 * f(u) - f(v), atol=1e-10)


def test_oracle_transfer_zero_cell_is_identity_plus_projector():
    m, mps, (A, W), LR, order, V = _case("L")
    Z = [a.like() for a in A]
    v = np.random.default_rng(2).standard_normal(V.data.size)
    got = transfer_hxv("L", 1, Z, Z, W, LR, 0, order, V, v, m.sym.dot_weight)
    inv = {p: k for k, p in order.items()}
    q0, i0 = inv[0]
    # by hand: LdotR = sum over vacuum-mid, slot-0, diagonal-QN blocks of tr(V LR)
    ldotr = 0.0
    lr = {tuple(LR.qin[i]): LR.block(i) for i in range(LR.n)}
    for i in range(V.n):
        if tuple(V.qmid[i]) == tuple(q0) and V.leg[i] == i0 and tuple(V.qin[i]) == tuple(V.qout[i]):
            blk = v[V.offset[i]:V.offset[i] + V.rows[i] * V.cols[i]].reshape(V.cols[i], V.rows[i]).T
            ldotr += np.trace(blk @ lr[tuple(V.qin[i])])
    # T V = 0: every slot-ab block that T V shares with Vin becomes Vin + LdotR * 1; all else is zero
    matched = 0
    mask = np.zeros(V.data.size, dtype=bool)
    for i in range(V.n):
        sl = slice(V.offset[i], V.offset[i] + V.rows[i] * V.cols[i])
        if not (tuple(V.qmid[i]) == tuple(q0) and V.leg[i] == i0):
            continue
        mask[sl] = True
        g = got[sl].reshape(V.cols[i], V.rows[i]).T
        if np.allclose(g, 0.0):
            continue
        blk = v[sl].reshape(V.cols[i], V.rows[i]).T
        assert np.allclose(g, blk + ldotr * np.eye(V.rows[i], V.cols[i]), atol=1e-12)
        matched += 1
    assert matched > 0 and abs(ldotr) > 0
    assert np.allclose(got[~mask], 0.0)
