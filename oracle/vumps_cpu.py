"""ORACLE -- test infrastructure, not product code.

HxV(MpoTransferMatrix, Vin, Vout) of VUMPS/VumpsMpoTransferMatrix.h:99-212 on
the CPU oracle: the cell chain of contract_L / contract_R (the oracle's literal
restatement of tensors/DmrgContractions.h:35-311 with CONTRACT_LR_MODE), the
scalar contract_LR(ab, L, R) of DmrgContractions.h:995-1053 and the update
Vout[slot ab] = Vin - T Vin + LdotR * 1 of :168-210, in plain numpy.
"""
from __future__ import annotations

import numpy as np

from . import OracleEnv


def _blocks(B):
    out = {}
    for i in range(B.n):
        key = (tuple(B.qin[i]), tuple(B.qout[i]))
        if B.qmid is not None:
            key = key + (tuple(B.qmid[i]), int(B.leg[i]))
        out[key] = B.data[B.offset[i]:B.offset[i] + B.rows[i] * B.cols[i]].reshape(B.cols[i], B.rows[i]).T
    return out


def transfer_hxv(direction, nq, Abra, Aket, W, LReigen, ab, order, V, vin, dot_weight, sym=None):
    """direction 'L' / 'R'; Abra/Aket/W: cell site tensors; LReigen: Biped; V: Tripod layout, vin its data;
    sym: the symmetry's component kinds (None: U(1) throughout)"""
    inv = {v: k for k, v in order.items()}
    abq, abi = inv[ab]
    n = len(W)
    E = V.like(np.array(vin, dtype=np.float64))
    sites = range(n) if direction == "L" else range(n - 1, -1, -1)
    for l in sites:
        if direction == "L":
            mode = "FIXED_COLS" if l == n - 1 else ("FIXED_ROWS" if l == 0 else "FULL")
        else:
            mode = "FIXED_ROWS" if l == 0 else ("FIXED_COLS" if l == n - 1 else "FULL")
        env = OracleEnv(direction, nq, E, Abra[l], W[l], Aket[l], mode=mode, fixed_ab=ab, order=order, sym=sym)
        E = env.run(E, Abra[l], Aket[l])
    T = _blocks(E)
    Vb = _blocks(V.like(np.array(vin, dtype=np.float64)))
    LR = _blocks(LReigen)
    vac = tuple(abq)
    # contract_LR: vacuum-mid blocks of Vin at slot ab with in == out, against LReigen(out, in)
    ldotr = 0.0
    for (qi, qo, qm, leg), blk in Vb.items():
        if qm == vac and leg == abi and qi == qo and (qo, qi) in LR:
            ldotr += np.trace(blk @ LR[(qo, qi)]) * dot_weight(qo)
    out = V.like()
    ob = _blocks(out)
    for key, tb in T.items():
        qi, qo, qm, leg = key
        if qm != tuple(abq) or leg != abi or key not in Vb:
            continue
        vb = Vb[key]
        ob[key][...] = vb - tb + ldotr * np.eye(*vb.shape)
    # write back (the views in ob are transposed views of out.data)
    for i in range(out.n):
        key = (tuple(out.qin[i]), tuple(out.qout[i]), tuple(out.qmid[i]), int(out.leg[i]))
        out.data[out.offset[i]:out.offset[i] + out.rows[i] * out.cols[i]] = ob[key].T.ravel()
    return out.data
