"""Writes tests/golden/mstag_heisenberg_L12.npz from the reference's own golden
data: programs/test_Heisenberg/ref/Mstag_Jxy=-1_Jz={0,-1,-2,-4}.dat, the staggered
magnetisation (1/L) sum_l (-1)^l <S^z_l>(t) of the L=12 Neel state under the XXZ
chain with Jxy=-1 (programs/test_Heisenberg/test_Heisenberg.cc:279-310, Ldyn=12 at
:97), columns t and M_stag(t), 31 time points at t = 0, 0.2, ..., 6.

Run from the repository root with the reference mounted:
    python tests/golden/make_mstag.py /path/to/reference
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
JZ = (0, -1, -2, -4)


def main(ref_root):
    out = {"Jz": np.array(JZ, dtype=np.float64), "Jxy": np.float64(-1.0), "L": np.int64(12)}
    for jz in JZ:
        path = os.path.join(ref_root, "programs", "test_Heisenberg", "ref", f"Mstag_Jxy=-1_Jz={jz}.dat")
        data = np.loadtxt(path)
        out[f"t_Jz{jz}"] = data[:, 0]
        out[f"mstag_Jz{jz}"] = data[:, 1]
    np.savez(os.path.join(HERE, "mstag_heisenberg_L12.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
