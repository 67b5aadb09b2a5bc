"""Golden cases: the problem dict for each fixture in tests/golden/ (the same
parameters make_golden.py passes to the reference harness)."""
import os

import numpy as np

from pansfem2_gb300 import problems as PB

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES = {
    "cantilever_12x6_oc": lambda: PB.cantilever_q4(12, 6),
    "cantilever_60x30_oc": lambda: PB.cantilever_q4(60, 30),
    "mbb_16x8_mma": lambda: PB.mbb_q4(16, 8),
    "mbb_48x24_mma": lambda: PB.mbb_q4(48, 24),
    "heatsink_10x10_oc": lambda: PB.heatsink_q4(10, 10, patch_w=1, patch_i0=4),
    "cantilever_h8_6x3x3_oc": lambda: PB.cantilever_h8(6, 3, 3, vf=0.3, R=1.5),
    "cantilever_12x6_heaviside": lambda: PB.cantilever_q4(12, 6, heaviside=1),
    "cantilever_60x40_conlin": lambda: PB.conlin_cantilever_q4(60, 40),
}


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}
