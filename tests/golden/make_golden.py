"""Generate tests/golden/oracle_golden.npz: seeded inputs and the CPU oracle's
outputs (T, Z, eigenvalues).  The reference (Julia) cannot run in this build
environment, so these fixtures pin the oracle against regressions only; the
oracle's agreement with the reference rests on the reference's own known answers
and property tests (tests/test_oracle.py).

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from common import godunov  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    for n in (1, 2, 3, 5, 8, 16):
        out["A_r%d" % n] = np.asfortranarray(rng.standard_normal((n, n)))
        out["A_c%d" % n] = np.asfortranarray((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2))
    out["A_godunov"] = np.asfortranarray(godunov()[0])
    for key in list(out):
        tag = key[2:]
        T, Z, w = po.gschur(out[key])
        out["T_" + tag], out["Z_" + tag], out["w_" + tag] = T, Z, w
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
