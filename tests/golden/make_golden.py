"""Generate tests/golden/oracle_golden.npz: seeded inputs and the CPU oracle's
outputs (T, Z, eigenvalues); and tests/golden/quad_256.npz: the two n = 256
benchmark inputs that carry a high-precision error statement -- one 256 x 256
ComplexF64 matrix with iid complex Gaussian entries (real and imaginary parts
N(0, 1/2), seed 0) and the 256-order analogue of the precision workload
(A = V diag(l) V^-1, |l| log-uniform in [1e-3, 1e3], cond(V) = 1e3, seed 6) --
with their eigenvalues from the oracle run in 113-bit arithmetic (rounded to
FP64) and that run's backward and orthogonality errors.  The reference (Julia) cannot run in this build
environment, so these fixtures pin the oracle against regressions only; the
oracle's agreement with the reference rests on the reference's own known answers
and property tests (tests/test_oracle.py).

Usage: python tests/golden/make_golden.py [mp256]
(mp256 alone regenerates only tests/golden/mp256_n256.npz, the 256-bit fixture.)
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
    quad()


def quad():
    sys.path.insert(0, os.path.join(ROOT, "genericschur.jl_gb300"))
    from genericschur_gb300.workloads import conditioned_matrix
    n = 256
    rng = np.random.default_rng(0)
    Ac = np.asfortranarray((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2))
    _, _, wc, resc = po.gschur_cplx_quad(Ac)
    Ar = conditioned_matrix(n, seed=6)
    _, _, wr, resr = po.gschur_quad(Ar)
    np.savez_compressed(os.path.join(HERE, "quad_256.npz"), A_c256=Ac, w_c256=wc, res_c256=np.array(resc),
                        A_cond256=Ar, w_cond256=wr, res_cond256=np.array(resr))
    print("quad residuals", resc, resr)


def mp256():
    """tests/golden/mp256_n256.npz: the same two n = 256 inputs decomposed by the oracle in
    256-bit MPFR arithmetic -- BigFloat's default precision, which the reference's own
    high-precision Schur runs use -- eigenvalues rounded to FP64, and that run's
    backward and orthogonality errors (needs libmpfr.so.6; about ten minutes)."""
    sys.path.insert(0, os.path.join(ROOT, "genericschur.jl_gb300"))
    from genericschur_gb300.workloads import conditioned_matrix
    n = 256
    rng = np.random.default_rng(0)
    Ac = np.asfortranarray((rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2))
    _, _, wc, resc = po.gschur_cplx_mp(Ac)
    Ar = conditioned_matrix(n, seed=6)
    _, _, wr, resr = po.gschur_mp(Ar)
    np.savez_compressed(os.path.join(HERE, "mp256_n256.npz"), A_c256=Ac, w_c256=wc, res_c256=np.array(resc),
                        A_cond256=Ar, w_cond256=wr, res_cond256=np.array(resr))
    print("256-bit residuals", resc, resr)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "mp256":
        mp256()
    else:
        main()
        mp256()
