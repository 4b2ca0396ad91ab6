"""Errors against high precision for the two n = 256 benchmark inputs that carry one:
the 256 x 256 ComplexF64 matrix (iid complex Gaussian, seed 0) and the 256-order
analogue of the precision workload (cond(V) = 1e3, |lambda| log-uniform in
[1e-3, 1e3], seed 6).  The reference states these errors against its own
BigFloat(256-bit) Schur, which needs Julia; the committed fixture
tests/golden/mp256_n256.npz holds the oracle's eigenvalues of the same inputs computed
in 256-bit MPFR arithmetic, BigFloat's precision (tests/golden/make_golden.py).  GPU eigenvalues must lie within
1e2 n eps ||A||_F / s_i of them, the Schur pairs within the FP64 bounds."""
import os

import numpy as np
import pytest

from common import assert_schur_cplx, assert_schur_real, eig_tolerances, match_eigenvalues
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "mp256_n256.npz"))


def test_complex256_vs_bigfloat(gs):
    A = G["A_c256"]
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    _, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, G["w_c256"], tol)
    assert ok, "worst err/tol %.3g" % worst


@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_conditioned256_vs_bigfloat(gs, form):
    A = G["A_cond256"]
    S = gs.gschur(A) if form == "fp64" else gs.gschur_mixed(A)
    assert_schur_real(A, S.T, S.Z, S.values)
    _, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, G["w_cond256"], tol)
    assert ok, "worst err/tol %.3g" % worst
