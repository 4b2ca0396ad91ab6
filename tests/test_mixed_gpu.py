"""GPU tests of the mixed-precision form: FP32 Schur + FP64 Newton refinement.
Same acceptance as the FP64 path (equal backward error <= 10 n eps_64):
standard-form quasi-triangular T, ||A - Z T Z^T||_F/||A||_F <= 10 n eps,
||Z^T Z - I||_F <= 10 n eps, eigenvalues matched to the oracle's."""
import numpy as np
import pytest

from common import EPS, assert_schur_real, eig_tolerances, match_eigenvalues, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [60, 150, 300, 600])
def test_mixed_random(gs, n):
    rng = np.random.default_rng(9500 + n)
    A = randn_matrix(rng, n)
    S, info = gs.gschur_mixed(A, return_info=True)
    assert info["residual"] <= 10 * n * EPS
    assert_schur_real(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


def test_mixed_scaled_input(gs):
    rng = np.random.default_rng(9600)
    n = 200
    A0 = randn_matrix(rng, n)
    for s in (1e-200, 1e200):
        S = gs.gschur_mixed(s * A0)
        be = np.linalg.norm(A0 - S.Z @ (S.T / s) @ S.Z.T) / np.linalg.norm(A0)
        assert be <= 10 * n * EPS


def test_mixed_conditioned_matrix(gs):
    """The precision workload's law at n=256: A = V diag(l) V^-1, |l| log-uniform in
    [1e-3, 1e3] with random signs, cond(V) = 1e3.  The small eigenvalues sit closer
    together than FP32 resolves them relative to ||A||, so the refinement may not
    converge: then the strict form reports non-convergence (never a silent miss) and
    the default form returns the FP64 recomputation, which meets the FP64 bounds."""
    from genericschur_gb300.workloads import conditioned_matrix
    A = conditioned_matrix(256, seed=6)
    try:
        S = gs.gschur_mixed(A, fallback=False)
        assert_schur_real(A, S.T, S.Z, S.values)
    except gs.UnconvergedException:
        pass
    S, info = gs.gschur_mixed(A, return_info=True)
    assert info["iterations"] >= -1
    assert_schur_real(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


def test_mixed_refinement_steps(gs):
    """Newton refinement converges quadratically from an FP32 start: at most three
    corrections reach the rounding level on a Gaussian matrix."""
    rng = np.random.default_rng(9700)
    A = randn_matrix(rng, 400)
    S, info = gs.gschur_mixed(A, return_info=True)
    assert 1 <= info["iterations"] <= 3
    assert info["residual"] <= 10 * 400 * EPS
