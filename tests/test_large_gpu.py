"""GPU tests of the large-matrix path (n > 128): whole-GPU Hessenberg reduction and
multishift QR.  Same criteria as the small-matrix tests: hesstest / schurtest
properties (test/real.jl:24-99) with the 10 n eps bounds, and eigenvalues matched to
the oracle's within 1e2 n eps ||A||_F / s_i."""
import numpy as np
import pytest

from common import EPS, assert_schur_real, eig_tolerances, match_eigenvalues, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [3, 40, 150, 300])
def test_hessenberg(gs, n):
    rng = np.random.default_rng(9000 + n)
    A = rng.standard_normal((n, n))
    Hp, tau, Q = gs.hessenberg(A)
    H = np.triu(Hp, -1)
    assert np.linalg.norm(A - Q @ H @ Q.T) / (n * np.linalg.norm(A) * EPS) < 10
    assert np.linalg.norm(np.eye(n) - Q @ Q.T) / (n * EPS) < 10
    # same reflectors as the oracle (up to rounding)
    Ho, tauo, Qo = po.hessenberg(A)
    assert np.max(np.abs(tau - tauo)) < 1e-10


@pytest.mark.parametrize("n", [129, 160, 256, 400])
def test_large_schur_random(gs, n):
    rng = np.random.default_rng(9100 + n)
    A = randn_matrix(rng, n)
    S = gs.gschur(A)
    assert_schur_real(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


@pytest.mark.parametrize("n", [1024])
def test_large_schur_properties(gs, n):
    rng = np.random.default_rng(9200 + n)
    A = randn_matrix(rng, n)
    S = gs.gschur(A)
    assert_schur_real(A, S.T, S.Z, S.values)
    ev = np.linalg.eigvals(A)
    assert np.allclose(np.sort_complex(ev), np.sort_complex(S.values), atol=1e-8 * np.abs(ev).max())


def test_large_orthogonal_and_scaled(gs):
    rng = np.random.default_rng(9300)
    n = 200
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    S = gs.gschur(Q)
    assert_schur_real(Q, S.T, S.Z, S.values)
    A0 = rng.standard_normal((n, n))
    S = gs.gschur(1e300 * A0)
    be = np.linalg.norm(A0 - S.Z @ (S.T / 1e300) @ S.Z.T) / np.linalg.norm(A0)
    assert be <= 10 * n * EPS


def test_large_wantz_false(gs):
    rng = np.random.default_rng(9400)
    A = rng.standard_normal((300, 300))
    S1 = gs.gschur(A)
    S0 = gs.gschur(A, wantZ=False)
    np.testing.assert_array_equal(S0.T, S1.T)


@pytest.mark.parametrize("n", [129, 256])
def test_large_complex_schur(gs, n):
    # the plain CPU-runnable workload's law: one n x n ComplexF64 matrix, re/im iid N(0, 1/2)
    rng = np.random.default_rng(9700 + n)
    A = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(A)
    from common import assert_schur_cplx
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst
