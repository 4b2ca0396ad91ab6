"""GPU parity tests of the complex FP64 Schur kernels against the CPU oracle.

Criteria: T upper triangular, values == diag(T) (test/complex.jl:1-34),
||A - Z T Z^H||_F / ||A||_F <= 10 n eps, ||Z^H Z - I||_F <= 10 n eps, eigenvalues
matched to the oracle's within 1e2 n eps ||A||_F / s_i.
"""
import numpy as np
import pytest

from common import EPS, assert_schur_cplx, eig_tolerances, godunov, match_eigenvalues, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 4, 5, 8, 16, 31, 32, 33, 64, 65, 96, 97, 112, 113, 127, 128]


@pytest.mark.parametrize("n", SIZES)
def test_single_random(gs, n):
    rng = np.random.default_rng(2000 + n)
    A = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


def test_batched_mixed_sizes(gs):
    rng = np.random.default_rng(5)
    ns = list(rng.integers(8, 129, size=120)) + [1, 2, 128, 0]
    mats = [randn_matrix(rng, int(n), cplx=True) for n in ns]
    Ts, Zs, ws, status = gs.gschur_batched(mats)
    assert np.all(status == 0)
    for A, T, Z, w in zip(mats, Ts, Zs, ws):
        if A.shape[0]:
            assert_schur_cplx(A, T, Z, w)
    for idx in range(0, len(mats), 13):
        A = mats[idx]
        if A.shape[0] == 0:
            continue
        w_ref, tol = eig_tolerances(A, po)
        ok, worst = match_eigenvalues(ws[idx], w_ref, tol)
        assert ok, "matrix %d: worst %.3g" % (idx, worst)


@pytest.mark.parametrize("n", [4, 32, 120])
def test_unitary_normal(gs, n):
    # random unitary: Schur form is diagonal (test/complex.jl:130-135)
    rng = np.random.default_rng(600 + n)
    Q, R = np.linalg.qr(randn_matrix(rng, n, cplx=True))
    U = Q @ np.diag(np.sign(np.diag(R)))
    S = gs.gschur(U)
    assert_schur_cplx(U, S.T, S.Z, S.values, tol=20.0)
    assert np.linalg.norm(np.triu(S.T, 1)) / (n * np.linalg.norm(U) * EPS) < 20


@pytest.mark.parametrize("n", [4, 32, 128])
def test_jordan(gs, n):
    A = (np.diag(np.ones(n - 1), 1) + np.eye(n)).astype(np.complex128)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values, tol=20.0)


@pytest.mark.parametrize("s", [1e-300, 1e300])
def test_extreme_scaling(gs, s):
    rng = np.random.default_rng(18)
    n = 20
    A0 = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(s * A0)
    be = np.linalg.norm(A0 - S.Z @ (S.T / s) @ S.Z.conj().T) / np.linalg.norm(A0)
    assert be <= 10 * n * EPS
    assert np.all(np.tril(S.T, -1) == 0)


def test_godunov_complex(gs):
    A, vals, econd = godunov()
    A = A.astype(np.complex128)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, worst


def test_real_input_as_complex(gs):
    rng = np.random.default_rng(19)
    A = rng.standard_normal((40, 40)).astype(np.complex128)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)


def test_unconverged_status(gs):
    rng = np.random.default_rng(20)
    A = randn_matrix(rng, 20, cplx=True)
    with pytest.raises(gs.UnconvergedException):
        gs.gschur(A, maxiter=3)
