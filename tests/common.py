"""Property checks and parity criteria shared by the tests.

The checks restate GenericSchur.jl's own test helpers:
  checkblocks       test/real.jl:3-22
  schurtest         test/real.jl:24-74, test/complex.jl:1-34
  checkeigvals      test/testfuncs.jl:57-86
  vectest           test/testfuncs.jl:5-54
plus the parity criteria for results of this library against the oracle:
  matched eigenvalues |l_gpu - l_ref| <= 1e2 * n * eps * ||A||_F / s_i, with s_i the
  reciprocal condition of eigenvalue i (rconde, pirates.jl:107-113, from the
  oracle's left and right eigenvectors); ||A - Z T Z^H||_F / ||A||_F <= 10 n eps;
  ||Z^H Z - I||_F <= 10 n eps.
"""
import numpy as np
from scipy.optimize import linear_sum_assignment

EPS = np.finfo(np.float64).eps


def checkblocks(T):
    n = T.shape[0]
    for j in range(n - 1):
        if T[j + 1, j] != 0:
            if not (T[j, j] == T[j + 1, j + 1] and T[j, j + 1] != 0 and np.sign(T[j, j + 1]) * np.sign(T[j + 1, j]) < 0):
                return False
    return True


def checkeigvals(T, w, tol):
    n = T.shape[0]
    ulp = EPS
    tiny = np.finfo(np.float64).tiny
    ok = all(T[j, j] == w[j].real for j in range(n))
    if n > 1:
        if T[1, 0] == 0:
            ok &= w[0].imag == 0
        if T[n - 1, n - 2] == 0:
            ok &= w[n - 1].imag == 0
    for j in range(n - 1):
        if T[j + 1, j] != 0:
            t = np.sqrt(abs(T[j + 1, j])) * np.sqrt(abs(T[j, j + 1]))
            cmp = max(ulp * t, tiny)
            ok &= abs(w[j].imag - t) / cmp < tol
            ok &= abs(w[j + 1].imag + t) / cmp < tol
        elif j > 0 and T[j + 1, j] == 0 and T[j, j - 1] == 0:
            ok &= w[j].imag == 0
    return bool(ok)


def backward_error(A, T, Z):
    A = np.asarray(A)
    na = np.linalg.norm(A)
    if na == 0:
        return np.linalg.norm(Z @ T @ Z.conj().T)
    return np.linalg.norm(A - Z @ T @ Z.conj().T) / na


def orth_error(Z):
    return np.linalg.norm(Z.conj().T @ Z - np.eye(Z.shape[0]))


def rconde(VL, VR):
    """Reciprocal eigenvalue condition numbers (pirates.jl:107-113)."""
    num = np.abs(np.sum(VL.conj() * VR, axis=0))
    return num / (np.linalg.norm(VL, axis=0) * np.linalg.norm(VR, axis=0))


def match_eigenvalues(w_test, w_ref, tol_ref):
    """Optimal one-to-one matching; returns (ok, worst ratio err/tol)."""
    w_test = np.asarray(w_test)
    w_ref = np.asarray(w_ref)
    if len(w_test) != len(w_ref):
        return False, np.inf
    if len(w_ref) == 0:
        return True, 0.0
    cost = np.abs(w_test[None, :] - w_ref[:, None])
    r, c = linear_sum_assignment(cost)
    ratio = cost[r, c] / tol_ref[r]
    return bool(np.all(ratio <= 1.0)), float(np.max(ratio))


def assert_schur_real(A, T, Z, w, tol=10.0):
    """Real Schur form properties; tolerances as multiples of n*eps."""
    n = A.shape[0]
    assert np.all(np.tril(T, -2) == 0), "T not quasi-triangular"
    assert checkblocks(T), "2x2 blocks not in standard form"
    be = backward_error(A, T, Z)
    oe = orth_error(Z)
    assert be <= tol * n * EPS, "backward error %.3g > %g n eps" % (be, tol)
    assert oe <= tol * n * EPS, "orthogonality error %.3g > %g n eps" % (oe, tol)
    assert checkeigvals(T, w, 20), "eigenvalues inconsistent with T"
    return be, oe


def assert_schur_cplx(A, T, Z, w, tol=10.0):
    n = A.shape[0]
    assert np.all(np.tril(T, -1) == 0), "T not triangular"
    be = backward_error(A, T, Z)
    oe = orth_error(Z)
    assert be <= tol * n * EPS, "backward error %.3g > %g n eps" % (be, tol)
    assert oe <= tol * n * EPS, "orthogonality error %.3g > %g n eps" % (oe, tol)
    assert np.array_equal(np.sort_complex(w), np.sort_complex(np.diag(T)))
    return be, oe


def eig_tolerances(A, oracle):
    """Per-eigenvalue tolerances from the oracle's Schur pair and eigenvectors."""
    n = A.shape[0]
    T, Z, w = oracle.gschur(A)
    VR = oracle.eigvecs(T, Z, left=False)
    VL = oracle.eigvecs(T, Z, left=True)
    s = np.maximum(rconde(VL, VR), 1e-300)
    tol = 1e2 * max(n, 1) * EPS * np.linalg.norm(A) / s
    tol = np.maximum(tol, np.finfo(np.float64).tiny)
    return w, tol


def randn_matrix(rng, n, cplx=False):
    if cplx:
        return (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2)
    return rng.standard_normal((n, n))


def godunov():
    """Godunov's matrix and its exact eigenvalues (test/testfuncs.jl:127-142)."""
    A = np.array([
        [289, 2064, 336, 128, 80, 32, 16],
        [1152, 30, 1312, 512, 288, 128, 32],
        [-29, -2000, 756, 384, 1008, 224, 48],
        [512, 128, 640, 0, 640, 512, 128],
        [1053, 2256, -504, -384, -756, 800, 208],
        [-287, -16, 1712, -128, 1968, -30, 2032],
        [-2176, -287, -1565, -512, -541, -1152, -289]], dtype=np.float64)
    return A, np.array([-4, -2, -1, 0, 1, 2, 4], dtype=np.float64), 7.0e16
