"""GPU parity tests of the eigenvector, triangularize and eigen paths.

Checks restate vectest (test/testfuncs.jl:5-54): ||A VR - VR L|| / (n ||A|| ulp) and
||A^H VL - VL conj(L)|| / (n ||A|| ulp) below tol; the vectors are normalised as
_enormalize! leaves them (unit 2-norm, largest-modulus entry real); and columns of
well-conditioned eigenvalues agree with the oracle's vectors.
"""
import numpy as np
import pytest

from common import EPS, randn_matrix, rconde
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 5, 8, 16, 33, 64, 65, 100, 128]
# orders above 128 take the tiled back-substitution path (one matrix per call)
LARGE_SIZES = [129, 161, 300]


def _vectest(A, w, VR, VL, tol=20.0):
    n = A.shape[0]
    nA = max(np.linalg.norm(A), np.finfo(float).tiny)
    if VR is not None:
        assert np.linalg.norm(A @ VR - VR @ np.diag(w)) / (n * nA * EPS) < tol
    if VL is not None:
        assert np.linalg.norm(A.conj().T @ VL - VL @ np.diag(w.conj())) / (n * nA * EPS) < tol


def _normalized(V):
    n = V.shape[0]
    assert np.all(np.abs(np.linalg.norm(V, axis=0) - 1) < 10 * n * EPS)
    for j in range(V.shape[1]):
        assert V[np.argmax(np.abs(V[:, j])), j].imag == 0


def _compare(V, Vref, s):
    good = s > 1e-4
    if np.any(good):
        assert np.max(np.abs(V[:, good] - Vref[:, good])) < 1e-9


@pytest.mark.parametrize("n", SIZES + LARGE_SIZES)
def test_eigvecs_complex(gs, n):
    rng = np.random.default_rng(3000 + n)
    A = randn_matrix(rng, n, cplx=True)
    T, Z, w = po.gschur_cplx(A)
    S = gs.Schur(T, Z, w)
    VR = gs.eigvecs(S)
    VL = gs.eigvecs(S, left=True)
    _vectest(A, w, VR, VL)
    _normalized(VR)
    _normalized(VL)
    VRr = po.eigvecs(T, Z)
    VLr = po.eigvecs(T, Z, left=True)
    s = rconde(VLr, VRr)
    _compare(VR, VRr, s)
    _compare(VL, VLr, s)


@pytest.mark.parametrize("n", SIZES + LARGE_SIZES)
def test_eigvecs_real(gs, n):
    rng = np.random.default_rng(4000 + n)
    A = randn_matrix(rng, n)
    T, Z, w = po.gschur_real(A)
    S = gs.Schur(T, Z, w)
    VR = gs.geigvecs(S)
    VL = gs.geigvecs(S, left=True)
    _vectest(A, w, VR, VL)
    VRr = po.eigvecs(T, Z)
    VLr = po.eigvecs(T, Z, left=True)
    s = rconde(VLr, VRr)
    _compare(VR, VRr, s)
    _compare(VL, VLr, s)


@pytest.mark.parametrize("n", [2, 7, 40, 128, 300])
def test_triangularize(gs, n):
    rng = np.random.default_rng(5000 + n)
    A = randn_matrix(rng, n)
    T, Z, w = po.gschur_real(A)
    Sc = gs.triangularize(gs.Schur(T, Z, w))
    Tr, Zr, wr = po.triangularize(T, Z)
    assert np.all(np.tril(Sc.T, -1) == 0)
    scale = np.linalg.norm(A)
    assert np.max(np.abs(Sc.T - Tr)) <= 1e-13 * scale
    assert np.max(np.abs(Sc.Z - Zr)) <= 1e-13
    np.testing.assert_array_equal(Sc.values, np.diag(Sc.T))
    assert np.linalg.norm(A - Sc.Z @ Sc.T @ Sc.Z.conj().T) / (n * scale * EPS) < 10


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("n", [50, 260])
def test_eigen(gs, cplx, n):
    rng = np.random.default_rng(6)
    A = randn_matrix(rng, n, cplx)
    E = gs.eigen(A)
    assert np.all(np.diff(E.values.real) >= 0)
    _vectest(A, E.values, E.vectors, None)
    _normalized(E.vectors)
    E2 = gs.eigen(A, permute=False, scale=False)
    _vectest(A, E2.values, E2.vectors, None)


def test_eigvecs_of_T_only(gs):
    rng = np.random.default_rng(7)
    n = 30
    T = np.triu(randn_matrix(rng, n, cplx=True))
    S = gs.Schur(T, None, np.diag(T))
    V = gs.eigvecs(S)
    _vectest(T, np.diag(T), V, None)


def test_eigvecs_batched(gs):
    rng = np.random.default_rng(8)
    mats = [randn_matrix(rng, int(n), cplx=True) for n in rng.integers(2, 129, size=40)]
    res = [po.gschur_cplx(A) for A in mats]
    Tp, ns, offs, woffs = gs.pack_batch([r[0] for r in res], np.complex128)
    Zp, _, _, _ = gs.pack_batch([r[1] for r in res], np.complex128)
    VR = gs.geigvecs_batched(Tp, Zp, ns, offs)
    VL = gs.geigvecs_batched(Tp, Zp, ns, offs, left=True)
    for A, (T, Z, w), vr, vl in zip(mats, res, gs.unpack_batch(VR, ns, offs), gs.unpack_batch(VL, ns, offs)):
        _vectest(A, w, vr, vl)


def test_eigvecs_batched_real(gs):
    rng = np.random.default_rng(9)
    mats = [randn_matrix(rng, int(n)) for n in rng.integers(2, 129, size=30)]
    Ts, Zs, ws, st = gs.gschur_batched(mats)
    Tp, ns, offs, woffs = gs.pack_batch(Ts)
    Zp, _, _, _ = gs.pack_batch(Zs)
    VR = gs.geigvecs_batched(Tp, Zp, ns, offs, woffs)
    for A, w, vr in zip(mats, ws, gs.unpack_batch(VR, ns, offs)):
        _vectest(A, w, vr, None)


def test_eigvecs_nonfinite_does_not_raise(gs):
    # test/complex.jl:393-406: only requires that nothing throws
    rng = np.random.default_rng(10)
    T, Z, w = po.gschur_cplx(randn_matrix(rng, 5, cplx=True))
    for bad in (np.inf, np.nan):
        T2 = T.copy()
        T2[1, 2] = bad
        S = gs.Schur(T2, Z, w)
        gs.eigvecs(S)
        gs.eigvecs(S, left=True)
