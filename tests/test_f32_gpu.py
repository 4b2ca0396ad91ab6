"""GPU tests of the Float32 entry points (gschur! on Float32 matrices computes in
Float32, as the reference's generic code does): the real Schur properties with
eps = eps(Float32), eigenvalues matched to the oracle's Float32 run and to its
Float64 run within 1e2 n eps32 ||A|| / s_i."""
import numpy as np
import pytest

from common import checkblocks, match_eigenvalues, randn_matrix, rconde
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)


def _check_f32(A, S, tol=10.0):
    n = A.shape[0]
    A64 = A.astype(np.float64)
    T = S.T.astype(np.float64)
    Z = S.Z.astype(np.float64)
    assert S.T.dtype == np.float32 and S.Z.dtype == np.float32
    assert np.all(np.tril(S.T, -2) == 0)
    assert checkblocks(S.T)
    be = np.linalg.norm(A64 - Z @ T @ Z.T) / max(np.linalg.norm(A64), 1e-300)
    oe = np.linalg.norm(Z.T @ Z - np.eye(n))
    assert be <= tol * n * EPS32, "backward error %.3g" % (be / (n * EPS32))
    assert oe <= tol * n * EPS32, "orthogonality %.3g" % (oe / (n * EPS32))


def _eig_tol32(A):
    A64 = A.astype(np.float64)
    n = A.shape[0]
    T, Z, w = po.gschur(A64)
    VR = po.eigvecs(T, Z, left=False)
    VL = po.eigvecs(T, Z, left=True)
    s = np.maximum(rconde(VL, VR), 1e-300)
    return w, 1e2 * n * EPS32 * np.linalg.norm(A64) / s


@pytest.mark.parametrize("n", [1, 2, 5, 17, 64, 100, 128, 129, 300])
def test_f32_random(gs, n):
    rng = np.random.default_rng(7100 + n)
    A = randn_matrix(rng, n).astype(np.float32)
    S = gs.gschur(A)
    _check_f32(A, S)
    w64, tol = _eig_tol32(A)
    ok, worst = match_eigenvalues(S.values, w64, tol)
    assert ok, "vs FP64 oracle: worst err/tol %.3g" % worst
    if n <= 128:
        # the oracle's own Float32 run (same arithmetic type as the reference would use)
        _, _, w32 = po.gschur_real(A, dtype=np.float32)
        ok, worst = match_eigenvalues(S.values, w32, tol)
        assert ok, "vs Float32 oracle: worst err/tol %.3g" % worst


def test_f32_batched(gs):
    rng = np.random.default_rng(7200)
    ns = rng.integers(8, 129, size=40)
    mats = [randn_matrix(rng, int(n)).astype(np.float32) for n in ns]
    Ts, Zs, ws, status = gs.gschur_batched(mats)
    assert np.all(status == 0)
    for A, T, Z, w in zip(mats, Ts, Zs, ws):
        assert T.dtype == np.float32
        _check_f32(A, gs.Schur(T, Z, w))


def test_f32_scaled(gs):
    """_scale! with Float32's own thresholds: tiny and huge inputs in range of Float32."""
    rng = np.random.default_rng(7300)
    A0 = randn_matrix(rng, 40)
    for s in (1e-30, 1e30):
        A = (s * A0).astype(np.float32)
        S = gs.gschur(A)
        assert np.all(np.isfinite(S.T)) and np.all(np.isfinite(S.Z))
        _check_f32(A, S)
