"""GPU tests of the large-matrix path (n > 128): whole-GPU Hessenberg reduction and
multishift QR.  Same criteria as the small-matrix tests: hesstest / schurtest
properties (test/real.jl:24-99) with the 10 n eps bounds, and eigenvalues matched to
the oracle's within 1e2 n eps ||A||_F / s_i."""
import numpy as np
import pytest

from common import EPS, assert_schur_real, checkblocks, eig_tolerances, match_eigenvalues, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["unblocked", "blocked"])
def hess_variant(request, monkeypatch):
    """Both FP64 Hessenberg reductions: the fused unblocked one (default for FP64) and
    the compact-WY blocked one (default for FP32, selected for FP64 from order 256 on by
    GS_HESS_BLOCKED_MIN, which the library reads at every call)."""
    if request.param == "blocked":
        monkeypatch.setenv("GS_HESS_BLOCKED_MIN", "256")
    else:
        monkeypatch.delenv("GS_HESS_BLOCKED_MIN", raising=False)
    return request.param


@pytest.mark.parametrize("n", [3, 40, 150, 257, 300, 515, 1030])
def test_hessenberg(gs, n, hess_variant):
    rng = np.random.default_rng(9000 + n)
    A = rng.standard_normal((n, n))
    Hp, tau, Q = gs.hessenberg(A)
    H = np.triu(Hp, -1)
    assert np.linalg.norm(A - Q @ H @ Q.T) / (n * np.linalg.norm(A) * EPS) < 10
    assert np.linalg.norm(np.eye(n) - Q @ Q.T) / (n * EPS) < 10
    # same reflectors as the oracle (up to rounding)
    Ho, tauo, Qo = po.hessenberg(A)
    assert np.max(np.abs(tau - tauo)) < 1e-10


@pytest.mark.parametrize("scale", [1e-300, 1e-155, 1e155, 1e300])
def test_hessenberg_extreme_scale(gs, scale, hess_variant):
    """Columns whose norms leave the range where squares are representable: the blocked
    reduction's one-pass (scale, sum of squares) norms and the reflector's rescaling loop
    (householder.jl:12-54) keep the reflectors equal to the oracle's."""
    rng = np.random.default_rng(9050)
    n = 300
    A0 = rng.standard_normal((n, n))
    A = A0 * scale
    Hp, tau, Q = gs.hessenberg(A)
    H = np.triu(Hp, -1)
    assert np.all(np.isfinite(Hp)) and np.all(np.isfinite(Q))
    assert np.linalg.norm(A0 - Q @ (H / scale) @ Q.T) / (n * np.linalg.norm(A0) * EPS) < 10
    Ho, tauo, Qo = po.hessenberg(A)
    assert np.max(np.abs(tau - tauo)) < 1e-10


@pytest.mark.parametrize("n", [129, 160, 256, 400])
def test_large_schur_random(gs, n, hess_variant):
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


def _structured(n, kind, rng):
    if kind == "zero":
        return np.zeros((n, n))
    if kind == "triangular":
        return np.triu(rng.standard_normal((n, n)))
    if kind == "blockdiag":
        A = np.zeros((n, n))
        cuts = [0, n // 3, n // 2, n]
        for a, b in zip(cuts[:-1], cuts[1:]):
            A[a:b, a:b] = rng.standard_normal((b - a, b - a))
        return A
    if kind == "companion":
        A = np.zeros((n, n))
        A[1:, :-1] = np.eye(n - 1)
        A[:, -1] = rng.standard_normal(n) / n
        return A
    if kind == "jordan":
        # identity plus a nilpotent Jordan part: one eigenvalue of multiplicity n
        return np.eye(n) + np.diag(np.ones(n - 1), 1)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["zero", "triangular", "blockdiag", "companion", "jordan"])
def test_large_structured(gs, kind):
    """Structured inputs of order > 128: the Schur form properties hold (the reference's
    deflation handles the zero subdiagonals from the start)."""
    n = 200
    rng = np.random.default_rng(9900)
    A = _structured(n, kind, rng)
    S = gs.gschur(A)
    assert np.all(np.tril(S.T, -2) == 0)
    assert checkblocks(S.T)
    nA = max(np.linalg.norm(A), 1.0)
    assert np.linalg.norm(A - S.Z @ S.T @ S.Z.T) / nA <= 10 * n * EPS
    assert np.linalg.norm(S.Z.T @ S.Z - np.eye(n)) <= 10 * n * EPS
    if kind in ("zero", "triangular"):
        np.testing.assert_allclose(np.sort(S.values.real), np.sort(np.diag(A)), atol=10 * n * EPS * nA)


def test_large_nonfinite_input_terminates(gs):
    """A NaN entry must end in an error or non-finite output, never in a hang (the
    sweep limit bounds the iteration)."""
    n = 150
    A = np.random.default_rng(9901).standard_normal((n, n))
    A[7, 3] = np.nan
    try:
        S = gs.gschur(A, maxiter=20 * n)
    except (gs.UnconvergedException, gs.ArgumentError):
        return
    assert not np.all(np.isfinite(S.T))


@pytest.mark.parametrize("n", [130, 200, 300])
def test_large_complex_multishift(gs, n):
    """Complex orders above 128 on the whole GPU (Hessenberg reduction, multishift QR,
    trailing blocks by the batched kernel): Schur properties and the oracle's eigenvalues."""
    from common import assert_schur_cplx
    rng = np.random.default_rng(9750 + n)
    A = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


def test_large_complex_600_vs_lapack(gs):
    import scipy.linalg
    from common import assert_schur_cplx, rconde
    n = 600
    rng = np.random.default_rng(9760)
    A = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w, VL, VR = scipy.linalg.eig(A, left=True, right=True)
    tol = 1e2 * n * EPS * np.linalg.norm(A) / np.maximum(rconde(VL, VR), 1e-300)
    ok, worst = match_eigenvalues(S.values, w, tol)
    assert ok, "worst err/tol %.3g" % worst


@pytest.mark.parametrize("kind", ["zero", "triangular", "blockdiag", "companion", "jordan", "unitary", "scaled"])
def test_large_complex_structured(gs, kind):
    """Structured complex inputs of order > 128 end in a Schur form within the FP64 bounds."""
    from common import assert_schur_cplx
    n = 180
    rng = np.random.default_rng(9770)
    if kind == "unitary":
        Q, R = np.linalg.qr(randn_matrix(rng, n, cplx=True))
        A = Q @ np.diag(np.sign(np.diag(R)))
    elif kind == "scaled":
        A = 1e300 * randn_matrix(rng, n, cplx=True)
    else:
        A = _structured(n, kind, rng).astype(np.complex128)
        if kind in ("triangular", "blockdiag"):
            A = A + 1j * _structured(n, kind, np.random.default_rng(9771))
    S = gs.gschur(A)
    assert np.all(np.tril(S.T, -1) == 0)
    if kind == "scaled":  # compare at unit scale (the products overflow at 1e300)
        A, S = A / 1e300, gs.Schur(S.T / 1e300, S.Z, S.values / 1e300)
    nA = max(np.linalg.norm(A), 1e-300)
    assert np.linalg.norm(A - S.Z @ S.T @ S.Z.conj().T) / nA <= 10 * n * EPS
    assert np.linalg.norm(S.Z.conj().T @ S.Z - np.eye(n)) <= 10 * n * EPS
    np.testing.assert_array_equal(S.values, np.diag(S.T))
    if kind in ("zero", "triangular"):
        np.testing.assert_allclose(np.sort_complex(S.values), np.sort_complex(np.diag(A)), atol=10 * n * EPS * nA)


def test_large_complex_wantz_false(gs):
    rng = np.random.default_rng(9780)
    A = randn_matrix(rng, 220, cplx=True)
    S1 = gs.gschur(A)
    S0 = gs.gschur(A, wantZ=False)
    from common import match_eigenvalues as mt
    tol = np.full(220, 1e-9 * np.abs(S1.values).max())
    ok, worst = mt(S0.values, S1.values, tol)
    assert ok, worst
