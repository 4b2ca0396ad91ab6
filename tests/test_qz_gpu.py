"""GPU tests of the generalized Schur decomposition of complex pencils, ggschur!(A, B)
(generalized.jl:21-80, _hessenberg! 82-113, _gqz! 125-487), restating the reference's
gschurtest (test/generalized.jl:1-37): S and T upper triangular, A = Q S Z' and
B = Q T Z' to 20 n eps |A|, Q and Z unitary to 20 n eps; on its "basic sanity" pencils
(rand, n = 4 and 32) and its "challenging" ones (test/generalized.jl:98-121: triangular
pencils with zero diagonal entries in A and in B, rotated by random unitaries), plus the
oracle's restatement on the same inputs: the same generalized eigenvalues (optimal
matching) and the same number of infinite ones (beta = 0)."""
import numpy as np
import pytest

from common import EPS, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _gschurtest(A, B, G, tol=20.0):
    n = A.shape[0]
    nA = max(np.linalg.norm(A), np.finfo(float).tiny)
    S, T, Q, Z = G.S, G.T, G.Q, G.Z
    assert np.all(np.tril(S, -1) == 0) and np.all(np.tril(T, -1) == 0)
    assert np.linalg.norm(A - Q @ S @ Z.conj().T) / (n * nA * EPS) < tol
    assert np.linalg.norm(B - Q @ T @ Z.conj().T) / (n * nA * EPS) < tol
    assert np.linalg.norm(np.eye(n) - Z @ Z.conj().T) / (n * EPS) < tol
    assert np.linalg.norm(np.eye(n) - Q @ Q.conj().T) / (n * EPS) < tol
    assert np.all(np.diag(T).imag == 0) and np.all(np.diag(T).real >= 0)
    assert np.array_equal(G.alpha, np.diag(S)) and np.array_equal(G.beta, np.diag(T))


def _match(w1, w2):
    from scipy.optimize import linear_sum_assignment
    fin1, fin2 = np.isfinite(w1), np.isfinite(w2)
    assert fin1.sum() == fin2.sum()
    a, b = w1[fin1], w2[fin2]
    if len(a) == 0:
        return 0.0
    C = np.abs(a[:, None] - b[None, :]) / np.maximum(1.0, np.abs(b[None, :]))
    r, c = linear_sum_assignment(C)
    return float(np.max(C[r, c]))


def _ratio(G):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(G.beta != 0, G.alpha / np.where(G.beta != 0, G.beta, 1), np.inf)


@pytest.mark.parametrize("n", [1, 2, 4, 32, 100])
@pytest.mark.parametrize("kind", ["complex", "real-as-complex"])
def test_ggschur_random(gs, n, kind):
    rng = np.random.default_rng(8000 + n)
    if kind == "complex":
        A = rng.random((n, n)) + 1j * rng.random((n, n))
        B = rng.random((n, n)) + 1j * rng.random((n, n))
    else:
        A, B = rng.random((n, n)).astype(complex), rng.random((n, n)).astype(complex)
    G = gs.ggschur(A, B)
    _gschurtest(A, B, G)
    S, T, al, be, Q, Z, st = po.ggschur(A, B)
    assert st == 0
    assert _match(_ratio(G), np.where(be != 0, al / np.where(be != 0, be, 1), np.inf)) < 1e-8
    w = gs.eigvals(A, B)
    assert _match(w, _ratio(G)) == 0.0


def _challenging(rng, n=32):
    n1 = n >> 2
    n2 = n - 2 * n1
    A0 = np.triu(rng.random((n, n)) - 0.5 + 1j * (rng.random((n, n)) - 0.5))
    B0 = np.triu(rng.random((n, n)) - 0.5 + 1j * (rng.random((n, n)) - 0.5))
    for j in range(n1):
        A0[j, j] = 0
    for j in range(n1, n2):
        B0[j, j] = 0
    Qa, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    Qb, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return Qa @ A0 @ Qa.conj().T, Qb @ B0 @ Qb.conj().T


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ggschur_challenging(gs, seed):
    """Singular pencils: zero diagonal entries of B take the reference's zero-chasing
    branches (split off the top, chase to the bottom, clear H[ilast, ilast-1])."""
    rng = np.random.default_rng(8100 + seed)
    A, B = _challenging(rng)
    G = gs.ggschur(A, B)
    _gschurtest(A, B, G)
    S, T, al, be, Q, Z, st = po.ggschur(A, B)
    assert st == 0
    nb = np.sum(np.abs(G.beta) <= 1e-10 * np.linalg.norm(B))
    nbo = np.sum(np.abs(be) <= 1e-10 * np.linalg.norm(B))
    assert nb == nbo


def test_ggschur_batched_matches_single(gs):
    rng = np.random.default_rng(8200)
    ns = [1, 3, 17, 40, 8, 64]
    As = [randn_matrix(rng, n, True) for n in ns]
    Bs = [randn_matrix(rng, n, True) for n in ns]
    out, st = gs.ggschur_batched(As, Bs)
    assert np.all(st == 0)
    for A, B, Gb in zip(As, Bs, out):
        G = gs.ggschur(A, B)
        np.testing.assert_array_equal(Gb.S, G.S)
        np.testing.assert_array_equal(Gb.T, G.T)
        np.testing.assert_array_equal(Gb.Q, G.Q)
        np.testing.assert_array_equal(Gb.Z, G.Z)
        _gschurtest(A, B, Gb)


@pytest.mark.parametrize("s", [1e-300, 1e300])
def test_ggschur_scaled(gs, s):
    """_scale! of A and B (generalized.jl:35-44): tiny and huge pencils."""
    rng = np.random.default_rng(8300)
    A0, B0 = randn_matrix(rng, 20, True), randn_matrix(rng, 20, True)
    G = gs.ggschur(s * A0, s * B0)
    assert np.all(np.isfinite(G.S)) and np.all(np.isfinite(G.T))
    G0 = gs.ggschur(A0, B0)
    assert _match(_ratio(G), _ratio(G0)) < 1e-10
    _gschurtest(A0, B0, gs.GeneralizedSchur(G.S / s, G.T / s, G.alpha / s, G.beta / s, G.Q, G.Z))


def _evcheck(gs, A, B, G, tol=20.0):
    """The eigenvector half of the reference's gschurtest (test/generalized.jl:33-38):
    ||(A VR) diag(beta) - (B VR) diag(alpha)|| and the same for the left vectors with
    A', B' and conj(alpha), conj(beta), each below tol n ||A|| eps."""
    n = A.shape[0]
    nA = max(np.linalg.norm(A), np.finfo(float).tiny)
    VR = gs.geigvecs(G)
    VL = gs.geigvecs(G, left=True)
    r = np.linalg.norm((A @ VR) @ np.diag(G.beta) - (B @ VR) @ np.diag(G.alpha))
    assert r / (n * nA * EPS) < tol
    Ah, Bh = A.conj().T, B.conj().T
    r = np.linalg.norm((Ah @ VL) @ np.diag(G.beta.conj()) - (Bh @ VL) @ np.diag(G.alpha.conj()))
    assert r / (n * nA * EPS) < tol
    return VR, VL


def _same_columns(V, Vo, tol):
    """Column-by-column agreement with the oracle's vectors for the same Schur pair (both
    scaled to max |re|+|im| = 1, so columns agree up to rounding)."""
    err = np.max(np.abs(V - Vo)) if V.size else 0.0
    assert err < tol, err


@pytest.mark.parametrize("n", [1, 2, 4, 32, 100])
@pytest.mark.parametrize("kind", ["complex", "real-as-complex"])
def test_ggeigvecs_random(gs, n, kind):
    rng = np.random.default_rng(8400 + n)
    if kind == "complex":
        A = rng.random((n, n)) + 1j * rng.random((n, n))
        B = rng.random((n, n)) + 1j * rng.random((n, n))
    else:
        A, B = rng.random((n, n)).astype(complex), rng.random((n, n)).astype(complex)
    G = gs.ggschur(A, B)
    VR, VL = _evcheck(gs, A, B, G)
    _same_columns(VR, po.ggeigvecs(G.S, G.T, G.Z), 1e-9)
    _same_columns(VL, po.ggeigvecs(G.S, G.T, G.Q, left=True), 1e-9)
    # the triangular pair's own eigenvectors (no back-transform)
    Gt = gs.GeneralizedSchur(G.S, G.T, G.alpha, G.beta, None, None)
    _same_columns(gs.geigvecs(Gt), po.ggeigvecs(G.S, G.T), 1e-9)
    _same_columns(gs.geigvecs(Gt, left=True), po.ggeigvecs(G.S, G.T, left=True), 1e-9)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ggeigvecs_challenging(gs, seed):
    """Singular pencils (zero diagonal entries in A and in B): infinite and zero
    eigenvalues, and the unit vectors of a singular pencil where S_kk = T_kk = 0."""
    rng = np.random.default_rng(8100 + seed)
    A, B = _challenging(rng)
    G = gs.ggschur(A, B)
    _evcheck(gs, A, B, G)
    _same_columns(gs.geigvecs(G), po.ggeigvecs(G.S, G.T, G.Z), 1e-8)
    _same_columns(gs.geigvecs(G, left=True), po.ggeigvecs(G.S, G.T, G.Q, left=True), 1e-8)


def test_ggeigvecs_singular_unit_vectors(gs):
    """A pencil with S_kk = T_kk = 0 (vectors.jl:769-772): unit eigenvector e_k."""
    rng = np.random.default_rng(8500)
    n = 12
    S = np.triu(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    T = np.triu(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    T[np.diag_indices(n)] = np.abs(np.diag(T))
    S[5, 5] = 0
    T[5, 5] = 0
    G = gs.GeneralizedSchur(S, T, np.diag(S), np.diag(T), None, None)
    for left in (False, True):
        V = gs.geigvecs(G, left=left)
        e = np.zeros(n)
        e[5] = 1
        np.testing.assert_array_equal(V[:, 5], e)
        _same_columns(V, po.ggeigvecs(S, T, left=left), 1e-9)



# ---------------------------------------------------------------------------
# real pencils: ggschur!(A::Real, B) (rgeneralized.jl:10-808)
# ---------------------------------------------------------------------------
def _gschurtest_real(A, B, G, tol=20.0, exact=True):
    """The reference's real gschurtest (test/generalized.jl:40-60): S quasi-triangular, T
    upper triangular, A = Q S Z' and B = Q T Z' to tol n ||A|| eps, Q and Z orthogonal; plus
    the form the real QZ leaves: diag(T) >= 0, B diagonal on each 2 x 2 block of S, whose
    eigenvalues form a complex pair."""
    n = A.shape[0]
    nA = max(np.linalg.norm(A), np.finfo(float).tiny)
    S, T, Q, Z = G.S, G.T, G.Q, G.Z
    assert not np.iscomplexobj(S) and not np.iscomplexobj(T)
    assert np.all(np.tril(S, -2) == 0) and np.all(np.tril(T, -1) == 0)
    assert np.linalg.norm(A - Q @ S @ Z.T) / (n * nA * EPS) < tol
    assert np.linalg.norm(B - Q @ T @ Z.T) / (n * nA * EPS) < tol
    assert np.linalg.norm(np.eye(n) - Z @ Z.T) / (n * EPS) < tol
    assert np.linalg.norm(np.eye(n) - Q @ Q.T) / (n * EPS) < tol
    assert np.all(np.diag(T) >= 0)
    for k in range(n - 1):
        if S[k + 1, k] != 0:
            assert T[k, k + 1] == 0 and T[k + 1, k] == 0
            w1, w2 = G.alpha[k] / G.beta[k], G.alpha[k + 1] / G.beta[k + 1]
            assert w1.imag != 0 and abs(w2 - np.conj(w1)) <= 1e-12 * abs(w1)
    one = [k for k in range(n) if (k == 0 or S[k, k - 1] == 0) and (k == n - 1 or S[k + 1, k] == 0)]
    for k in one:
        if exact:
            assert G.alpha[k] == S[k, k] and G.beta[k] == T[k, k]
        else:  # factors rescaled by the caller (complex vs real division)
            assert abs(G.alpha[k] - S[k, k]) <= 4 * EPS * abs(S[k, k]) and abs(G.beta[k] - T[k, k]) <= 4 * EPS * abs(T[k, k])


def _real_pencil_check(gs, A, B, oracle_tol=1e-8):
    G = gs.ggschur(A, B)
    _gschurtest_real(A, B, G)
    S, T, al, be, Q, Z, st = po.ggschur_real(A, B)
    assert st == 0
    assert _match(_ratio(G), np.where(be != 0, al / np.where(be != 0, be, 1), np.inf)) < oracle_tol
    return G


@pytest.mark.parametrize("n", [1, 2, 3, 4, 8, 32, 100])
def test_ggschur_real_random(gs, n):
    """The reference's basic sanity case for Float64 (test/generalized.jl:62-81: rand pencils
    of order 4 and 32) and other orders: eigenvalues as the oracle's real QZ and LAPACK's."""
    rng = np.random.default_rng(8600 + n)
    A, B = rng.random((n, n)), rng.random((n, n))
    G = _real_pencil_check(gs, A, B)
    import scipy.linalg as sl
    assert _match(_ratio(G), sl.eigvals(A, B)) < 1e-8
    np.testing.assert_array_equal(gs.eigvals(A, B), _ratio(G))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ggschur_real_singular(gs, seed):
    """Real pencils with zero diagonal entries in A and in B (rotated by random orthogonal
    matrices): infinite and zero eigenvalues through the singular-B branches of the real
    iteration (split off the top, chase the zero to the bottom)."""
    rng = np.random.default_rng(8700 + seed)
    n = 32
    n1 = n >> 2
    n2 = n - 2 * n1
    A0 = np.triu(rng.random((n, n)) - 0.5)
    B0 = np.triu(rng.random((n, n)) - 0.5)
    A0[np.arange(n1), np.arange(n1)] = 0
    B0[np.arange(n1, n2), np.arange(n1, n2)] = 0
    Qa, _ = np.linalg.qr(rng.standard_normal((n, n)))
    Qb, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A, B = Qa @ A0 @ Qa.T, Qb @ B0 @ Qb.T
    G = gs.ggschur(A, B)
    _gschurtest_real(A, B, G)
    S, T, al, be, Q, Z, st = po.ggschur_real(A, B)
    assert st == 0
    nb = np.sum(np.abs(G.beta) <= 1e-10 * np.linalg.norm(B))
    assert nb == np.sum(np.abs(be) <= 1e-10 * np.linalg.norm(B))


def test_ggschur_real_batched_matches_single(gs):
    rng = np.random.default_rng(8800)
    ns = [1, 2, 5, 17, 40, 64]
    As = [rng.standard_normal((n, n)) for n in ns]
    Bs = [rng.standard_normal((n, n)) for n in ns]
    out, st = gs.ggschur_batched(As, Bs)
    assert np.all(st == 0)
    for A, B, Gb in zip(As, Bs, out):
        G = gs.ggschur(A, B)
        np.testing.assert_array_equal(Gb.S, G.S)
        np.testing.assert_array_equal(Gb.T, G.T)
        np.testing.assert_array_equal(Gb.Q, G.Q)
        np.testing.assert_array_equal(Gb.Z, G.Z)
        _gschurtest_real(A, B, Gb)


@pytest.mark.parametrize("s", [1e-300, 1e300])
def test_ggschur_real_scaled(gs, s):
    """_scale! of A and B (rgeneralized.jl:25-33) and the unscaling of S, T, alpha, beta."""
    rng = np.random.default_rng(8900)
    A0, B0 = rng.standard_normal((20, 20)), rng.standard_normal((20, 20))
    G = gs.ggschur(s * A0, s * B0)
    assert np.all(np.isfinite(G.S)) and np.all(np.isfinite(G.T))
    G0 = gs.ggschur(A0, B0)
    assert _match(_ratio(G), _ratio(G0)) < 1e-10
    _gschurtest_real(A0, B0, gs.GeneralizedSchur(G.S / s, G.T / s, G.alpha / s, G.beta / s, G.Q, G.Z), exact=False)



def _evcheck_real(gs, A, B, G, tol=20.0):
    """The eigenvector half of the reference's real gschurtest (test/generalized.jl:55-59):
    ||(A VR) diag(beta) - (B VR) diag(alpha)|| and ||diag(beta) (VL' A) - diag(alpha) (VL' B)||
    below tol n ||A|| eps."""
    n = A.shape[0]
    nA = max(np.linalg.norm(A), np.finfo(float).tiny)
    VR = gs.geigvecs(G)
    VL = gs.geigvecs(G, left=True)
    r = np.linalg.norm((A @ VR) @ np.diag(G.beta) - (B @ VR) @ np.diag(G.alpha))
    assert r / (n * nA * EPS) < tol
    r = np.linalg.norm(np.diag(G.beta) @ (VL.conj().T @ A) - np.diag(G.alpha) @ (VL.conj().T @ B))
    assert r / (n * nA * EPS) < tol
    return VR, VL


@pytest.mark.parametrize("n", [1, 2, 3, 4, 8, 32, 100])
def test_ggeigvecs_real(gs, n):
    """Real pencils: the reference's eigenvector check, and the same columns as the oracle's
    restatement on the same Schur pair (with and without the back-transform)."""
    rng = np.random.default_rng(9100 + n)
    A, B = rng.random((n, n)), rng.random((n, n))
    G = gs.ggschur(A, B)
    VR, VL = _evcheck_real(gs, A, B, G)
    _same_columns(VR, po.rgeigvecs(G.S, G.T, G.Z), 1e-9)
    _same_columns(VL, po.rgeigvecs(G.S, G.T, G.Q, left=True), 1e-9)
    Gt = gs.GeneralizedSchur(G.S, G.T, G.alpha, G.beta, None, None)
    _same_columns(gs.geigvecs(Gt), po.rgeigvecs(G.S, G.T), 1e-9)
    _same_columns(gs.geigvecs(Gt, left=True), po.rgeigvecs(G.S, G.T, left=True), 1e-9)
    for k in range(n - 1):
        if G.S[k + 1, k] != 0:
            np.testing.assert_array_equal(VR[:, k + 1], VR[:, k].conj())
            np.testing.assert_array_equal(VL[:, k + 1], VL[:, k].conj())


@pytest.mark.parametrize("seed", [0, 1])
def test_ggeigvecs_real_singular(gs, seed):
    rng = np.random.default_rng(8700 + seed)
    n = 32
    n1 = n >> 2
    n2 = n - 2 * n1
    A0 = np.triu(rng.random((n, n)) - 0.5)
    B0 = np.triu(rng.random((n, n)) - 0.5)
    A0[np.arange(n1), np.arange(n1)] = 0
    B0[np.arange(n1, n2), np.arange(n1, n2)] = 0
    Qa, _ = np.linalg.qr(rng.standard_normal((n, n)))
    Qb, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A, B = Qa @ A0 @ Qa.T, Qb @ B0 @ Qb.T
    G = gs.ggschur(A, B)
    _evcheck_real(gs, A, B, G)
    # eigenvectors of singular pencils can be ill-conditioned: the tolerance is ten times
    # the change of the oracle's own vectors under 1-ulp relative perturbations of S and T
    for left, M in ((False, G.Z), (True, G.Q)):
        Vo = po.rgeigvecs(G.S, G.T, M, left=left)
        sens = 0.0
        for t in range(3):
            r = np.random.default_rng(t)
            Sp = G.S * (1 + EPS * r.standard_normal(G.S.shape))
            Tp = G.T * (1 + EPS * r.standard_normal(G.T.shape))
            sens = max(sens, float(np.max(np.abs(po.rgeigvecs(Sp, Tp, M, left=left) - Vo))))
        _same_columns(gs.geigvecs(G, left=left), Vo, max(1e-9, 10 * sens))



# ---------------------------------------------------------------------------
# gordschur! of complex generalized Schur forms (ordschur.jl:147-305)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ggordschur_checkord(gs, seed):
    """The reference's checkord for ComplexF64 (test/gordschur.jl:139-186): n = 16, B shifted
    by I, the last half selected; S, T triangular, A = Q S Z', B = Q T Z' and Q, Z unitary to
    10 n eps, the wanted eigenvalues in front; and the oracle's reordering of the same form."""
    rng = np.random.default_rng(9200 + seed)
    n = 16
    A = rng.random((n, n)) + 1j * rng.random((n, n))
    B = rng.random((n, n)) + 1j * rng.random((n, n)) - (0.5 + 0.5j) + np.eye(n)
    G = gs.ggschur(A, B)
    select = np.ones(n, dtype=bool)
    select[: n >> 1] = False
    G2 = gs.gordschur(G, select)
    tol = 10
    nA, nB = np.linalg.norm(A), np.linalg.norm(B)
    assert np.linalg.norm(np.tril(G2.S, -1)) / (n * nA * EPS) < tol
    assert np.linalg.norm(np.tril(G2.T, -1)) / (n * nA * EPS) < tol
    assert np.linalg.norm(A - G2.Q @ G2.S @ G2.Z.conj().T) / (n * nA * EPS) < tol
    assert np.linalg.norm(B - G2.Q @ G2.T @ G2.Z.conj().T) / (n * nB * EPS) < tol
    assert np.linalg.norm(np.eye(n) - G2.Z @ G2.Z.conj().T) / (n * EPS) < tol
    assert np.linalg.norm(np.eye(n) - G2.Q @ G2.Q.conj().T) / (n * EPS) < tol
    w = G.alpha / G.beta
    wanted = list(w[select])
    for i in range(int(select.sum())):
        x = G2.alpha[i] / G2.beta[i]
        d = np.abs(np.array(wanted) - x)
        j = int(np.argmin(d))
        assert d[j] / (EPS + abs(x)) < tol
        wanted.pop(j)
    S, T, al, be, Q, Z, st = po.ggordschur(G.S, G.T, G.Q, G.Z, select)
    assert st == 0
    np.testing.assert_allclose(G2.alpha / G2.beta, al / be, rtol=1e-10, atol=0)
    assert np.max(np.abs(G2.S - S)) < 1e-10 * nA and np.max(np.abs(G2.T - T)) < 1e-10 * nB


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_ggordschur_real(gs, seed):
    """gordschur! of real generalized Schur forms (rordschur.jl:542-1178) on the GPU: the
    reference's real checkord (test/gordschur.jl:90-137, n = 16, the second half selected)
    and random selections at n = 16 and 40, through the GPU ggschur; against the oracle's
    restatement on the same pair: the same eigenvalue order and the same leading deflating
    subspaces.  Entry by entry the two differ by signs: each 2 x 2-block swap chooses
    between re-triangularizing by RQ or by QR by comparing two residuals of order eps
    (rordschur.jl:841-858), so the choice, and with it the signs of rows and columns,
    follows rounding -- the oracle's own output changes so under 1-ulp perturbations."""
    from common import check_gordschur_real, selected_with_pairs
    rng = np.random.default_rng(4700 + seed)
    for n, half in ((16, True), (16, False), (40, False)):
        A = rng.random((n, n))
        B = rng.random((n, n)) - 0.5 + np.eye(n)
        G = gs.ggschur(A, B)
        sel = np.ones(n, bool)
        if half:
            sel[: n >> 1] = False
        else:
            sel = rng.integers(0, 2, n).astype(bool)
        G2 = gs.gordschur(G, sel)
        check_gordschur_real(A, B, G.alpha / G.beta, sel, G2.S, G2.T, G2.alpha, G2.beta, G2.Q, G2.Z)
        S, T, a, b, Q, Z, st = po.ggordschur_real(G.S, G.T, G.Q, G.Z, sel.astype(np.int32))
        assert st == 0
        np.testing.assert_allclose(G2.alpha / G2.beta, a / b, rtol=1e-9, atol=0)
        k = int(selected_with_pairs(G.alpha / G.beta, sel).sum())
        for M2, Mo in ((G2.Z, Z), (G2.Q, Q)):
            P2 = M2[:, :k] @ M2[:, :k].T
            Po = Mo[:, :k] @ Mo[:, :k].T
            assert np.abs(P2 - Po).max() <= 1e-8, (k, np.abs(P2 - Po).max())


def test_ggordschur_real_noop_and_pairs(gs):
    """Nothing or everything selected leaves the eigenvalue order; selecting only one member
    of a complex pair moves the pair."""
    from common import check_gordschur_real
    rng = np.random.default_rng(4800)
    n = 20
    A = rng.standard_normal((n, n))
    B = rng.standard_normal((n, n))
    G = gs.ggschur(A, B)
    vals = G.alpha / G.beta
    for sel in (np.zeros(n, bool), np.ones(n, bool)):
        G2 = gs.gordschur(G, sel)
        np.testing.assert_allclose(G2.alpha / G2.beta, vals, rtol=1e-12)
    pairs = [j for j in range(n - 1) if vals[j].imag > 0]
    assert pairs, "the pencil should have a complex pair"
    sel = np.zeros(n, bool)
    sel[pairs[-1] + 1] = True
    G2 = gs.gordschur(G, sel)
    check_gordschur_real(A, B, vals, sel, G2.S, G2.T, G2.alpha, G2.beta, G2.Q, G2.Z)
    assert abs(G2.alpha[0] / G2.beta[0] - vals[pairs[-1]]) < 1e-8 * abs(vals[pairs[-1]]) or \
        abs(G2.alpha[0] / G2.beta[0] - vals[pairs[-1] + 1]) < 1e-8 * abs(vals[pairs[-1]])
