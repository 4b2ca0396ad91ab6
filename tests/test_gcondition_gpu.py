"""GPU tests of the generalized Sylvester solvers and the condition estimates of complex
generalized Schur forms: trsylvester! / adjtrsylvester! (gsylvester.jl:23-155),
eigvalscond(S::GeneralizedSchur) (gcondition.jl:121-165) and subspacesep(S::GeneralizedSchur;
pnorm) (gcondition.jl:169-260, _trgsep 8-115).

* The reference's checkgsyl / checkgasyl (test/gordschur.jl:6-87) on the GPU solves, and
  the GPU solution equal to the oracle's to the bit: both run the reference's element
  order and complex formulas in plain IEEE arithmetic.
* eigvalscond / subspacesep against the oracle on the same pair, and pl, pr against LAPACK
  ztgsen (which solves the same equation).
* The reference's KPTest (test/gordschur.jl:193-295) through the GPU ggschur, gordschur and
  condition estimates.
* The reference's failure points: a 2 x 2 solve that needs rescaling, and a singular 2 x 2
  system of the look-ahead estimate (a shared eigenvalue), both reported as errors."""
import numpy as np
import pytest

from common import EPS, check_gsyl_errors, gsyl_errors, gsyl_problem, kp_pencil, kp_truth, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _close(a, b, rtol):
    a, b = np.atleast_1d(a), np.atleast_1d(b)
    return np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)))


@pytest.mark.parametrize("adjoint", [False, True])
@pytest.mark.parametrize("m,n", [(2, 4), (4, 2), (24, 24)])
def test_gtrsylvester_checkgsyl(gs, m, n, adjoint):
    rng = np.random.default_rng(1234 + 10 * m + n + adjoint)
    A, B, C, D, E, F, X, Y = gsyl_problem(rng, m, n, adjoint)
    fn = gs.adjtrsylvester if adjoint else gs.trsylvester
    X2, Y2, scale, pert = fn(A, B, C, D, E, F)
    assert scale == 1.0 and not pert
    check_gsyl_errors(m, n, gsyl_errors(A, B, C, D, E, F, X, Y, X2, Y2, scale, adjoint))


@pytest.mark.parametrize("adjoint", [False, True])
@pytest.mark.parametrize("m,n", [(1, 1), (1, 7), (7, 1), (24, 24), (33, 65), (130, 70), (256, 256)])
def test_gtrsylvester_matches_oracle(gs, m, n, adjoint):
    """The wavefront solve pulls, for each element, the updates the reference pushes into
    it, in the reference's order: the same bits as the oracle's element-by-element solve."""
    rng = np.random.default_rng(900 + m + 3 * n + adjoint)
    A, B, C, D, E, F, X, Y = gsyl_problem(rng, m, n, adjoint)
    fn = gs.adjtrsylvester if adjoint else gs.trsylvester
    X2, Y2, scale, _ = fn(A, B, C, D, E, F)
    Xo, Yo, so = po.gtrsylvester(A, B, C, D, E, F, adjoint=adjoint)
    assert scale == so == 1.0
    assert np.array_equal(X2, Xo) and np.array_equal(Y2, Yo)
    # past the reference's 24 x 24 these triangular problems are ill-conditioned (|R| grows
    # to 1e66 at 256 x 256): the normwise backward error, against the computed solution
    if adjoint:
        ra = A.conj().T @ X2 + D.conj().T @ Y2 - C
        rb = X2 @ B.conj().T + Y2 @ E.conj().T + F
    else:
        ra = A @ X2 - Y2 @ B - C
        rb = D @ X2 - Y2 @ E - F
    nx = np.linalg.norm(X2) + np.linalg.norm(Y2)
    assert np.linalg.norm(ra) <= 100 * EPS * ((np.linalg.norm(A) + np.linalg.norm(B)) * nx + np.linalg.norm(C))
    assert np.linalg.norm(rb) <= 100 * EPS * ((np.linalg.norm(D) + np.linalg.norm(E)) * nx + np.linalg.norm(F))


def test_gtrsylvester_perturbed(gs):
    """A shared eigenvalue of (A, D) and (B, E) makes a 2 x 2 system singular: its pivot is
    raised to smin and the perturbed flag returned, as in _safe_lu_solve!."""
    rng = np.random.default_rng(31)
    A, B, C, D, E, F, X, Y = gsyl_problem(rng, 3, 2, False)
    B[1, 1], E[1, 1] = A[0, 0], D[0, 0]
    X2, Y2, scale, pert = gs.trsylvester(A, B, C, D, E, F)
    Xo, Yo, so = po.gtrsylvester(A, B, C, D, E, F)
    assert pert and scale == 1.0
    assert np.array_equal(X2, Xo) and np.array_equal(Y2, Yo)


def test_gtrsylvester_rescale_raises(gs):
    """A solution past the overflow threshold needs the right-hand side rescaled, where the
    reference's trsylvester! raises (lmul!(view, scale) has no method)."""
    A, B = np.array([[1e-20]]), np.array([[2e-20]])
    D, E = np.array([[3e-20]]), np.array([[5e-20]])
    C, F = np.array([[1e280]]), np.array([[1e280]])
    with pytest.raises(gs.ArgumentError, match="rescaling"):
        gs.trsylvester(A, B, C, D, E, F)


def _pencil(gs, n, seed):
    """A complex generalized Schur pair of a random pencil (the oracle's ggschur makes the
    input; the GPU ggschur is exercised by the KPTest below)."""
    rng = np.random.default_rng(seed)
    S, T, al, be, Q, Z, st = po.ggschur(randn_matrix(rng, n, True), randn_matrix(rng, n, True))
    assert st == 0
    return gs.GeneralizedSchur(S, T, al, be, Q, Z)


@pytest.mark.parametrize("n,nsub", [(8, 3), (16, 1), (40, 20), (60, 59), (150, 37), (300, 150)])
def test_geigvalscond_matches_oracle_and_tgsen(gs, n, nsub):
    lapack = pytest.importorskip("scipy.linalg.lapack")
    G = _pencil(gs, n, 7100 + n + nsub)
    pl, pr = gs.eigvalscond(G, nsub)
    plo, pro = po.geigvalscond(G.S, G.T, nsub)
    assert _close([pl, pr], [plo, pro], 1e-13), (pl, pr, plo, pro)
    sel = np.zeros(n, np.int32)
    sel[:nsub] = 1
    r = lapack.ztgsen(sel, G.S, G.T, G.Q, G.Z, ijob=1, lwork=2 * n * n + 4, liwork=2 * n * n + 8)
    assert r[-1] == 0
    assert _close([pl, pr], [r[7], r[8]], 1e-10), (pl, pr, r[7], r[8])


@pytest.mark.parametrize("n,nsub", [(8, 3), (16, 1), (40, 20), (60, 59), (150, 37), (300, 150)])
def test_gsubspacesep_frobenius_matches_oracle(gs, n, nsub):
    """The look-ahead estimate's sign choices follow the accumulated right-hand sides, which
    are the oracle's to the bit; the norm of [R L] is summed in another order."""
    G = _pencil(gs, n, 7200 + n + nsub)
    sep = gs.subspacesep(G, nsub)
    sep_o = po.gsubspacesep(G.S, G.T, nsub)
    assert _close(sep, sep_o, 1e-12), (sep, sep_o)
    assert _close(gs.subspacesep(G, nsub, pnorm="Frobenius"), sep_o, 1e-12)


@pytest.mark.parametrize("n,nsub", [(6, 2), (12, 5), (20, 19), (40, 13)])
def test_gsubspacesep_onenorm_matches_oracle(gs, n, nsub):
    """pnorm = 1: norm1est! over the GPU generalized Sylvester operator and its adjoint,
    against the oracle's restatement over its own solves, and a lower bound on the exact
    one-norm of the inverse operator."""
    G = _pencil(gs, n, 7300 + n + nsub)
    sep = gs.subspacesep(G, nsub, pnorm=1)
    sep_o = po.gsubspacesep1(G.S, G.T, nsub)
    assert _close(sep, sep_o, 1e-9), (sep, sep_o)
    S, T, k = G.S, G.T, nsub
    for (A_, B_, D_, E_), s in zip(((S[:k, :k], S[k:, k:], T[:k, :k], T[k:, k:]),
                                    (S[k:, k:], S[:k, :k], T[k:, k:], T[:k, :k])), sep):
        m, q = A_.shape[0], B_.shape[0]
        Im, Iq = np.eye(m), np.eye(q)
        Zk = np.block([[np.kron(Iq, A_), -np.kron(B_.T, Im)], [np.kron(Iq, D_), -np.kron(E_.T, Im)]])
        assert 1.0 / s <= np.linalg.norm(np.linalg.inv(Zk), 1) * (1 + 1e-10)


@pytest.mark.parametrize("dtype", [2, 1])
def test_gcondition_kptest(gs, dtype):
    """KPTest (test/gordschur.jl:193-295, alpha = beta = x = y = 1) on the GPU: ggschur,
    gordschur to bring each eigenvalue to the front, eigvalscond and subspacesep within two
    orders of magnitude of the known values."""
    A, B, atrue, YH, X = kp_pencil(dtype=dtype)
    G = gs.ggschur(A, B)
    est = G.alpha / G.beta
    for j in range(5):
        idx = int(np.argmin(np.abs(est - atrue[j])))
        sel = np.zeros(5, bool)
        sel[idx] = True
        G2 = G if idx == 0 else gs.gordschur(G, sel)
        pl, pr = gs.eigvalscond(G2, 1)
        sep = gs.subspacesep(G2, 1)
        rcond, difl = kp_truth(A, B, YH, X, G2.S, G2.T, j, atrue[j], dtype)
        assert abs(np.log10(pl / rcond)) < 2 and abs(np.log10(pr / rcond)) < 2
        assert abs(np.log10(sep[0] / difl)) < 2 and abs(np.log10(sep[1] / difl)) < 2


def test_gcondition_edges(gs):
    G = _pencil(gs, 6, 7400)
    assert gs.eigvalscond(G, 0) == (1.0, 1.0) and gs.eigvalscond(G, 6) == (1.0, 1.0)
    assert np.array_equal(gs.subspacesep(G, 0), [0.0, 0.0]) and np.array_equal(gs.subspacesep(G, 6), [0.0, 0.0])
    with pytest.raises(gs.ArgumentError):
        gs.subspacesep(G, 0, pnorm=1)
    with pytest.raises(gs.ArgumentError):
        gs.subspacesep(G, 2, pnorm=2)


def test_gsubspacesep_singular_raises(gs):
    """The same eigenvalue on both sides of the split makes a look-ahead system singular,
    where the reference's lu(Z) raises SingularException."""
    S = np.triu(np.ones((3, 3), dtype=complex))
    T = np.eye(3, dtype=complex)
    G = gs.GeneralizedSchur(S, T, np.diag(S), np.diag(T), np.eye(3), np.eye(3))
    with pytest.raises(gs.ArgumentError, match="singular"):
        gs.subspacesep(G, 1)


def test_gcondition_real_triangular(gs):
    """A real upper triangular pair: the complex path is the reference's real arithmetic;
    pl, pr equal LAPACK dtgsen's."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(7500)
    n, k = 30, 11
    S = np.triu(rng.standard_normal((n, n))) + 2 * np.diag(rng.standard_normal(n))
    T = np.triu(rng.standard_normal((n, n))) + 3 * np.eye(n)
    G = gs.GeneralizedSchur(S, T, np.diag(S), np.diag(T), np.eye(n), np.eye(n))
    pl, pr = gs.eigvalscond(G, k)
    sel = np.zeros(n, np.int32)
    sel[:k] = 1
    r = lapack.dtgsen(sel, S, T, np.eye(n), np.eye(n), ijob=1, lwork=4 * n * n + 16, liwork=2 * n * n + 8)
    assert r[-1] == 0
    assert _close([pl, pr], [r[8], r[9]], 1e-10), (pl, pr, r[8], r[9])
    sep = gs.subspacesep(G, k)
    assert _close(sep, po.gsubspacesep(S.astype(complex), T.astype(complex), k), 1e-12)


def test_gcondition_large_timing(gs):
    """A random 1200 x 1200 triangular pair split in half: the wavefront solves against the
    oracle, with the GPU time of each estimate printed."""
    n, k = 1200, 600
    rng = np.random.default_rng(7600)
    S = np.triu(randn_matrix(rng, n, True), 1) / np.sqrt(n) + np.diag(randn_matrix(rng, n, True)[0])
    T = np.triu(randn_matrix(rng, n, True), 1) / np.sqrt(n) + np.diag(1 + 0.5 * rng.random(n))
    G = gs.GeneralizedSchur(S, T, np.diag(S), np.diag(T), np.eye(n), np.eye(n))
    ctx = gs.get_context()
    pl, pr = gs.eigvalscond(G, k)
    t_e = ctx.last_kernel_ms()
    sep = gs.subspacesep(G, k)
    t_s = ctx.last_kernel_ms()
    plo, pro = po.geigvalscond(G.S, G.T, k)
    sep_o = po.gsubspacesep(G.S, G.T, k)
    print("n=%d nsub=%d eigvalscond %.2f ms subspacesep %.2f ms" % (n, k, t_e, t_s))
    assert _close([pl, pr], [plo, pro], 1e-12)
    assert _close(sep, sep_o, 1e-12)
