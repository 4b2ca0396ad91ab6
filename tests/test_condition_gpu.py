"""GPU tests of the condition estimators of a Schur form: eigvalscond and subspacesep
(ordschur.jl:84-140, over trsylvester! / adjtrsylvester! of sylvester.jl and norm1est!
of norm1est.jl) and the per-eigenvalue loop of eigen!(A; jcv = true) (pirates.jl:136-153).

The reference's own check (test/ordschur.jl:35-54) compares eigvalscond / subspacesep
after ordschur with LAPACK's trsen s and sep; the same comparison runs here, next to the
oracle's restatement on the same reordered T.  Condition numbers are smooth functions of
T, so GPU and oracle (whose Sylvester sums run in different orders) agree to a relative
1e-9 on well-separated spectra; subspacesep's estimator takes discrete steps (argmax
picks), which coincide unless two candidates tie to rounding."""
import numpy as np
import pytest

from common import randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def _close(a, b, rtol=RTOL):
    return abs(a - b) <= rtol * max(abs(a), abs(b))


def _cplx_schur(gs, n, seed):
    rng = np.random.default_rng(seed)
    S = gs.gschur(randn_matrix(rng, n, cplx=True))
    return S, rng


@pytest.mark.parametrize("n,nsub", [(8, 3), (32, 3), (33, 1), (100, 40), (130, 64), (300, 100), (300, 1)])
def test_condition_complex_matches_oracle(gs, n, nsub):
    S, _ = _cplx_schur(gs, n, 6000 + n + nsub)
    s_g = gs.eigvalscond(S, nsub)
    sep_g = gs.subspacesep(S, nsub)
    s_o, sep_o = po.condition(S.T, nsub)
    assert _close(s_g, s_o), (s_g, s_o)
    assert _close(sep_g, sep_o), (sep_g, sep_o)


def test_condition_vs_trsen(gs):
    """test/ordschur.jl:35-54: three random eigenvalues moved to the front by ordschur,
    then eigvalscond / subspacesep equal LAPACK trsen's s and sep."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    for trial in range(3):
        n = 32
        S, rng = _cplx_schur(gs, n, 6100 + trial)
        select = np.zeros(n, dtype=bool)
        select[rng.integers(0, n, 3)] = True
        S2 = gs.gordschur(S, select)
        k = int(select.sum())
        _, _, _, m, s1, sep1, info = lapack.ztrsen(select.astype(np.int32), S.T, S.Z, lwork=2 * n * n)
        assert info == 0 and m == k
        assert _close(gs.eigvalscond(S2, k), s1, 1e-8)
        assert _close(gs.subspacesep(S2, k), sep1, 1e-8)


@pytest.mark.parametrize("n,nsub", [(40, 7), (97, 50)])
def test_condition_real(gs, n, nsub):
    """Float64 forms: an upper triangular T (all eigenvalues real), and a real Schur form
    with 2x2 blocks, whose subdiagonal entries the reference's triangular solver does
    not read (the GPU and the oracle both follow it)."""
    rng = np.random.default_rng(6200 + n)
    T = np.triu(randn_matrix(rng, n)) + 3 * np.diag(rng.standard_normal(n))
    s_o, sep_o = po.condition(T, nsub)
    assert _close(gs.eigvalscond(T, nsub), s_o)
    assert _close(gs.subspacesep(T, nsub), sep_o)
    S = gs.gschur(randn_matrix(rng, n))
    # a split that keeps every 2x2 block whole, then one through a block (the diagonal
    # difference of the two halves of a pair is 0 -> smin: ill-conditioned, looser check)
    whole = nsub if S.T[nsub, nsub - 1] == 0 else nsub + 1
    s_o, sep_o = po.condition(S.T, whole)
    assert _close(gs.eigvalscond(S, whole), s_o)
    assert _close(gs.subspacesep(S, whole), sep_o)
    cut = [k for k in range(1, n) if S.T[k, k - 1] != 0][0]
    s_o, sep_o = po.condition(S.T, cut)
    assert _close(gs.eigvalscond(S, cut), s_o, 1e-6)
    assert _close(gs.subspacesep(S, cut), sep_o, 1e-6)


def test_condition_repeated_eigenvalue(gs):
    """A repeated eigenvalue across the split: the diagonal difference is replaced by
    smin = max(small, eps |T11|_max |T22|_max) (sylvester.jl:55-60)."""
    rng = np.random.default_rng(6300)
    n = 50
    T = np.triu(randn_matrix(rng, n, cplx=True))
    T[30, 30] = T[3, 3]
    for nsub in (10, 25):
        s_o, sep_o = po.condition(T, nsub)
        assert _close(gs.eigvalscond(T, nsub), s_o, 1e-7)
        assert _close(gs.subspacesep(T, nsub), sep_o, 1e-7)


def test_condition_overflow_rescaling(gs):
    """An entry of the solution that would overflow: the reference rescales the whole
    right-hand side (scaloc = 1 / |v|_1, sylvester.jl:61-70); the GPU then reruns the
    solve in the reference's element order with the same rescaling."""
    rng = np.random.default_rng(6400)
    n = 40
    T = np.triu(randn_matrix(rng, n, cplx=True))
    T[1, 1] = T[0, 0]
    T[0, 1] = 1e290
    s_o, sep_o = po.condition(T, 1)
    s_g = gs.eigvalscond(T, 1)
    assert s_o < 1e-300  # subnormal: about 40 significant bits
    assert _close(s_g, s_o, 1e-9)
    sep_g = gs.subspacesep(T, 1)
    assert _close(sep_g, sep_o, 1e-9)


def test_condition_edges(gs):
    S, _ = _cplx_schur(gs, 10, 6500)
    assert gs.eigvalscond(S, 0) == 1.0
    assert gs.eigvalscond(S, 10) == 1.0
    with pytest.raises(gs.ArgumentError):
        gs.subspacesep(S, 0)
    T = np.array([[2.0, 1.0], [0.0, -1.0]])
    s_o, sep_o = po.condition(T, 1)
    assert _close(gs.eigvalscond(T, 1), s_o) and _close(gs.subspacesep(T, 1), sep_o)


def test_eigen_jcv(gs):
    """eigen!(A; jce = true, jcv = true): rconde[j] = eigvalscond and rcondv[j] =
    subspacesep after moving eigenvalue j to the front, the values LAPACK's trsen gives
    for select = e_j (and the oracle on trsen's reordered T)."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(6600)
    n = 24
    A = randn_matrix(rng, n, cplx=True)
    E = gs.eigen(A, permute=False, scale=False, jce=True, jcv=True, sortby=None)
    S = gs.gschur(A)
    assert np.allclose(E.values, S.values)
    for j in range(n):
        sel = np.zeros(n, dtype=np.int32)
        sel[j] = 1
        ts, _, _, _, s1, sep1, info = lapack.ztrsen(sel, S.T, S.Z, lwork=2 * n * n)
        assert info == 0
        s_o, sep_o = po.condition(ts, 1)
        assert _close(E.rconde[j], s1, 1e-7) and _close(E.rconde[j], s_o, 1e-7)
        assert _close(E.rcondv[j], sep1, 1e-7) and _close(E.rcondv[j], sep_o, 1e-7)


@pytest.mark.parametrize("possign", [False, True])
@pytest.mark.parametrize("adjoint", [False, True])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n", [(5, 7), (33, 65), (100, 40)])
def test_trsylvester_std(gs, m, n, cplx, adjoint, possign):
    """trsylvester!(A, B, C; possign) / adjtrsylvester! (sylvester.jl:11-139) through the
    C-ABI: the oracle's solution (the tiled GPU solve sums in another order) and the
    residual of the equation."""
    rng = np.random.default_rng(5200 + m + n + 2 * cplx + 4 * adjoint + 8 * possign)
    A = np.triu(randn_matrix(rng, m, cplx)) + 3 * np.eye(m)
    B = np.triu(randn_matrix(rng, n, cplx)) - 3 * np.eye(n)
    if possign:
        B = B + 6 * np.eye(n)
    C = randn_matrix(rng, max(m, n), cplx)[:m, :n]
    fn = gs.adjtrsylvester if adjoint else gs.trsylvester
    X, sc, pert = fn(A, B, C, possign=possign)
    Xo, so, po_ = po.trsylvester(A, B, C, adjoint=adjoint, possign=possign)
    assert sc == so == 1.0 and pert == po_
    assert np.abs(X - Xo).max() <= 1e-10 * np.abs(Xo).max()
    sg = 1.0 if possign else -1.0
    Ah, Bh = (A.conj().T, B.conj().T) if adjoint else (A, B)
    res = Ah @ X + sg * X @ Bh - C
    assert np.abs(res).max() <= 1e-12 * (np.abs(A).max() + np.abs(B).max()) * np.abs(X).max()


def test_trsylvester_std_rescale(gs):
    """A solution past the overflow threshold: the reference's rescaling (scale < 1), in its
    element order, to the oracle's scale and solution; and a shared eigenvalue perturbed."""
    A, B, C = np.array([[1e-200]]), np.array([[-1e-200]]), np.array([[1e100]])
    X, sc, pert = gs.trsylvester(A, B, C)
    Xo, so, _ = po.trsylvester(A, B, C)
    assert sc == so and sc < 1.0 and X[0, 0] == Xo[0, 0]
    A = np.triu(np.ones((3, 3)))
    B = np.triu(np.ones((2, 2)))
    X, sc, pert = gs.trsylvester(A, B, np.ones((3, 2)))
    _, _, po_ = po.trsylvester(A, B, np.ones((3, 2)))
    assert pert and po_
