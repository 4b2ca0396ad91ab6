"""Pin the CPU oracle against the reference's own known answers and property tests.

The oracle is the checker for every GPU parity test, so it is validated here
first, on the CPU:
  * Godunov's matrix, exact eigenvalues {-4,-2,-1,0,1,2,4} (test/testfuncs.jl:127-142,
    test/real.jl:142-157, test/complex.jl:139-154), in 113-bit arithmetic;
  * schurtest / hesstest / vectest properties (test/real.jl, test/complex.jl,
    test/testfuncs.jl) on random, Jordan, orthogonal and scaled matrices;
  * the near-degenerate _gs2x2! case (test/real.jl:311-317);
  * the non-real-subdiagonal ArgumentError (test/errors.jl:1-5);
  * the committed golden fixtures (tests/golden, made by make_golden.py).
"""
import os

import numpy as np
import pytest

from common import (EPS, assert_schur_cplx, assert_schur_real, backward_error, check_gordschur_real, check_gsyl_errors,
                    checkblocks, godunov,
                    st_errors, st_testmat1, st_testmat2,
                    gsyl_errors, gsyl_problem, kp_pencil, kp_truth, orth_error, randn_matrix)
from oracle import pyoracle as po

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_godunov_real_quad():
    A, vals, econd = godunov()
    T, Z, w, (be, oe) = po.gschur_quad(A)
    # reference tolerance: delta < 100 eps(80-bit) ||A||, t = 3 delta econd (test/real.jl:148-151)
    delta = be * np.linalg.norm(A)
    assert delta < 100 * 2.0 ** -79 * np.linalg.norm(A)
    t = 3 * delta * econd
    got = np.sort(w.real)
    assert np.all(np.abs(w.imag) <= t)
    assert np.allclose(got, vals, atol=max(t, 1e-12))


def test_godunov_complex_quad():
    A, vals, econd = godunov()
    T, Z, w, (be, oe) = po.gschur_cplx_quad(A.astype(np.complex128))
    delta = be * np.linalg.norm(A)
    assert delta < 100 * 2.0 ** -79 * np.linalg.norm(A)
    t = 3 * delta * econd
    got = w[np.lexsort((w.imag, w.real))]
    assert np.allclose(got, vals, atol=max(t, 1e-12))


def _mp_available():
    try:
        po.mplib()
        return True
    except OSError:
        return False


@pytest.mark.skipif(not _mp_available(), reason="the 256-bit oracle needs libmpfr.so.6")
def test_godunov_256bit():
    """Godunov's known answer at BigFloat precision (256 bits), as the reference's BigFloat
    tests run it: with delta ~ 2^-256 ||A|| the eigenvalues (condition ~7e16) are exact to
    far below FP64 rounding, so they round to {-4, -2, -1, 0, 1, 2, 4} (test/real.jl:142-157,
    test/testfuncs.jl:127-142), real and complex drivers alike."""
    A, vals, econd = godunov()
    for fn, M in ((po.gschur_mp, A), (po.gschur_cplx_mp, A.astype(np.complex128))):
        T, Z, w, (be, oe) = fn(M)
        assert be < 100 * 2.0 ** -255 and oe < 100 * 2.0 ** -255
        t = 3 * be * np.linalg.norm(A) * econd
        assert t < 1e-50
        got = w[np.lexsort((w.imag, w.real))]
        assert np.all(np.abs(got.imag) <= 1e-50)
        assert np.allclose(got.real, vals, rtol=0, atol=1e-50)


@pytest.mark.skipif(not _mp_available(), reason="the 256-bit oracle needs libmpfr.so.6")
@pytest.mark.parametrize("n", [5, 24])
def test_oracle_256bit_vs_113bit(n):
    """The 256-bit and 113-bit instances of the same restatement agree on random inputs
    (to FP64 rounding of the 113-bit eigenvalues), with residuals at their own precision."""
    rng = np.random.default_rng(7100 + n)
    A = rng.standard_normal((n, n))
    _, _, wm, (bm, om) = po.gschur_mp(A)
    _, _, wq, (bq, oq) = po.gschur_quad(A)
    assert bm < 1e-74 and om < 1e-74 and bq < 1e-31
    assert np.max(np.abs(np.sort_complex(wm) - np.sort_complex(wq))) <= 1e-14 * np.abs(wq).max()


def test_mp256_fixture_pins_fp64_oracle():
    """The 256-bit fixture of the n = 256 inputs (BigFloat precision): residuals at that
    precision, agreement with the 113-bit fixture, and the FP64 oracle's eigenvalues
    within the parity tolerance of it."""
    from common import eig_tolerances, match_eigenvalues
    path = os.path.join(GOLDEN, "mp256_n256.npz")
    if not os.path.exists(path):
        pytest.skip("no 256-bit fixture")
    G = np.load(path)
    Q = np.load(os.path.join(GOLDEN, "quad_256.npz"))
    assert max(G["res_c256"]) < 1e-70 and max(G["res_cond256"]) < 1e-70
    for key in ("c256", "cond256"):
        np.testing.assert_array_equal(G["A_" + key], Q["A_" + key])
        A = G["A_" + key]
        w, tol = eig_tolerances(A, po)
        ok, worst = match_eigenvalues(w, G["w_" + key], tol)
        assert ok, "%s: worst err/tol %.3g" % (key, worst)
        # the 113-bit eigenvalues are the 256-bit ones to far below the parity tolerance
        ok, worst = match_eigenvalues(Q["w_" + key], G["w_" + key], tol * 1e-10)
        assert ok, "%s: 113-bit vs 256-bit worst err/tol %.3g" % (key, worst)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 32, 64])
def test_oracle_real_random(n):
    rng = np.random.default_rng(100 + n)
    A = rng.random((n, n))
    T, Z, w = po.gschur_real(A)
    assert_schur_real(A, T, Z, w, tol=10.0)
    # eigenvalues agree with LAPACK (third-party cross-check)
    ev = np.linalg.eigvals(A)
    assert np.allclose(np.sort_complex(ev), np.sort_complex(w), atol=1e-10 * max(1, np.abs(ev).max()))


@pytest.mark.parametrize("n", [1, 2, 4, 32])
def test_oracle_complex_random(n):
    rng = np.random.default_rng(200 + n)
    A = rng.random((n, n)) + 1j * rng.random((n, n))
    T, Z, w = po.gschur_cplx(A)
    assert_schur_cplx(A, T, Z, w, tol=10.0)


@pytest.mark.parametrize("n", [4, 32])
def test_oracle_orthogonal_normal(n):
    # random orthogonal: Schur form is block diagonal (test/real.jl:133-138)
    rng = np.random.default_rng(300 + n)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    T, Z, w = po.gschur_real(Q)
    assert_schur_real(Q, T, Z, w, tol=10.0)
    assert np.linalg.norm(np.triu(T, 2)) / (n * np.linalg.norm(Q) * EPS) < 10


@pytest.mark.parametrize("n", [4, 32])
def test_oracle_jordan(n):
    A = np.diag(np.ones(n - 1), 1) + np.eye(n)  # test/real.jl:180-191
    T, Z, w = po.gschur_real(A)
    assert_schur_real(A, T, Z, w, tol=20.0)


@pytest.mark.parametrize("scale", [100 * np.finfo(float).tiny, np.finfo(float).max / 100])
def test_oracle_hessenberg_extreme_scale(scale):
    # hesstest with tiny and huge entries (test/real.jl:104-116)
    rng = np.random.default_rng(7)
    n = 32
    A = scale * rng.random((n, n))
    H, tau, Q = po.hessenberg(A)
    HH = np.triu(H, -1)
    As, HHs = A / scale, HH / scale
    assert np.linalg.norm(As - Q @ HHs @ Q.T) / (n * np.linalg.norm(As) * EPS) < 10
    assert np.linalg.norm(np.eye(n) - Q @ Q.T) / (n * EPS) < 10


def test_oracle_scaled_schur():
    # _scale! path: entries near overflow and underflow (test/real.jl:178, magns)
    rng = np.random.default_rng(8)
    for s in (1e-300, 1e300):
        A = s * rng.standard_normal((16, 16))
        T, Z, w = po.gschur_real(A)
        be = np.linalg.norm(A / s - Z @ (T / s) @ Z.T) / np.linalg.norm(A / s)
        assert be <= 10 * 16 * EPS
        assert orth_error(Z) <= 10 * 16 * EPS


@pytest.mark.parametrize("n", [2, 5, 32])
def test_oracle_vectest(n):
    rng = np.random.default_rng(400 + n)
    for cplx in (False, True):
        A = randn_matrix(rng, n, cplx)
        T, Z, w = po.gschur(A)
        VR = po.eigvecs(T, Z, left=False)
        VL = po.eigvecs(T, Z, left=True)
        nA = np.linalg.norm(A)
        assert np.linalg.norm(A @ VR - VR @ np.diag(w)) / (n * nA * EPS) < 20
        assert np.linalg.norm(A.conj().T @ VL - VL @ np.diag(w.conj())) / (n * nA * EPS) < 20
        # _enormalize!: unit norm, largest entry real (util.jl:572-592)
        assert np.all(np.abs(np.linalg.norm(VR, axis=0) - 1) / (n * EPS) < 10)
        for j in range(n):
            assert VR[np.argmax(np.abs(VR[:, j])), j].imag == 0


def test_oracle_triangularize():
    rng = np.random.default_rng(9)
    n = 32
    A = rng.standard_normal((n, n))
    T, Z, w = po.gschur_real(A)
    Tc, Zc, wc = po.triangularize(T, Z)
    assert np.all(np.tril(Tc, -1) == 0)
    assert np.linalg.norm(A - Zc @ Tc @ Zc.conj().T) / (n * np.linalg.norm(A) * EPS) < 10
    assert np.linalg.norm(np.eye(n) - Zc @ Zc.conj().T) / (n * EPS) < 10
    assert np.array_equal(np.sort_complex(wc), np.sort_complex(np.diag(Tc)))


def test_oracle_gs2x2_near_degenerate():
    # test/real.jl:311-317
    rng = np.random.default_rng(10)
    l1, l2 = 1 + 2 * EPS, 1 - 2 * EPS
    B = np.diag([l1, l2]) + (EPS / 4) * rng.random((2, 2))
    Bs, cs, sn, w1, w2 = po.gs2x2(B)
    assert abs(max(w1.real, w2.real) - l1) < 2 * EPS
    assert abs(min(w1.real, w2.real) - l2) < 2 * EPS


def test_oracle_nonreal_subdiagonal_raises():
    # test/errors.jl:2-5
    n = 5
    rng = np.random.default_rng(11)
    A = np.diag(np.full(n - 1, -1.0 + 1.0j), -1) + np.triu(rng.random((n, n)))
    st, _, _, _ = po.gschur_hess_cplx(A)
    assert st == 2


def test_oracle_unconverged():
    rng = np.random.default_rng(12)
    with pytest.raises(po.Unconverged):
        po.gschur_real(rng.standard_normal((16, 16)), maxiter=2)


def test_oracle_golden_fixtures():
    """The oracle reproduces the committed golden outputs bit for bit."""
    path = os.path.join(GOLDEN, "oracle_golden.npz")
    g = np.load(path)
    for key in [k for k in g.files if k.startswith("A_")]:
        tag = key[2:]
        A = g[key]
        T, Z, w = po.gschur(A)
        np.testing.assert_array_equal(T, g["T_" + tag])
        np.testing.assert_array_equal(Z, g["Z_" + tag])
        np.testing.assert_array_equal(w, g["w_" + tag])


def test_quad_fixture_pins_fp64_oracle():
    """The 113-bit fixture of the n = 256 inputs: its own residuals are at quad level,
    and the FP64 oracle's eigenvalues agree with it within the parity tolerance."""
    import os
    from common import eig_tolerances, match_eigenvalues
    G = np.load(os.path.join(os.path.dirname(__file__), "golden", "quad_256.npz"))
    assert max(G["res_c256"]) < 1e-28 and max(G["res_cond256"]) < 1e-28
    for key in ("c256", "cond256"):
        A = G["A_" + key]
        w, tol = eig_tolerances(A, po)
        ok, worst = match_eigenvalues(w, G["w_" + key], tol)
        assert ok, "%s: worst err/tol %.3g" % (key, worst)


def test_oracle_balance_restatement():
    """balance! restated (balance.jl:33-185): eigenvalues are preserved, the block
    structure [T1 X Y; 0 C Z; 0 0 T2] holds, and lmul!(B, V) maps eigenvectors of the
    balanced matrix to eigenvectors of A."""
    rng = np.random.default_rng(4700)
    A = rng.standard_normal((10, 10))
    A[7:, :7] = 0.0
    A[8, 7] = 0.0
    A[9, 7:9] = 0.0
    d = 10.0 ** rng.integers(-4, 5, size=10)
    A = (A * d[None, :]) / d[:, None]
    Ab, B = po.balance(A)
    ilo, ihi = B[0], B[1]
    assert np.all(Ab[ihi:, :ihi] == 0) and np.all(Ab[ilo - 1:, :ilo - 1] == 0)
    wb, Vb = np.linalg.eig(Ab)
    V = po.balancer_apply(Vb, B)
    assert np.linalg.norm(A @ V - V @ np.diag(wb)) <= 1e-10 * np.linalg.norm(A) * np.linalg.norm(V)


@pytest.mark.parametrize("cplx", [True, False])
def test_oracle_condition_vs_trsen(cplx):
    """eigvalscond / subspacesep restated (ordschur.jl:84-140 over sylvester.jl and
    norm1est.jl), pinned as the reference pins them (test/ordschur.jl:35-54): equal to
    LAPACK's trsen s and sep for the same reordered Schur form.  Complex forms from
    random matrices; real forms upper triangular (the reference's solver reads only the
    upper triangle)."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    import scipy.linalg as sl
    rng = np.random.default_rng(4900 + cplx)
    for trial in range(4):
        n = 32
        sel = np.zeros(n, dtype=np.int32)
        sel[rng.integers(0, n, 3)] = 1
        if cplx:
            T0, Z0 = sl.schur(rng.random((n, n)) + 1j * rng.random((n, n)), output="complex")
            ts, _, _, m, s1, sep1, info = lapack.ztrsen(sel, T0, Z0, lwork=2 * n * n)
        else:
            T0 = np.triu(rng.standard_normal((n, n))) + 4 * np.diag(rng.standard_normal(n))
            ts, _, _, _, m, s1, sep1, info = lapack.dtrsen(sel, T0, np.eye(n), lwork=2 * n * n, liwork=n * n)
        assert info == 0
        s2, sep2 = po.condition(ts, int(m))
        assert abs(s1 - s2) <= 1e-8 * s1
        assert abs(sep1 - sep2) <= 1e-8 * sep1


def test_oracle_trsylvester_residual():
    """trsylvester! / adjtrsylvester! restated (sylvester.jl:11-139): A X - X B = C and
    A^H X - X B^H = C to working accuracy; a repeated eigenvalue is perturbed to smin."""
    rng = np.random.default_rng(4950)
    for cplx in (False, True):
        m, p = 7, 11
        A = np.triu(randn_matrix(rng, m, cplx))
        B = np.triu(randn_matrix(rng, p, cplx))
        C = randn_matrix(rng, m, cplx)[:, :1] @ randn_matrix(rng, p, cplx)[:1, :] + \
            (rng.standard_normal((m, p)) if not cplx else rng.standard_normal((m, p)) * 1j)
        X, scale, pert = po.trsylvester(A, B, C)
        assert scale == 1.0 and not pert
        assert np.linalg.norm(A @ X - X @ B - C) <= 100 * EPS * np.linalg.norm(X) * (np.linalg.norm(A) + np.linalg.norm(B))
        Xh, scale, pert = po.trsylvester(A, B, C, adjoint=True)
        Ah, Bh = A.conj().T, B.conj().T
        assert np.linalg.norm(Ah @ Xh - Xh @ Bh - C) <= 100 * EPS * np.linalg.norm(Xh) * (np.linalg.norm(A) + np.linalg.norm(B))
    A = np.triu(rng.standard_normal((3, 3)))
    B = np.triu(rng.standard_normal((2, 2)))
    B[1, 1] = A[0, 0]
    _, _, pert = po.trsylvester(A, B, rng.standard_normal((3, 2)))
    assert pert


@pytest.mark.parametrize("adjoint", [False, True])
@pytest.mark.parametrize("m,n", [(2, 4), (4, 2), (24, 24)])
def test_oracle_gsylvester(m, n, adjoint):
    """trsylvester! / adjtrsylvester! for pencils restated (gsylvester.jl:23-155), on the
    reference's checkgsyl / checkgasyl problems."""
    rng = np.random.default_rng(1234 + 10 * m + n + adjoint)
    A, B, C, D, E, F, X, Y = gsyl_problem(rng, m, n, adjoint)
    X2, Y2, scale = po.gtrsylvester(A, B, C, D, E, F, adjoint=adjoint)
    assert scale == 1.0
    check_gsyl_errors(m, n, gsyl_errors(A, B, C, D, E, F, X, Y, X2, Y2, scale, adjoint))


def test_oracle_geigvalscond_vs_tgsen():
    """eigvalscond(S::GeneralizedSchur) restated (gcondition.jl:121-165): pl and pr equal
    LAPACK ztgsen's (ijob = 4), which solves the same generalized Sylvester equation."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(4242)
    for n, k in ((8, 3), (16, 1), (40, 20), (60, 59)):
        A = randn_matrix(rng, n, True)
        B = randn_matrix(rng, n, True)
        S, T, al, be, Q, Z, st = po.ggschur(A, B)
        assert st == 0
        sel = np.zeros(n, np.int32)
        sel[:k] = 1
        r = lapack.ztgsen(sel, S, T, Q, Z, ijob=4, lwork=2 * n * n + 4, liwork=2 * n * n + 8)
        assert r[-1] == 0
        pl, pr = po.geigvalscond(S, T, k)
        assert abs(pl - r[7]) <= 1e-12 * pl and abs(pr - r[8]) <= 1e-12 * pr
        # the look-ahead separations estimate the same quantities as ztgsen's dif (whose
        # 2 x 2 solves pivot completely where the reference's lu pivots by rows)
        sep = po.gsubspacesep(S, T, k)
        assert np.all(sep > 0) and np.all(np.abs(np.log10(sep / r[9])) < 1)


@pytest.mark.parametrize("dtype", [2, 1])
def test_oracle_gcondition_kptest(dtype):
    """KPTest (test/gordschur.jl:193-295, alpha = beta = x = y = 1): every eigenvalue of the
    CHK4 pencil moved to the front by gordschur!, then pl, pr within two orders of magnitude
    of its known reciprocal condition and sep within two orders of Difl."""
    A, B, atrue, YH, X = kp_pencil(dtype=dtype)
    S, T, al, be, Q, Z, st = po.ggschur(A, B)
    assert st == 0
    est = al / be
    for j in range(5):
        idx = int(np.argmin(np.abs(est - atrue[j])))
        sel = np.zeros(5, np.int32)
        sel[idx] = 1
        if idx == 0:
            S2, T2 = S, T
        else:
            S2, T2, _, _, _, _, st = po.ggordschur(S, T, Q, Z, sel)
            assert st == 0
        pl, pr = po.geigvalscond(S2, T2, 1)
        sep = po.gsubspacesep(S2, T2, 1)
        rcond, difl = kp_truth(A, B, YH, X, S2, T2, j, atrue[j], dtype)
        assert abs(np.log10(pl / rcond)) < 2 and abs(np.log10(pr / rcond)) < 2
        assert abs(np.log10(sep[0] / difl)) < 2 and abs(np.log10(sep[1] / difl)) < 2


def test_oracle_gsubspacesep_onenorm():
    """subspacesep(.; pnorm = 1) with the solves applied in place: 1 / est is a lower
    bound on the one-norm of the inverse generalized Sylvester operator (its Kronecker
    form), and for these pencils within a factor of three of it."""
    rng = np.random.default_rng(777)
    for n, k in ((6, 2), (12, 5), (20, 19)):
        A = randn_matrix(rng, n, True)
        B = randn_matrix(rng, n, True)
        S, T, *_ = po.ggschur(A, B)
        sep = po.gsubspacesep1(S, T, k)
        for (A_, B_, D_, E_), s in zip(((S[:k, :k], S[k:, k:], T[:k, :k], T[k:, k:]),
                                        (S[k:, k:], S[:k, :k], T[k:, k:], T[:k, :k])), sep):
            m, q = A_.shape[0], B_.shape[0]
            Im, Iq = np.eye(m), np.eye(q)
            Zk = np.block([[np.kron(Iq, A_), -np.kron(B_.T, Im)], [np.kron(Iq, D_), -np.kron(E_.T, Im)]])
            inv1 = np.linalg.norm(np.linalg.inv(Zk), 1)
            assert 1.0 / s <= inv1 * (1 + 1e-10)
            assert 1.0 / s >= inv1 / 3


@pytest.mark.parametrize("n", [32, 100, 257])
def test_oracle_stedc_batch(n):
    """The reference's SymTridiagonal batch (test/symtridiag.jl:158-178, 221-225) with
    DivideAndConquer(): both matrix classes, residual and orthogonality below 50 (scaled by
    n eps); the reference runs it at n = 32 (one merge), the larger orders build deeper trees.
    The eigenvalues also match LAPACK's (numpy eigvalsh) to 50 n eps |T|."""
    rng = np.random.default_rng(2100 + n)
    cases = [st_testmat1(n, it, rng) for it in range(1, 10)] + [st_testmat2(n, it) for it in range(1, 9)]
    for D, E in cases:
        lam, V, st = po.stedc(D, E)
        assert st == 0
        de, ve = st_errors(D, E, lam, V)
        assert de < 50 and ve < 50, (de, ve)
        T = np.diag(D) + np.diag(E, 1) + np.diag(E, -1)
        ref = np.linalg.eigvalsh(T)
        assert np.abs(np.sort(lam) - ref).max() <= 50 * len(D) * EPS * np.abs(T).max()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_ggordschur_real_checkord(seed):
    """gordschur! for real pencils restated (rordschur.jl:542-1178) on the reference's real
    checkord problem (test/gordschur.jl:90-137: A = rand, B = rand - 1/2 + I, n = 16, the
    second half selected) and on a random selection at n = 40: quasi-triangular, backward
    stable, orthogonal, and exactly the selected eigenvalues (pairs travel together) lead."""
    rng = np.random.default_rng(1600 + seed)
    for n, half in ((16, True), (40, False)):
        A = rng.random((n, n))
        B = rng.random((n, n)) - 0.5 + np.eye(n)
        S, T, al, be, Q, Z, st = po.ggschur_real(A, B)
        assert st == 0
        sel = np.ones(n, np.int32)
        if half:
            sel[: n >> 1] = 0
        else:
            sel = rng.integers(0, 2, n).astype(np.int32)
        S2, T2, a, b, Q2, Z2, st = po.ggordschur_real(S, T, Q, Z, sel)
        assert st == 0
        check_gordschur_real(A, B, al / be, sel, S2, T2, a, b, Q2, Z2)


def test_oracle_gsubspacesep_onenorm_vs_tgsen():
    """subspacesep(.; pnorm = 1) restated with the solves applied in place: its Difu equals
    LAPACK ztgsen's one-norm estimate (ijob = 5) on these pencils, where both estimators reach
    the exact 1 / |Zu^-1|_1 (Difl differs: the estimators take different steps there)."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(5)
    for n, k in ((8, 3), (16, 1), (20, 10), (30, 29), (24, 5)):
        A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        S, T, al, be, Q, Z, st = po.ggschur(A, B)
        assert st == 0
        sel = np.zeros(n, np.int32)
        sel[:k] = 1
        r = lapack.ztgsen(sel, S, T, Q, Z, ijob=5, lwork=2 * n * n + 4, liwork=2 * n * n + 8)
        assert r[-1] == 0
        sep = po.gsubspacesep1(S, T, k)
        assert abs(sep[0] - r[9][0]) <= 1e-10 * r[9][0]


def test_oracle_ggordschur_real_vs_tgsen():
    """The real-pencil reordering restated (rordschur.jl:542-1178, after dtgexc / dtgex2)
    against LAPACK dtgsen (ijob = 0) on the same generalized Schur pair and selection: the
    same eigenvalue order and the same leading deflating subspaces."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    from common import selected_with_pairs
    rng = np.random.default_rng(9)
    for trial in range(6):
        n = 16 if trial < 3 else 30
        A = rng.random((n, n))
        B = rng.random((n, n)) - 0.5 + np.eye(n)
        S, T, al, be, Q, Z, st = po.ggschur_real(A, B)
        assert st == 0
        sel = rng.integers(0, 2, n).astype(np.int32)
        S2, T2, a2, b2, Q2, Z2, st2 = po.ggordschur_real(S, T, Q, Z, sel)
        assert st2 == 0
        r = lapack.dtgsen(sel, S, T, Q, Z, ijob=0, lwork=4 * n * n + 4 * n + 16, liwork=n + 8)
        assert r[-1] == 0
        lv = (r[2] + 1j * r[3]) / r[4]
        ov = a2 / b2
        assert np.abs(lv - ov).max() <= 1e-12 * np.abs(ov).max()
        k = int(selected_with_pairs(al / be, sel).sum())
        for Mo, Ml in ((Z2, r[6]), (Q2, r[5])):
            assert np.abs(Mo[:, :k] @ Mo[:, :k].T - Ml[:, :k] @ Ml[:, :k].T).max() <= 1e-12


def test_oracle_ggordschur_cplx_vs_tgsen():
    """The complex-pencil reordering restated (ordschur.jl:147-305, after ztgexc / ztgex2)
    against LAPACK ztgsen (ijob = 0): the same eigenvalue order and leading deflating
    subspaces."""
    lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(10)
    for trial in range(4):
        n = 16 if trial < 2 else 30
        A = randn_matrix(rng, n, True)
        B = randn_matrix(rng, n, True)
        S, T, al, be, Q, Z, st = po.ggschur(A, B)
        assert st == 0
        sel = rng.integers(0, 2, n).astype(np.int32)
        S2, T2, a2, b2, Q2, Z2, st2 = po.ggordschur(S, T, Q, Z, sel)
        assert st2 == 0
        r = lapack.ztgsen(sel, S, T, Q, Z, ijob=0, lwork=4 * n * n + 16, liwork=n + 8)
        assert r[-1] == 0
        ov = a2 / b2
        assert np.abs(r[2] / r[3] - ov).max() <= 1e-12 * np.abs(ov).max()
        k = int(sel.sum())
        for Mo, Ml in ((Z2, r[5]), (Q2, r[4])):
            assert np.abs(Mo[:, :k] @ Mo[:, :k].conj().T - Ml[:, :k] @ Ml[:, :k].conj().T).max() <= 1e-12


def _match_sets(a, b):
    from scipy.optimize import linear_sum_assignment
    C = np.abs(a[:, None] - b[None, :]) / np.maximum(1.0, np.abs(b[None, :]))
    r, c = linear_sum_assignment(C)
    return float(C[r, c].max())


@pytest.mark.parametrize("cplx", [False, True])
def test_oracle_hermitian_and_qz_vs_lapack(cplx):
    """The Hermitian (hessenberg.jl, symtridiag.jl) and QZ (generalized.jl, rgeneralized.jl)
    restatements against LAPACK on the same inputs: eigenvalues (eigh / ggev), the
    decompositions' backward errors, and the generalized eigenvectors' residuals
    (vectors.jl:723-1513): beta A v = alpha B v, u^H (beta A - alpha B) = 0."""
    import scipy.linalg
    rng = np.random.default_rng(8800 + cplx)
    n = 24
    H = randn_matrix(rng, n, cplx)
    H = (H + H.conj().T) / 2
    for uplo in ("L", "U"):
        w, V, st = po.heev(H, uplo)
        assert st == 0
        assert np.abs(w - np.linalg.eigvalsh(H)).max() <= 20 * n * EPS * np.abs(H).max()
        assert np.abs(H @ V - V * w).max() <= 20 * n * EPS * np.abs(H).max()
    A = randn_matrix(rng, n, cplx)
    B = randn_matrix(rng, n, cplx)
    if cplx:
        S, T, al, be, Q, Z, st = po.ggschur(A, B)
        VR = po.ggeigvecs(S, T, Z)
        VL = po.ggeigvecs(S, T, Q, left=True)
    else:
        S, T, al, be, Q, Z, st = po.ggschur_real(A, B)
        VR = po.rgeigvecs(S, T, Z)
        VL = po.rgeigvecs(S, T, Q, left=True)
    assert st == 0
    nA, nB = np.linalg.norm(A), np.linalg.norm(B)
    assert np.linalg.norm(A - Q @ S @ Z.conj().T) <= 20 * n * EPS * nA
    assert np.linalg.norm(B - Q @ T @ Z.conj().T) <= 20 * n * EPS * nB
    assert _match_sets(al / be, scipy.linalg.eigvals(A, B)) < 1e-8
    for j in range(n):
        r = be[j] * (A @ VR[:, j]) - al[j] * (B @ VR[:, j])
        assert np.linalg.norm(r) <= 1e3 * n * EPS * (abs(be[j]) * nA + abs(al[j]) * nB) * np.linalg.norm(VR[:, j])
        l = VL[:, j].conj() @ (be[j] * A - al[j] * B)
        assert np.linalg.norm(l) <= 1e3 * n * EPS * (abs(be[j]) * nA + abs(al[j]) * nB) * np.linalg.norm(VL[:, j])
