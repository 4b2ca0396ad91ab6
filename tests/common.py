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


def kp_pencil(alpha=1.0, beta=1.0, x=1.0, y=1.0, dtype=2):
    """The CHK4 pencils of Kagstrom and Poromaa (LAWN 87) as the reference's KPTest builds
    them (test/gordschur.jl:203-225): A = YH \\ (Da / X), B = YH \\ (I / X), with known
    eigenvalues atrue and eigenvector factors YH, X."""
    n = 5
    if dtype == 1:
        Da = np.diag(np.array([1, 2, 3, 4, 5], dtype=complex)) + alpha * np.eye(n)
        atrue = np.array([1, 2, 3, 4, 5], dtype=complex) + alpha
    else:
        Da = (np.diag(np.array([1, 1, 1, 1 + alpha, 1 + alpha], dtype=complex))
              + np.diag(np.array([-1, 0, 0, 1 + beta], dtype=complex), 1)
              + np.diag(np.array([1, 0, 0, -1 - beta], dtype=complex), -1))
        atrue = np.array([1 - 1j, 1 + 1j, 1, 1 + alpha - (1 + beta) * 1j, 1 + alpha + (1 + beta) * 1j])
    YH = (np.eye(n, dtype=complex) + np.diag([0, -y, 0, 0], 1) + np.diag([-y, y, 0], 2)
          + np.diag([y, -y], 3) + np.diag([-y], 4))
    X = (np.eye(n, dtype=complex) + np.diag([0, x, 0, 0], 1) + np.diag([-x, -x, 0], 2)
         + np.diag([-x, -x], 3) + np.diag([x], 4))
    A = np.linalg.solve(YH, Da @ np.linalg.inv(X))
    B = np.linalg.solve(YH, np.linalg.inv(X))
    return A, B, atrue, YH, X


def kp_truth(A, B, YH, X, S2, T2, j, lam, dtype):
    """The known reciprocal condition of eigenvalue j and Difl of the reordered pair
    (S2, T2) with lam in front (test/gordschur.jl:238-268)."""
    n = 5
    if dtype == 1 or j == 2:
        yv, xv = YH[j, :], X[:, j]
    else:
        rows = {0: (0, 1, 1), 1: (0, 1, -1), 3: (3, 4, -1), 4: (3, 4, 1)}[j]
        a, b, sgn = rows
        yv = YH[a, :] + sgn * 1j * YH[b, :]
        xv = X[:, a] + sgn * 1j * X[:, b]
    # dot(y, M x) conjugates y
    rcond = (np.sqrt(abs(np.vdot(yv, A @ xv)) ** 2 + abs(np.vdot(yv, B @ xv)) ** 2)
             / (np.linalg.norm(xv) * np.linalg.norm(yv))) / np.sqrt(3.0)
    I4 = np.eye(n - 1)
    Zl = np.block([[lam * I4, -S2[1:, 1:]], [I4, -T2[1:, 1:]]])
    difl = np.linalg.svd(Zl, compute_uv=False).min()
    return rcond, difl


def gsyl_problem(rng, m, n, adjoint):
    """checkgsyl / checkgasyl (test/gordschur.jl:6-74): triangular A, B, D, E with separated
    spectra and right-hand sides made from known X, Y."""
    r = 0.5 * (1 + 1j)
    A = np.triu(rng.random((m, m)) + 1j * rng.random((m, m)) - r) + 2 * np.eye(m)
    B = np.triu(rng.random((n, n)) + 1j * rng.random((n, n)) - r) + np.eye(n)
    X = rng.random((m, n)) + 1j * rng.random((m, n))
    D = np.triu(rng.random((m, m)) + 1j * rng.random((m, m)) - r) + 4 * np.eye(m)
    E = np.triu(rng.random((n, n)) + 1j * rng.random((n, n)) - r) + np.eye(n)
    Y = rng.random((m, n)) + 1j * rng.random((m, n))
    if adjoint:
        C = A.conj().T @ X + D.conj().T @ Y
        F = -X @ B.conj().T - Y @ E.conj().T
    else:
        C = A @ X - Y @ B
        F = D @ X - Y @ E
    return A, B, C, D, E, F, X, Y


def gsyl_errors(A, B, C, D, E, F, X, Y, X2, Y2, scale, adjoint):
    fa = np.linalg.norm(scale * X - X2) / np.linalg.norm(X)
    fb = np.linalg.norm(scale * Y - Y2) / np.linalg.norm(Y)
    if adjoint:
        ra = A.conj().T @ X2 + D.conj().T @ Y2 - scale * C
        rb = X2 @ B.conj().T + Y2 @ E.conj().T + scale * F
    else:
        ra = A @ X2 - Y2 @ B - scale * C
        rb = D @ X2 - Y2 @ E - scale * F
    nx = np.linalg.norm(X)
    ba = np.linalg.norm(ra) / ((np.linalg.norm(A) + np.linalg.norm(B)) * nx)
    bb = np.linalg.norm(rb) / ((np.linalg.norm(D) + np.linalg.norm(E)) * nx)
    return fa, fb, ba, bb


def check_gsyl_errors(m, n, errs):
    # the reference's bounds: tol = 2, forward errors only below order 10
    fa, fb, ba, bb = errs
    stol = 2 * max(m, n) * EPS
    if max(m, n) < 10:
        assert fa < np.sqrt(stol) and fb < np.sqrt(stol)
    assert ba < 2 and bb < 2
    # and the working accuracy actually reached
    assert ba < 100 * EPS and bb < 100 * EPS


# ---- symmetric tridiagonal test matrices (test/symtridiag.jl:9-176) ----------------------
def _wilkinson(n):
    if n % 2 == 1:
        nh = (n - 1) // 2
        D = np.concatenate([np.arange(nh, 0, -1), [0], np.arange(1, nh + 1)]).astype(float)
    else:
        D = np.abs(np.arange(-(n - 1), n, 2, dtype=float) / 2)
    return D, np.ones(n - 1)


def st_testmat1(n, itype, rng):
    """LAPACK-style class 1 (test/symtridiag.jl:50-103): A = Q' diag(lam) Q for a random
    orthogonal Q, reduced to tridiagonal form; returns (d, e)."""
    ulp = np.finfo(float).eps
    kpar = 1 / ulp
    lam = np.zeros(n)
    j = np.arange(1, n + 1)
    if itype == 1:
        lam = 1.0 / j
    elif itype == 2:
        lam[:] = 1.0
        lam[-1] = 1.0 / n
    elif itype == 3:
        lam = 1.0 / kpar ** ((j - 1) / (n - 1))
    elif itype == 4:
        lam = 1.0 - ((j - 1) / (n - 1)) * (1 - 1 / kpar)
    elif itype == 5:
        lam = np.exp(-np.log(n) * rng.random(n))
    elif itype == 6:
        lam = rng.standard_normal(n)
    elif itype == 7:
        lam[:-1] = np.arange(1, n) * ulp
        lam[-1] = 1.0
    elif itype == 8:
        lam[0] = ulp
        lam[1:-1] = 1 + np.sqrt(ulp) * np.arange(2, n)
        lam[-1] = 2.0
    elif itype == 9:
        lam[0] = 1.0
        for k in range(1, n):
            lam[k] = lam[k - 1] + 100 * ulp
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = Q.T @ np.diag(lam) @ Q
    import scipy.linalg
    H = scipy.linalg.hessenberg((A + A.T) / 2)
    return np.diag(H).copy(), np.diag(H, -1).copy()


def st_testmat2(n, itype):
    """Class 2 (test/symtridiag.jl:107-155): constant, Wilkinson, Clement, Legendre, Laguerre,
    Hermite, and three Wilkinson blocks at extreme scales glued with zero couplings."""
    ulp = np.finfo(float).eps
    i = np.arange(1, n)
    if itype == 1:
        return np.ones(n), np.zeros(n - 1)
    if itype == 2:
        return np.full(n, 2.0), np.ones(n - 1)
    if itype == 3:
        return _wilkinson(n)
    if itype == 4:
        return np.zeros(n), np.sqrt(i * (n + 1 - i).astype(float))
    if itype == 5:
        k = np.arange(2, n + 1)
        return np.zeros(n), k / np.sqrt(((2 * k - 1) * (2 * k) + 1).astype(float))
    if itype == 6:
        return np.arange(3, 2 * n + 2, 2, dtype=float), np.arange(2, n + 1, dtype=float)
    if itype == 7:
        return np.zeros(n), np.sqrt(i.astype(float))
    if itype == 8:
        small = np.finfo(float).tiny / ulp
        large = np.finfo(float).max * ulp
        D1, E1 = _wilkinson(n)
        D = np.concatenate([small * D1, D1, large * D1])
        E = np.concatenate([small * E1, [0.0], E1, [0.0], large * E1])
        return D, E
    raise ValueError(itype)


def st_errors(D, E, lam, V):
    """runtest (test/symtridiag.jl:181-218): the scaled residual and orthogonality errors."""
    n = len(D)
    T = np.diag(D) + np.diag(E, 1) + np.diag(E, -1)
    myeps = np.finfo(float).eps
    ntol = n
    resnorm = np.abs(V @ np.diag(lam) @ V.T - T).max()
    Tnorm = max(np.abs(T).sum(axis=0).max(), np.finfo(float).tiny)
    if resnorm < Tnorm:
        d_err = (resnorm / Tnorm) / (myeps * ntol)
    elif Tnorm < 1:
        d_err = (min(resnorm, Tnorm * ntol) / Tnorm) / (myeps * ntol)
    else:
        d_err = min(resnorm / Tnorm, ntol) / (myeps * ntol)
    v_err = np.abs(V @ V.T - np.eye(n)).max() / (myeps * ntol)
    return d_err, v_err


def check_gordschur_real(A, B, vals, select, S2, T2, a, b, Q2, Z2, tol=10):
    """The reference's real checkord criteria (test/gordschur.jl:90-137): quasi-triangular,
    backward stable, orthogonal; and that the leading block holds exactly the selected
    eigenvalues (a complex pair counts as selected when either member is)."""
    n = A.shape[0]
    nA, nB = np.linalg.norm(A), np.linalg.norm(B)
    assert np.linalg.norm(np.tril(S2, -2)) / (n * nA * EPS) < tol
    assert np.linalg.norm(np.tril(T2, -1)) / (n * nA * EPS) < tol
    assert np.linalg.norm(A - Q2 @ S2 @ Z2.T) / (n * nA * EPS) < tol
    assert np.linalg.norm(B - Q2 @ T2 @ Z2.T) / (n * nB * EPS) < tol
    assert np.linalg.norm(np.eye(n) - Z2 @ Z2.T) / (n * EPS) < tol
    assert np.linalg.norm(np.eye(n) - Q2 @ Q2.T) / (n * EPS) < tol
    # the selected set, with pairs (the reference's own list, select[j] || (select[j + 1] &&
    # imag(values[j]) != 0), also admits the second member of an unselected pair followed by a
    # selected eigenvalue, so its matching can pair a leading eigenvalue with a wrong one)
    sel = selected_with_pairs(vals, select)
    k = int(sel.sum())
    got = a[:k] / b[:k]
    want = vals[sel]
    from scipy.optimize import linear_sum_assignment
    C = np.abs(got[:, None] - want[None, :]) / np.maximum(1.0, np.abs(want[None, :]))
    r, c = linear_sum_assignment(C)
    assert C[r, c].max() < 1e-8


def selected_with_pairs(vals, select):
    """select with each complex pair of a real generalized Schur form selected when either
    member is (rordschur.jl:563-583)."""
    n = len(vals)
    sel = np.array(select, dtype=bool).copy()
    j = 0
    while j < n:
        if vals[j].imag != 0 and j < n - 1:
            sel[j] = sel[j + 1] = sel[j] or sel[j + 1]
            j += 2
        else:
            j += 1
    return sel
