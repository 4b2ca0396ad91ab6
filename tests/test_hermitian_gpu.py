"""GPU tests of the Hermitian / real symmetric path: geigen! / geigvals! of Hermitian(A,
uplo) (GenericSchur.jl:126-146), hessenberg!(Hermitian) (hessenberg.jl:26-96) and the
tridiagonal QL/QR iteration (symtridiag.jl:79-368), restating the reference's own checks:
  * test/symtridiag.jl:157-224: the LAPACK-style classes (eigenvalue distributions
    1-9 through Q' diag(l) Q; zero, identity, (1,2,1), Wilkinson, Clement, Legendre,
    Laguerre, Hermite and the glued small/normal/large scaling case), with
    d_err = max|V diag(l) V' - T| / (|T|_1 eps n) < 50 and v_err = max|V V' - I| / (eps n) < 50;
  * test/complex.jl:63-113 (hesstest on Hermitian :U and :L, also scaled by 100 floatmin):
    |A - Q H Q'| / (n |A| eps) < 10, |I - Q Q'| / (n eps) < 10, real subdiagonal;
and comparing with the oracle's restatement: eigenvalues to 10 n eps |A|_2 (Weyl),
eigenvectors of separated eigenvalues up to phase, the tridiagonal factors elementwise."""
import numpy as np
import pytest

from common import EPS, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _herm(rng, n, cplx):
    A = randn_matrix(rng, n, cplx)
    return (A + A.conj().T) / 2


def _check_eigen(A, w, V, tol=10.0):
    n = A.shape[0]
    nA = max(np.linalg.norm(A, 2), np.finfo(float).tiny)
    assert np.all(np.diff(w) >= 0)
    assert np.linalg.norm(A @ V - V * w[None, :]) / (n * nA * EPS) < tol
    assert np.linalg.norm(V.conj().T @ V - np.eye(n)) / (n * EPS) < tol


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("n", [1, 2, 3, 10, 64, 129, 300])
def test_heev_matches_oracle(gs, cplx, uplo, n):
    rng = np.random.default_rng(7000 + n + 7 * cplx)
    A = _herm(rng, n, cplx)
    # only the `uplo` triangle may be read: spoil the other one
    Ain = A.copy()
    if n > 1:
        junk = np.triu(np.full((n, n), np.nan), 1)
        Ain = Ain + (junk if uplo == "L" else junk.T)
    E = gs.eigen(gs.Hermitian(Ain, uplo))
    _check_eigen(A, E.values, E.vectors)
    wo, Vo, st = po.heev(A, uplo)
    assert st == 0
    nA = max(np.linalg.norm(A, 2), 1e-300)
    assert np.max(np.abs(E.values - wo)) <= 10 * n * EPS * nA
    wv = gs.eigvals(gs.Hermitian(Ain, uplo))
    assert np.max(np.abs(wv - wo)) <= 10 * n * EPS * nA
    # vectors of well-separated eigenvalues agree up to a phase
    gaps = np.full(n, np.inf)
    if n > 1:
        dw = np.diff(wo)
        gaps[:-1] = np.minimum(gaps[:-1], dw)
        gaps[1:] = np.minimum(gaps[1:], dw)
    for j in range(n):
        if gaps[j] > 1e-3 * nA:
            c = abs(np.vdot(Vo[:, j], E.vectors[:, j]))
            assert abs(1 - c) < 1e-8 * max(1.0, nA / gaps[j]) ** 2


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("uplo", ["U", "L"])
def test_hetrd_matches_oracle(gs, cplx, uplo):
    """hessenberg!(Hermitian(A, uplo)): d, e, tau and the stored reflectors equal the
    oracle's (same algorithm; summation order only) and Q H Q' = A (test/complex.jl:63-79)."""
    rng = np.random.default_rng(7100 + cplx)
    n = 45
    A = _herm(rng, n, cplx)
    H = gs.hessenberg_hermitian(gs.Hermitian(A, uplo))
    d, e, tau, F = po.hetrd(A, uplo)
    nA = np.linalg.norm(A)
    # the upper form runs the lower one on the index-reversed matrix: the reflector
    # tails are summed in the opposite order, and tau = (beta - alpha) / beta amplifies
    # that by |alpha| / |beta - alpha|
    tol = 1e3 * EPS * nA
    assert np.max(np.abs(H.dv - d)) < tol and np.max(np.abs(H.ev - e)) < tol
    assert np.max(np.abs(H.tau - tau)) < 1e-10
    tri = np.tril(np.ones((n, n), bool)) if uplo == "L" else np.triu(np.ones((n, n), bool))
    assert np.max(np.abs(H.factors[tri] - F[tri])) < 1e-10 * nA
    assert np.all(np.isreal(H.ev))


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("scale", [1.0, 100 * np.finfo(float).tiny])
def test_hermitian_hesstest(gs, cplx, uplo, scale):
    """test/complex.jl:99-113: rand(T, 32, 32) wrapped Hermitian, also scaled by 100
    floatmin; the eigen decomposition (Q from the tridiagonalization times the rotations)
    reproduces A to 10 n eps."""
    rng = np.random.default_rng(7200 + cplx)
    n = 32
    R = rng.random((n, n)) + (1j * rng.random((n, n)) if cplx else 0)
    A = scale * R
    Ah = np.tril(A) + np.tril(A, -1).conj().T if uplo == "L" else np.triu(A) + np.triu(A, 1).conj().T
    Ah = Ah - 1j * np.diag(np.diag(Ah).imag) if cplx else Ah
    E = gs.eigen(gs.Hermitian(A, uplo))
    V, w = E.vectors, E.values
    # numpy's norms square the entries: measure in units of `scale`
    Ah, w = Ah / scale, w / scale
    nA = np.linalg.norm(Ah)
    assert np.linalg.norm(Ah - (V * w[None, :]) @ V.conj().T) / (n * nA * EPS) < 10
    assert np.linalg.norm(np.eye(n) - V @ V.conj().T) / (n * EPS) < 10


def _class1(n, itype, rng):
    ulp = EPS
    kpar = 1 / ulp
    lam = np.zeros(n)
    if itype == 1:
        lam[0] = 1
        lam[1:] = 1 / np.arange(2, n + 1)
    elif itype == 2:
        lam[:] = 1
        lam[-1] = 1 / n
    elif itype == 3:
        lam = 1 / kpar ** (np.arange(n) / (n - 1))
    elif itype == 4:
        lam = 1 - (np.arange(n) / (n - 1)) * (1 - 1 / kpar)
    elif itype == 5:
        lam = np.exp(-np.log(n) * rng.random(n))
    elif itype == 6:
        lam = rng.standard_normal(n)
    elif itype == 7:
        lam[:n - 1] = np.arange(1, n) * ulp
        lam[-1] = 1
    elif itype == 8:
        lam[0] = ulp
        lam[1:n - 1] = 1 + np.sqrt(ulp) * np.arange(2, n)
        lam[-1] = 2
    elif itype == 9:
        lam = 1 + 100 * ulp * np.arange(n)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = Q.T @ np.diag(lam) @ Q
    d, e, _, _ = po.hetrd((A + A.T) / 2, "L")
    return d, e


def _wilkinson(n):
    if n % 2:
        nh = (n - 1) // 2
        D = np.concatenate([np.arange(nh, 0, -1), [0], np.arange(1, nh + 1)]).astype(float)
    else:
        D = np.abs(np.arange(-(n - 1), n, 2) / 2.0)
    return D, np.ones(n - 1)


def _class2(n, itype):
    if itype == 0:
        return np.zeros(n), np.zeros(n - 1)
    if itype == 1:
        return np.ones(n), np.zeros(n - 1)
    if itype == 2:
        return np.full(n, 2.0), np.ones(n - 1)
    if itype == 3:
        return _wilkinson(n)
    if itype == 4:
        return np.zeros(n), np.sqrt(np.array([i * (n + 1 - i) for i in range(1, n)], float))
    if itype == 5:
        return np.zeros(n), np.array([i / np.sqrt((2 * i - 1) * (2 * i) + 1) for i in range(2, n + 1)])
    if itype == 6:
        return np.arange(3, 2 * n + 2, 2, dtype=float), np.arange(2, n + 1, dtype=float)
    if itype == 7:
        return np.zeros(n), np.sqrt(np.arange(1, n, dtype=float))
    if itype == 8:
        small = np.finfo(float).tiny / EPS
        large = np.finfo(float).max * EPS
        D1, E1 = _wilkinson(n)
        D = np.concatenate([small * D1, D1, large * D1])
        E = np.concatenate([small * E1, [0.0], E1, [0.0], large * E1])
        return D, E
    raise ValueError(itype)


def _runtest(D, E, lam, V):
    """runtest (test/symtridiag.jl:190-218)."""
    n = len(D)
    T = np.diag(D) + np.diag(E, 1) + np.diag(E, -1)
    res = np.max(np.abs((V * lam[None, :]) @ V.T - T))
    Tn = max(np.max(np.sum(np.abs(T), axis=0)), np.finfo(float).tiny)
    if res < Tn:
        derr = (res / Tn) / (EPS * n)
    elif Tn < 1:
        derr = (min(res, Tn * n) / Tn) / (EPS * n)
    else:
        derr = min(res / Tn, n) / (EPS * n)
    verr = np.max(np.abs(V @ V.T - np.eye(n))) / (EPS * n)
    return derr, verr


@pytest.mark.parametrize("case", [("1", t) for t in range(1, 10)] + [("2", t) for t in range(0, 9)],
                         ids=lambda c: "class%s-type%d" % c)
def test_symtridiag_classes(gs, case):
    """test/symtridiag.jl:157-188, n = 32, QRIteration, threshold 50."""
    cls, itype = case
    rng = np.random.default_rng(7300 + itype)
    n = 32
    D, E = _class1(n, itype, rng) if cls == "1" else _class2(n, itype)
    Eg = gs.geigen(gs.SymTridiagonal(D.copy(), E.copy()))
    derr, verr = _runtest(D, E, Eg.values, Eg.vectors)
    assert derr < 50 and verr < 50, (derr, verr)
    # the same iteration in the oracle: eigenvalues agree (sorted)
    wo, Zo, st = po.steqr(D.copy(), E.copy())
    assert st == 0
    scale = max(np.max(np.abs(D)), np.max(np.abs(E)) if len(E) else 0.0, np.finfo(float).tiny)
    assert np.max(np.abs(np.sort(wo) - Eg.values)) <= 50 * len(D) * EPS * scale
    wv = gs.eigvals(gs.SymTridiagonal(D.copy(), E.copy()))
    assert np.max(np.abs(wv - Eg.values)) <= 50 * len(D) * EPS * scale


def test_symtridiag_unsorted_matches_oracle(gs):
    """_gschur!(SymTridiagonal, QRIteration, Z) runs the reference's sweeps in order: the
    unsorted eigenvalues and the accumulated rotations match the oracle's run."""
    rng = np.random.default_rng(7400)
    n = 200
    D, E = rng.standard_normal(n), rng.standard_normal(n - 1)
    d, e, Z = gs.gschur_symtridiag(gs.SymTridiagonal(D, E), np.eye(n))
    do, Zo, st = po.steqr(D.copy(), E.copy())
    assert st == 0
    assert np.max(np.abs(d - do)) < 1e-12 * np.max(np.abs(do))
    s = np.sign(np.sum(Z * Zo, axis=0))
    assert np.max(np.abs(Z - Zo * s[None, :])) < 1e-9
    dv = gs.gschur_symtridiag(gs.SymTridiagonal(D, E))[0]
    assert np.max(np.abs(np.sort(dv) - np.sort(do))) < 1e-12 * np.max(np.abs(do))


def test_hermitian_large(gs):
    """n = 1000 complex: the GPU-wide tridiagonalization and the cooperative sweep kernel
    (many blocks applying rotations) at size."""
    rng = np.random.default_rng(7500)
    n = 1000
    A = _herm(rng, n, True)
    E = gs.eigen(gs.Hermitian(A, "L"))
    _check_eigen(A, E.values, E.vectors)
    w = np.linalg.eigvalsh(A)
    assert np.max(np.abs(E.values - w)) <= 10 * n * EPS * np.linalg.norm(A, 2)


def test_hermitian_edges(gs):
    for A in (np.zeros((5, 5)), np.eye(6), np.diag([3.0, -1.0, 2.0, 2.0])):
        E = gs.eigen(gs.Hermitian(A))
        assert np.allclose(E.values, np.sort(np.diag(A)))
        _check_eigen(A, E.values, E.vectors)
    w = gs.eigvals(gs.Hermitian(np.zeros((0, 0))))
    assert len(w) == 0
