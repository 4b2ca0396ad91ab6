"""GPU tests of the divide-and-conquer eigensolver (src/symtri_dc.jl, _gschur!(A::
SymTridiagonal, DivideAndConquer(), Z)) and of geigen!(Hermitian(A), DivideAndConquer()).

* The reference's SymTridiagonal batch (test/symtridiag.jl:158-225) with DivideAndConquer():
  both matrix classes, the residual and orthogonality errors below 50 (scaled by n eps); the
  reference runs it at n = 32 (one merge); larger orders build deeper trees and reach the
  tensor-core GEMM of the large merges.
* Against the oracle's restatement on the same tridiagonal: the same eigenvalues (to
  rounding: the reference's BLAS products are GEMMs here) and the same eigenvectors up to
  sign where the eigenvalues are separated.
* The Hermitian driver with alg = DivideAndConquer, real and complex: residual,
  orthogonality and eigenvalues against LAPACK (numpy eigh).
* Deflation-heavy matrices (repeated and glued spectra), the split into independent blocks,
  and the orders around the 25 x 25 leaf size."""
import numpy as np
import pytest

from common import EPS, st_errors, st_testmat1, st_testmat2
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

DC = "DivideAndConquer"


def _tri(D, E):
    return np.diag(D) + np.diag(E, 1) + np.diag(E, -1)


@pytest.mark.parametrize("n", [32, 100, 257, 700])
def test_stedc_batch(gs, n):
    rng = np.random.default_rng(3100 + n)
    cases = [st_testmat1(n, it, rng) for it in range(1, 10)] + [st_testmat2(n, it) for it in range(1, 9)]
    for c, (D, E) in enumerate(cases):
        Eg = gs.geigen(gs.SymTridiagonal(D.copy(), E.copy()), alg=DC)
        de, ve = st_errors(D, E, Eg.values, Eg.vectors)
        assert de < 50 and ve < 50, (c, de, ve)
        assert np.all(np.diff(Eg.values) >= 0)


@pytest.mark.parametrize("n", [26, 51, 300, 1000, 2048])
def test_stedc_matches_oracle(gs, n):
    rng = np.random.default_rng(3200 + n)
    D, E = rng.standard_normal(n), rng.standard_normal(n - 1)
    d, _, Z = gs.gschur_symtridiag(gs.SymTridiagonal(D.copy(), E.copy()), np.eye(n), alg=DC)
    do, Zo, st = po.stedc(D, E)
    assert st == 0
    T = _tri(D, E)
    nT = np.abs(T).max()
    # the same eigenvalues
    assert np.abs(np.sort(d) - np.sort(do)).max() <= 20 * n * EPS * nT
    assert np.abs(np.sort(d) - np.linalg.eigvalsh(T)).max() <= 20 * n * EPS * nT
    # residual and orthogonality of the unsorted output (the algorithm's order)
    assert np.abs(T @ Z - Z * d).max() <= 20 * n * EPS * nT
    assert np.abs(Z.T @ Z - np.eye(n)).max() <= 20 * n * EPS
    # eigenvectors against the oracle, up to sign, where the eigenvalue is separated
    pg, po_ = np.argsort(d, kind="stable"), np.argsort(do, kind="stable")
    ds = np.sort(do)
    gap = np.minimum(np.r_[np.inf, np.diff(ds)], np.r_[np.diff(ds), np.inf])
    for j in range(n):
        if gap[j] < 1e-6 * nT:
            continue
        a, b = Z[:, pg[j]], Zo[:, po_[j]]
        err = min(np.abs(a - b).max(), np.abs(a + b).max())
        assert err <= 100 * n * EPS * nT / gap[j], (j, err, gap[j])


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("n", [1, 7, 25, 26, 40, 300, 1000])
def test_geigen_hermitian_dc(gs, n, cplx):
    rng = np.random.default_rng(3300 + n + cplx)
    A = rng.standard_normal((n, n)) + (1j * rng.standard_normal((n, n)) if cplx else 0)
    A = (A + A.conj().T) / 2
    for uplo in ("L", "U"):
        E = gs.geigen(gs.Hermitian(A, uplo), alg=DC)
        V, w = E.vectors, E.values
        nA = np.abs(A).max()
        assert np.abs(A @ V - V * w).max() <= 30 * n * EPS * nA * np.sqrt(n)
        assert np.abs(V.conj().T @ V - np.eye(n)).max() <= 30 * n * EPS
        assert np.abs(w - np.linalg.eigvalsh(A)).max() <= 30 * n * EPS * nA
        wq = gs.geigvals(gs.Hermitian(A, uplo), alg=DC)
        assert np.abs(wq - w).max() <= 30 * n * EPS * nA


@pytest.mark.parametrize("kind", ["identity", "repeated", "wilkinson", "glued", "split"])
def test_stedc_deflation(gs, kind):
    """Spectra that deflate most of each merge: the identity (every z deflates), a matrix
    with n - 1 equal eigenvalues, Wilkinson's close pairs, three Wilkinson blocks glued at
    1e-300 / 1 / 1e300 scales, and a tridiagonal split by zero couplings into blocks below
    and above the leaf size."""
    rng = np.random.default_rng(3400)
    if kind == "identity":
        D, E = np.ones(300), np.zeros(299)
    elif kind == "repeated":
        D, E = st_testmat1(400, 2, rng)
    elif kind == "wilkinson":
        D, E = st_testmat2(401, 3)
    elif kind == "glued":
        D, E = st_testmat2(120, 8)
    else:
        D, E = rng.standard_normal(500), rng.standard_normal(499)
        for c in (10, 30, 31, 200, 460):
            E[c] = 0.0
    Eg = gs.geigen(gs.SymTridiagonal(D.copy(), E.copy()), alg=DC)
    de, ve = st_errors(D, E, Eg.values, Eg.vectors)
    assert de < 50 and ve < 50, (de, ve)
    do, Zo, st = po.stedc(D, E)
    assert st == 0
    T = _tri(D, E)
    assert np.abs(Eg.values - np.sort(do)).max() <= 20 * len(D) * EPS * np.abs(T).max()


@pytest.mark.parametrize("n", [1, 2, 3, 24, 25, 26, 27, 50, 51])
def test_stedc_small_orders(gs, n):
    rng = np.random.default_rng(3500 + n)
    D, E = rng.standard_normal(n), rng.standard_normal(max(n - 1, 0))
    Eg = gs.geigen(gs.SymTridiagonal(D.copy(), E.copy()), alg=DC)
    if n == 1:
        assert Eg.values[0] == D[0] and Eg.vectors[0, 0] == 1.0
        return
    de, ve = st_errors(D, E, Eg.values, Eg.vectors)
    assert de < 50 and ve < 50
    w = gs.geigvals(gs.SymTridiagonal(D.copy(), E.copy()), alg=DC)
    assert np.abs(w - Eg.values).max() <= 20 * n * EPS * np.abs(_tri(D, E)).max()


def test_stedc_timing(gs):
    """A random 4096 x 4096 tridiagonal with eigenvectors: the divide-and-conquer and QR
    times on the GPU, printed; both results checked."""
    n = 4096
    rng = np.random.default_rng(3600)
    D, E = rng.standard_normal(n), rng.standard_normal(n - 1)
    ctx = gs.get_context()
    times = {}
    for alg in ("QRIteration", DC):
        Z = np.eye(n)
        gs.gschur_symtridiag(gs.SymTridiagonal(D.copy(), E.copy()), Z, alg=alg)
        d, _, Z = gs.gschur_symtridiag(gs.SymTridiagonal(D.copy(), E.copy()), np.eye(n), alg=alg)
        times[alg] = ctx.last_kernel_ms()
        T = _tri(D, E)
        assert np.abs(np.sort(d) - np.linalg.eigvalsh(T)).max() <= 20 * n * EPS * np.abs(T).max()
        assert np.abs(Z.T @ Z - np.eye(n)).max() <= 20 * n * EPS
    print("n=%d tridiagonal eigenvectors: QR %.1f ms, divide and conquer %.1f ms" % (n, times["QRIteration"], times[DC]))


def test_eigen_alg_keyword(gs):
    """eigen!/eigvals!(::Hermitian; alg) and (::SymTridiagonal; alg) (pirates.jl:162-197)
    reach divide and conquer; the default stays QRIteration."""
    rng = np.random.default_rng(3700)
    n = 60
    A = rng.standard_normal((n, n))
    A = (A + A.T) / 2
    ref = np.linalg.eigvalsh(A)
    for alg in (None, DC):
        E = gs.eigen(gs.Hermitian(A, "L"), alg=alg)
        assert np.abs(E.values - ref).max() <= 30 * n * EPS * np.abs(A).max()
        assert np.abs(gs.eigvals(gs.Hermitian(A, "U"), alg=alg) - ref).max() <= 30 * n * EPS * np.abs(A).max()
    D, E2 = rng.standard_normal(n), rng.standard_normal(n - 1)
    w = gs.eigvals(gs.SymTridiagonal(D.copy(), E2.copy()), alg=DC)
    assert np.abs(w - np.linalg.eigvalsh(_tri(D, E2))).max() <= 20 * n * EPS * np.abs(_tri(D, E2)).max()
