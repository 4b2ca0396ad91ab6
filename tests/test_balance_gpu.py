"""GPU tests of balancing (balance!, balance.jl:33-185), the Balancer's action on
eigenvectors (lmul!/ldiv!, balance.jl:189-261) and eigen! with its default
balancing (pirates.jl:63-89).  Balancing moves entries by exact operations (row and
column swaps, power-of-two scalings), so the GPU's balanced matrix, permutation
record, scale factors and ilo/ihi must equal the oracle's exactly."""
import numpy as np
import pytest

from common import EPS, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(4400)
    out = []
    for n in (1, 2, 5, 17, 64, 130):
        A = randn_matrix(rng, n)
        d = 10.0 ** rng.integers(-6, 7, size=n)
        out.append(("graded%d" % n, (A * d[None, :]) / d[:, None]))
    # isolated eigenvalues: rows / columns that permute out
    A = randn_matrix(rng, 12)
    A[8:, :8] = 0.0
    A[10, 8:10] = 0.0
    A[11, 8:11] = 0.0
    A[:, 0] = 0.0
    A[0, 0] = 3.0
    out.append(("isolated", A))
    U = np.triu(randn_matrix(rng, 9))
    out.append(("triangular", U))
    Cz = randn_matrix(rng, 40, cplx=True)
    dz = 2.0 ** rng.integers(-30, 31, size=40)
    out.append(("complex", (Cz * dz[None, :]) / dz[:, None]))
    # the overflow / underflow guards of the scaling loop compare the largest |x| of a
    # row or column (found through |x|^2 for complex entries) with the safe range:
    # magnitudes near 1e+-150 (|x|^2 outside the range) and 1e-165 (|x|^2 underflows)
    Cg = randn_matrix(rng, 24, cplx=True)
    dg = 2.0 ** rng.integers(-20, 21, size=24)
    Cg = (Cg * dg[None, :]) / dg[:, None]
    for tag, mag in (("tiny", 1e-150), ("huge", 1e150), ("subtiny", 1e-165)):
        out.append(("complex_" + tag, Cg * mag))
    return out


@pytest.mark.parametrize("name,A", _cases(), ids=[c[0] for c in _cases()])
@pytest.mark.parametrize("mode", [(True, True), (True, False), (False, True)])
def test_balance_matches_oracle(gs, name, A, mode):
    scale, permute = mode
    Ab, B = gs.balance(A, scale=scale, permute=permute)
    Ao, (ilo, ihi, sp, D, trivial) = po.balance(A, scale=scale, permute=permute)
    assert (B.ilo, B.ihi) == (ilo, ihi)
    np.testing.assert_array_equal(B.D, D)
    n = A.shape[0]
    # the permutation record is defined outside [ilo, ihi]
    for j in list(range(1, ilo)) + list(range(ihi + 1, n + 1)):
        assert B.prow_pcol[j - 1] == sp[j - 1]
    np.testing.assert_array_equal(Ab, Ao)
    assert B.trivial == trivial
    if n > 1:
        w0 = np.sort_complex(np.linalg.eigvals(A))
        w1 = np.sort_complex(np.linalg.eigvals(Ab))
        assert np.max(np.abs(w0 - w1)) <= 1e-8 * max(np.max(np.abs(w0)), 1.0)


@pytest.mark.parametrize("inverse", [False, True])
def test_balancer_apply_matches_oracle(gs, inverse):
    rng = np.random.default_rng(4500)
    for name, A in _cases():
        n = A.shape[0]
        _, B = gs.balance(A)
        _, Bo = po.balance(A)
        V = randn_matrix(rng, n, cplx=True)
        Vg = gs.balancer_ldiv(B, V) if inverse else gs.balancer_lmul(B, V)
        Vo = po.balancer_apply(V, Bo, inverse=inverse)
        np.testing.assert_array_equal(Vg, Vo)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("n", [40, 200])
def test_eigen_with_balancing(gs, cplx, n):
    """eigen(A) with the reference's defaults (permute=true, scale=true) on a badly
    graded matrix: A V = V diag(w) to working accuracy, unit vectors with the
    largest entry real, eigenvalues sorted."""
    rng = np.random.default_rng(4600 + n)
    A0 = randn_matrix(rng, n, cplx)
    d = 10.0 ** rng.integers(-5, 6, size=n)
    A = (A0 * d[None, :]) / d[:, None]
    E = gs.eigen(A)
    V, w = E.vectors, E.values
    assert np.all(np.diff(w.real) >= 0)
    res = np.linalg.norm(A @ V - V @ np.diag(w), axis=0) / (np.linalg.norm(A) * np.linalg.norm(V, axis=0))
    assert np.max(res) <= 100 * n * EPS
    assert np.all(np.abs(np.linalg.norm(V, axis=0) - 1) < 10 * n * EPS)
    for j in range(n):
        assert V[np.argmax(np.abs(V[:, j])), j].imag == 0


def test_eigen_left_vectors_and_condition_numbers(gs):
    """eigen!(A; jvl = true, jce = true) (pirates.jl:91-160): left vectors satisfy
    A^H VL = VL conj(diag(w)) after ldiv! by the Balancer, and rconde equals the oracle's
    condition numbers of the same (balanced) form."""
    from common import rconde as rconde_np
    rng = np.random.default_rng(4800)
    n = 60
    A0 = randn_matrix(rng, n)
    d = 10.0 ** rng.integers(-3, 4, size=n)
    A = (A0 * d[None, :]) / d[:, None]
    E = gs.eigen(A, jvl=True, jce=True)
    w, V, VL, rce = E.values, E.vectors, E.vectorsl, E.rconde
    nA = np.linalg.norm(A)
    assert np.linalg.norm(A @ V - V @ np.diag(w)) / (n * nA) < 1e-12
    assert np.linalg.norm(A.conj().T @ VL - VL @ np.diag(w.conj())) / (n * nA) < 1e-12
    # condition numbers of the balanced form, as the reference computes them
    Ab, _ = po.balance(A)
    T, Z, wo = po.gschur(Ab)
    s_ref = rconde_np(po.eigvecs(T, Z, left=True), po.eigvecs(T, Z))
    # match by eigenvalue (same sort as eigen's)
    order_gpu = np.lexsort((w.imag, w.real))
    order_ref = np.lexsort((wo.imag, wo.real))
    assert np.max(np.abs(rce[order_gpu] - s_ref[order_ref])) < 1e-8
