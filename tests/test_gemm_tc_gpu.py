"""GPU tests of the FP64 product on the BF16 tensor cores (gs_gemm_f64_tc, exact
splitting), the product the mixed-precision refinement forms Z^T A Z and Z^T Z with.

Accuracy contract: per entry, |C - C_exact| / (max_k |op(A)_ik| * max_k |B_kj|) no worse
than an FP64 GEMM's (numpy's, against the same extended-precision product), and below
32 eps absolutely in those units.  Zero rows give zero, Inf/NaN rows give NaN rows."""
import numpy as np
import pytest

from common import EPS

pytestmark = pytest.mark.gpu


def _exact(Aop, B):
    return Aop.astype(np.longdouble) @ B.astype(np.longdouble)


def _rel_err(C, Cex, Aop, B):
    mu = np.abs(Aop).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :]
    mu = np.where(mu == 0, 1.0, mu)
    return float(np.max(np.abs(C.astype(np.longdouble) - Cex) / mu))


@pytest.mark.parametrize("m,p,q", [(1, 1, 1), (5, 7, 3), (128, 128, 64), (130, 20, 70), (300, 200, 500),
                                   (96, 65, 4100)])
@pytest.mark.parametrize("transA", [False, True])
def test_gemm_tc_matches_exact(gs, m, p, q, transA):
    rng = np.random.default_rng(1000 * m + 10 * p + q + (7 if transA else 0))
    Aop = rng.standard_normal((m, q)) * np.exp(rng.uniform(-4, 4, (m, 1)))
    B = rng.standard_normal((q, p)) * np.exp(rng.uniform(-4, 4, (1, p)))
    A = np.asfortranarray(Aop.T) if transA else Aop
    C = gs.gemm_f64_tc(A, B, transA=transA)
    Cex = _exact(Aop, B)
    e_tc = _rel_err(C, Cex, Aop, B)
    e_64 = _rel_err(Aop @ B, Cex, Aop, B)
    assert e_tc <= 32 * EPS, (e_tc, e_64)
    assert e_tc <= 2 * e_64 + 4 * EPS, (e_tc, e_64)


def test_gemm_tc_special_rows(gs):
    rng = np.random.default_rng(77)
    m, p, q = 150, 140, 90
    A = rng.standard_normal((m, q))
    B = rng.standard_normal((q, p))
    A[3, :] = 0.0
    B[:, 5] = 0.0
    A[10, :] *= 1e-200
    A[11, :] *= 1e200
    B[:, 12] *= 1e-150
    A[20, 7] = np.nan
    B[40, 30] = np.inf
    C = gs.gemm_f64_tc(A, B)
    # zero row / column give zeros, except where they meet the non-finite column / row
    # (0 * Inf is NaN, as in an FP64 product)
    assert np.all(np.delete(C[3, :], 30) == 0) and np.all(np.delete(C[:, 5], 20) == 0)
    assert np.isnan(C[3, 30]) and np.isnan(C[20, 5])
    assert np.all(np.isnan(C[20, :])) and np.all(np.isnan(C[:, 30]))
    good_r = np.setdiff1d(np.arange(m), [20])
    good_c = np.setdiff1d(np.arange(p), [30])
    Ag, Bg = A[good_r], B[:, good_c]
    Cg = C[np.ix_(good_r, good_c)]
    assert np.all(np.isfinite(Cg))
    assert _rel_err(Cg, _exact(Ag, Bg), Ag, Bg) <= 32 * EPS


def test_gemm_tc_empty_inner(gs):
    C = gs.gemm_f64_tc(np.zeros((4, 0)), np.zeros((0, 3)))
    assert C.shape == (4, 3) and np.all(C == 0)


def test_gemm_tc_refinement_shapes(gs):
    """The refinement's products at n = 2048: Z^T (A Z) and Z^T Z for an orthogonal Z."""
    rng = np.random.default_rng(2048)
    n = 2048
    Z, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = rng.standard_normal((n, n))
    AZ = gs.gemm_f64_tc(A, Z)
    At = gs.gemm_f64_tc(Z, AZ, transA=True)
    ref = Z.T @ (A @ Z)
    assert np.linalg.norm(At - ref) / np.linalg.norm(ref) <= 4 * np.sqrt(n) * EPS
    G = gs.gemm_f64_tc(Z, Z, transA=True)
    assert np.linalg.norm(G - np.eye(n)) <= np.linalg.norm(Z.T @ Z - np.eye(n)) * 2 + n * EPS
