"""Parity on the benchmark workloads themselves, at their stated sizes and seeds.

Every input below is generated exactly as the benchmark generates it
(genericschur_gb300.workloads), and every result is held to the parity rule of the
Schur tests, which restates the reference's schurtest / checkblocks / checkeigvals
(test/real.jl:3-74, test/complex.jl:1-34, test/testfuncs.jl:57-86):
  * real T upper quasi-triangular with standard-form 2x2 blocks, complex T triangular;
  * ||A - Z T Z^H||_F / ||A||_F <= 10 n eps and ||Z^H Z - I||_F <= 10 n eps;
  * eigenvalues matched one-to-one to the reference eigenvalues within
    1e2 n eps ||A||_F / s_i, s_i the reciprocal condition of eigenvalue i
    (rconde, pirates.jl:107-113).
Reference eigenvalues and s_i come from the CPU oracle (the restatement of gschur!
and of the left/right eigenvector solves) where it finishes in seconds; at n = 1024
and 2048 they come from LAPACK's dgeev left and right eigenvectors (scipy), which is
said in each test.
"""
import numpy as np
import pytest

from common import EPS, assert_schur_cplx, assert_schur_real, eig_tolerances, match_eigenvalues, rconde
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _unpack(packed, ns, offs):
    return [packed[o:o + n * n].reshape((n, n), order="F") for o, n in zip(offs, ns)]


def _sample(count, k, seed):
    return np.sort(np.random.default_rng(seed).choice(count, size=min(k, count), replace=False))


def test_batched_real_workload_20000(gs):
    """The headline batch: 20,000 real N(0,1) matrices, orders ~ U{8..128}, seed 4, in
    one call.  Status and the Schur-form properties on all 20,000; eigenvalues matched
    to the oracle's on a seeded sample of 1,000 matrices."""
    from genericschur_gb300.workloads import batched_real
    packed, ns, offs, woffs = batched_real(20000, seed=4)
    T, Z, w, st = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True)
    assert np.all(st == 0), np.unique(st, return_counts=True)
    As, Ts, Zs = _unpack(packed, ns, offs), _unpack(T, ns, offs), _unpack(Z, ns, offs)
    worst_be = worst_oe = 0.0
    for b in range(len(ns)):
        n = int(ns[b])
        be, oe = assert_schur_real(As[b], Ts[b], Zs[b], w[woffs[b]:woffs[b] + n])
        worst_be = max(worst_be, be / (n * EPS))
        worst_oe = max(worst_oe, oe / (n * EPS))
    assert worst_be <= 10 and worst_oe <= 10
    for b in _sample(len(ns), 1000, 40):
        n = int(ns[b])
        w_ref, tol = eig_tolerances(As[b], po)
        ok, worst = match_eigenvalues(w[woffs[b]:woffs[b] + n], w_ref, tol)
        assert ok, "matrix %d (n=%d): worst err/tol %.3g" % (b, n, worst)


def test_batched_real_workload_20000_mixed(gs):
    """The headline batch through the mixed form (GS_MIXED: FP32 Schur sweeps, FP64
    Newton refinement, FP64 recomputation where the refinement stalls), in one call:
    status and the Schur-form properties on all 20,000, backward and orthogonality errors
    within 10 n eps; eigenvalues matched to the oracle's on a seeded sample of 1,000."""
    from genericschur_gb300.workloads import batched_real
    packed, ns, offs, woffs = batched_real(20000, seed=4)
    T, Z, w, st = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True, mixed=True)
    assert np.all(st == 0), np.unique(st, return_counts=True)
    As, Ts, Zs = _unpack(packed, ns, offs), _unpack(T, ns, offs), _unpack(Z, ns, offs)
    worst_be = worst_oe = 0.0
    for b in range(len(ns)):
        n = int(ns[b])
        be, oe = assert_schur_real(As[b], Ts[b], Zs[b], w[woffs[b]:woffs[b] + n])
        worst_be = max(worst_be, be / (n * EPS))
        worst_oe = max(worst_oe, oe / (n * EPS))
    assert worst_be <= 10 and worst_oe <= 10
    for b in _sample(len(ns), 1000, 41):
        n = int(ns[b])
        w_ref, tol = eig_tolerances(As[b], po)
        ok, worst = match_eigenvalues(w[woffs[b]:woffs[b] + n], w_ref, tol)
        assert ok, "matrix %d (n=%d): worst err/tol %.3g" % (b, n, worst)


def test_batched_complex_workload_5000(gs):
    """The complex batch: 5,000 ComplexF64 matrices, orders ~ U{8..128}, re/im iid
    N(0, 1/2), seed 5.  Status and properties on all; eigenvalues matched to the
    oracle's on a seeded sample of 1,000."""
    from genericschur_gb300.workloads import batched_cplx
    packed, ns, offs, woffs = batched_cplx(5000, seed=5)
    T, Z, w, st = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True)
    assert np.all(st == 0), np.unique(st, return_counts=True)
    As, Ts, Zs = _unpack(packed, ns, offs), _unpack(T, ns, offs), _unpack(Z, ns, offs)
    for b in range(len(ns)):
        n = int(ns[b])
        assert_schur_cplx(As[b], Ts[b], Zs[b], w[woffs[b]:woffs[b] + n])
    for b in _sample(len(ns), 1000, 50):
        n = int(ns[b])
        w_ref, tol = eig_tolerances(As[b], po)
        ok, worst = match_eigenvalues(w[woffs[b]:woffs[b] + n], w_ref, tol)
        assert ok, "matrix %d (n=%d): worst err/tol %.3g" % (b, n, worst)


def _lapack_tolerances(A):
    """Reference eigenvalues and the parity tolerance 1e2 n eps ||A||_F / s_i from
    LAPACK dgeev's left and right eigenvectors (the oracle's n^3 single-core solves
    take minutes at these orders)."""
    import scipy.linalg
    n = A.shape[0]
    w, VL, VR = scipy.linalg.eig(A, left=True, right=True)
    s = np.maximum(rconde(VL, VR), 1e-300)
    return w, 1e2 * n * EPS * np.linalg.norm(A) / s


@pytest.mark.parametrize("n", [1024, 2048])
@pytest.mark.parametrize("form", ["fp64", "mixed"])
def test_large_real_workload(gs, n, form):
    """The large real workload: one n x n matrix with iid N(0,1) entries (seed 2 for
    n = 1024, seed 3 for n = 2048), by the plain FP64 path and by the FP32 + FP64
    refinement path; eigenvalues matched to LAPACK's within 1e2 n eps ||A||_F / s_i
    (s_i from LAPACK's left/right eigenvectors)."""
    from genericschur_gb300.workloads import large_real
    A = large_real(n)
    if form == "fp64":
        S = gs.gschur(A)
    else:
        S, info = gs.gschur_mixed(A, return_info=True)
        assert info["iterations"] >= 1  # refined, not recomputed in FP64
    assert_schur_real(A, S.T, S.Z, S.values)
    w_ref, tol = _lapack_tolerances(A)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


def test_complex256_workload(gs):
    """The plain CPU-runnable workload as configured: one 256 x 256 ComplexF64 matrix,
    real and imaginary parts iid N(0, 1/2), seed 0, no balancing, Z accumulated.
    Schur properties, eigenvalues matched to the oracle's FP64 run (tolerance from the
    oracle's eigenvectors) and to the oracle's 256-bit (BigFloat-precision) run (committed
    fixture)."""
    import os
    n = 256
    rng = np.random.default_rng(0)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2)
    G = np.load(os.path.join(os.path.dirname(__file__), "golden", "mp256_n256.npz"))
    np.testing.assert_array_equal(A, G["A_c256"])
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "vs FP64 oracle: worst err/tol %.3g" % worst
    ok, worst = match_eigenvalues(S.values, G["w_c256"], tol)
    assert ok, "vs 256-bit oracle: worst err/tol %.3g" % worst


def test_differentiation_workload_plain_central_differences(gs):
    """The differentiation workload with the finite-difference check as configured:
    plain central differences with h = 1e-6 on 50 random directions, 1e-6 relative.
    The directions have the law of the inputs (complex N(0, 1/2) / sqrt(64) entries), and
    each matrix's loss difference L_b(A_b + h E_b) - L_b(A_b - h E_b) is formed before the
    batch sum, so the rounding of the 4,096-term total does not enter the difference."""
    from genericschur_gb300.workloads import adjoint_batch
    n = 64
    tau = 0.1
    packed, ns, offs, woffs = adjoint_batch(4096, n, seed=7)

    def losses(p):
        _, _, w, st = gs.gschur_batched(packed=p, ns=ns, offs=offs, woffs=woffs)
        assert np.all(st == 0)
        x = w.reshape(-1, n).real / tau
        m = x.max(axis=1)
        return m + np.log(np.exp(x - m[:, None]).sum(axis=1))

    T, Z, w, st = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs)
    x = w.reshape(-1, n).real / tau
    e = np.exp(x - x.max(axis=1, keepdims=True))
    gbar = (e / e.sum(axis=1, keepdims=True) / tau).astype(np.complex128).ravel()
    G = gs.eig_adjoint_batched(T, Z, ns, offs, woffs, gbar)
    rng = np.random.default_rng(71)
    h = 1e-6
    worst = 0.0
    for _ in range(50):
        E = (rng.standard_normal(len(packed)) + 1j * rng.standard_normal(len(packed))) / np.sqrt(2.0) / np.sqrt(n)
        fd = float(np.sum(losses(packed + h * E) - losses(packed - h * E)) / (2 * h))
        an = float(np.real(np.vdot(G, E)))
        worst = max(worst, abs(fd - an) / abs(an))
    assert worst <= 1e-6, worst
