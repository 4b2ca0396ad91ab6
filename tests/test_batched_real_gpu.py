"""GPU parity tests of the real FP64 Schur kernels against the CPU oracle.

Criteria (the parity bar, restating the reference's schurtest checks):
T upper quasi-triangular with standard-form 2x2 blocks (test/real.jl:3-33),
||A - Z T Z^T||_F / ||A||_F <= 10 n eps, ||Z^T Z - I||_F <= 10 n eps, eigenvalues
consistent with T (test/testfuncs.jl:57-86) and matched to the oracle's within
1e2 n eps ||A||_F / s_i.
"""
import numpy as np
import pytest

from common import EPS, assert_schur_real, eig_tolerances, match_eigenvalues, randn_matrix, godunov
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 4, 5, 7, 8, 16, 31, 32, 33, 47, 64, 65, 80, 96, 97, 111, 127, 128]


@pytest.mark.parametrize("n", SIZES)
def test_single_random(gs, n):
    rng = np.random.default_rng(1000 + n)
    A = randn_matrix(rng, n)
    S = gs.gschur(A)
    assert_schur_real(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "eigenvalue mismatch, worst err/tol = %.3g" % worst


def test_batched_mixed_sizes(gs):
    rng = np.random.default_rng(4)
    ns = list(rng.integers(8, 129, size=200)) + [1, 2, 3, 128, 0]
    mats = [randn_matrix(rng, int(n)) for n in ns]
    Ts, Zs, ws, status = gs.gschur_batched(mats)
    assert np.all(status == 0)
    for A, T, Z, w in zip(mats, Ts, Zs, ws):
        if A.shape[0] == 0:
            continue
        assert_schur_real(A, T, Z, w)
    for idx in range(0, len(mats), 17):
        A = mats[idx]
        if A.shape[0] == 0:
            continue
        w_ref, tol = eig_tolerances(A, po)
        ok, worst = match_eigenvalues(ws[idx], w_ref, tol)
        assert ok, "matrix %d (n=%d): worst err/tol %.3g" % (idx, A.shape[0], worst)


def test_batched_graph_replay_matches(gs):
    rng = np.random.default_rng(5)
    mats = [randn_matrix(rng, int(n)) for n in rng.integers(8, 129, size=64)]
    packed, ns, offs, woffs = gs.pack_batch(mats)
    T1, Z1, w1, s1 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True)
    T2, Z2, w2, s2 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True)
    T3, Z3, w3, s3 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=False)
    # same kernels, same inputs: identical results
    np.testing.assert_array_equal(T1, T2)
    np.testing.assert_array_equal(T1, T3)
    np.testing.assert_array_equal(Z1, Z3)
    np.testing.assert_array_equal(w1, w3)


@pytest.mark.parametrize("n", [4, 32, 100])
def test_orthogonal_normal(gs, n):
    rng = np.random.default_rng(300 + n)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    S = gs.gschur(Q)
    assert_schur_real(Q, S.T, S.Z, S.values)
    assert np.linalg.norm(np.triu(S.T, 2)) / (n * np.linalg.norm(Q) * EPS) < 10


@pytest.mark.parametrize("n", [4, 32, 128])
def test_jordan(gs, n):
    A = np.diag(np.ones(n - 1), 1) + np.eye(n)
    S = gs.gschur(A)
    assert_schur_real(A, S.T, S.Z, S.values, tol=20.0)


@pytest.mark.parametrize("s", [1e-300, 1e-200, 1e200, 1e300])
def test_extreme_scaling(gs, s):
    rng = np.random.default_rng(8)
    n = 24
    A0 = rng.standard_normal((n, n))
    A = s * A0
    S = gs.gschur(A)
    assert np.all(np.tril(S.T, -2) == 0)
    be = np.linalg.norm(A0 - S.Z @ (S.T / s) @ S.Z.T) / np.linalg.norm(A0)
    assert be <= 10 * n * EPS
    assert np.linalg.norm(S.Z.T @ S.Z - np.eye(n)) <= 10 * n * EPS


def test_special_matrices(gs):
    for A in [np.zeros((6, 6)), np.eye(9), np.diag(np.arange(1.0, 11.0)), np.triu(np.ones((12, 12))),
              np.diag(np.ones(15), -1)]:
        S = gs.gschur(A)
        assert_schur_real(A, S.T, S.Z, S.values, tol=20.0)


def test_godunov_double(gs):
    A, vals, econd = godunov()
    S = gs.gschur(A)
    assert_schur_real(A, S.T, S.Z, S.values)
    # In FP64 these eigenvalues (condition ~7e16) are not resolvable; the reference
    # tests them only at 80 bits.  Parity here is the conditioned match to the oracle.
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, worst


def test_wantz_false_and_eigvals(gs):
    rng = np.random.default_rng(13)
    A = rng.standard_normal((40, 40))
    S1 = gs.gschur(A)
    S0 = gs.gschur(A, wantZ=False)
    np.testing.assert_array_equal(S0.T, S1.T)
    w = gs.eigvals(A)
    assert np.all(np.diff(w.real) >= 0)


def test_unconverged_status(gs):
    rng = np.random.default_rng(14)
    A = rng.standard_normal((20, 20))
    with pytest.raises(gs.UnconvergedException):
        gs.gschur(A, maxiter=3)


@pytest.mark.parametrize("bad_n", [129, 300, -3])
def test_device_orders_out_of_range(gs, bad_n):
    """GS_DEVICE batches: orders are read on the device only.  An order outside
    [0, 128] must give that matrix status GS_BADARG (the reference raises
    ArgumentError/DimensionMismatch for bad sizes) and leave it untouched, while the
    other matrices are decomposed as usual."""
    torch = pytest.importorskip("torch")
    from genericschur_gb300 import _capi
    rng = np.random.default_rng(77)
    ns = np.array([20, 128, 7, bad_n, 64, 100], dtype=np.int32)
    room = np.maximum(ns, 0).astype(np.int64) ** 2
    offs = np.concatenate([[0], np.cumsum(room)[:-1]]).astype(np.int64)
    woffs = np.concatenate([[0], np.cumsum(np.maximum(ns, 0))[:-1]]).astype(np.int64)
    packed = rng.standard_normal(int(room.sum()))
    dev = torch.device("cuda", 0)
    ctx = gs.get_context(0)
    stream = torch.cuda.Stream(dev)
    A = torch.from_numpy(packed).to(dev)
    Z = torch.zeros_like(A)
    nw = int(np.maximum(ns, 0).sum())
    wr = torch.zeros(nw, dtype=torch.float64, device=dev)
    wi = torch.zeros(nw, dtype=torch.float64, device=dev)
    st = torch.full((len(ns),), -1, dtype=torch.int32, device=dev)
    dns, doffs, dwoffs = (torch.from_numpy(x).to(dev) for x in (ns, offs, woffs))
    torch.cuda.synchronize()
    ctx.set_stream(stream.cuda_stream)
    try:
        rc = ctx.lib.gs_schur_batched_f64(ctx.handle, len(ns), dns.data_ptr(), doffs.data_ptr(), dwoffs.data_ptr(),
                                          A.data_ptr(), Z.data_ptr(), wr.data_ptr(), wi.data_ptr(), st.data_ptr(),
                                          _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE)
        assert rc == 0
        stream.synchronize()
    finally:
        ctx.set_stream(None)
    status = st.cpu().numpy()
    T = A.cpu().numpy()
    Zh = Z.cpu().numpy()
    w = wr.cpu().numpy() + 1j * wi.cpu().numpy()
    for b, n in enumerate(ns):
        o = int(offs[b])
        if n < 0 or n > 128:
            assert status[b] == _capi.GS_BADARG
            np.testing.assert_array_equal(T[o:o + room[b]], packed[o:o + room[b]])
            continue
        assert status[b] == 0
        A0 = packed[o:o + n * n].reshape(n, n, order="F")
        q = int(woffs[b])
        assert_schur_real(A0, T[o:o + n * n].reshape(n, n, order="F"), Zh[o:o + n * n].reshape(n, n, order="F"),
                          w[q:q + n])


def test_host_buffer_pipeline_matches(gs):
    """Host-buffer calls of 2,048 or more matrices stored in order run as a pipeline
    (runs of matrices whose copies overlap the other runs' kernels).  Each matrix's
    computation does not depend on how the batch is cut, so the results equal those of
    the unpipelined call (the graph-replayed one) bit for bit; a batch stored out of order
    takes the unpipelined path and is correct too."""
    from genericschur_gb300.workloads import batched_real
    packed, ns, offs, woffs = batched_real(3000, seed=9)
    T1, Z1, w1, s1 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs)
    T2, Z2, w2, s2 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True)
    assert np.all(s1 == 0) and np.all(s2 == 0)
    np.testing.assert_array_equal(T1, T2)
    np.testing.assert_array_equal(Z1, Z2)
    np.testing.assert_array_equal(w1, w2)
    # reversed storage order: offsets decrease, so no pipeline
    rev = np.arange(len(ns))[::-1]
    T3, Z3, w3, s3 = gs.gschur_batched(packed=packed, ns=ns[rev].copy(), offs=offs[rev].copy(),
                                       woffs=woffs[rev].copy())
    assert np.all(s3 == 0)
    np.testing.assert_array_equal(T3, T1)
    np.testing.assert_array_equal(w3, w1)
    for b in range(0, len(ns), 97):
        n = int(ns[b])
        o, q = int(offs[b]), int(woffs[b])
        A = packed[o:o + n * n].reshape(n, n, order="F")
        assert_schur_real(A, T1[o:o + n * n].reshape(n, n, order="F"), Z1[o:o + n * n].reshape(n, n, order="F"),
                          w1[q:q + n])
