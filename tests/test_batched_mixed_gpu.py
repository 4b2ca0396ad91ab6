"""GPU parity tests of the mixed-precision batched real Schur form (GS_MIXED):
FP32 Schur pairs refined to FP64 by Newton steps, FP64 recomputation where the
refinement cannot finish.

The bar is the FP64 path's: T upper quasi-triangular with standard-form 2x2 blocks
(test/real.jl:3-33), ||A - Z T Z^T||_F / ||A||_F <= 10 n eps, ||Z^T Z - I||_F <= 10 n eps,
eigenvalues consistent with T (test/testfuncs.jl:57-86) and matched to the oracle's
within 1e2 n eps ||A||_F / s_i.
"""
import numpy as np
import pytest

from common import EPS, assert_schur_real, backward_error, eig_tolerances, match_eigenvalues, orth_error, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _unpack(packed, ns, offs):
    return [packed[o:o + n * n].reshape((n, n), order="F") for o, n in zip(offs, ns)]


def test_mixed_sizes(gs):
    rng = np.random.default_rng(4)
    ns = list(rng.integers(8, 129, size=200)) + [1, 2, 3, 128, 0, 16, 17, 33, 64, 65, 96, 97]
    mats = [randn_matrix(rng, int(n)) for n in ns]
    Ts, Zs, ws, status = gs.gschur_batched(mats, mixed=True)
    assert np.all(status == 0)
    for A, T, Z, w in zip(mats, Ts, Zs, ws):
        if A.shape[0] == 0:
            continue
        assert_schur_real(A, T, Z, w)
    for idx in range(0, len(mats), 13):
        A = mats[idx]
        if A.shape[0] == 0:
            continue
        w_ref, tol = eig_tolerances(A, po)
        ok, worst = match_eigenvalues(ws[idx], w_ref, tol)
        assert ok, "matrix %d (n=%d): worst err/tol %.3g" % (idx, A.shape[0], worst)


def test_mixed_backward_error_like_fp64(gs):
    """Same inputs through both forms: the mixed results' backward and orthogonality
    errors stay within a small factor of the FP64 path's (the spec comparison is
    at equal backward error)."""
    rng = np.random.default_rng(41)
    mats = [randn_matrix(rng, int(n)) for n in rng.integers(64, 129, size=64)]
    T1, Z1, w1, s1 = gs.gschur_batched(mats)
    T2, Z2, w2, s2 = gs.gschur_batched(mats, mixed=True)
    assert np.all(s1 == 0) and np.all(s2 == 0)
    be1 = np.array([backward_error(A, T, Z) / (A.shape[0] * EPS) for A, T, Z in zip(mats, T1, Z1)])
    be2 = np.array([backward_error(A, T, Z) / (A.shape[0] * EPS) for A, T, Z in zip(mats, T2, Z2)])
    oe2 = np.array([orth_error(Z) / (Z.shape[0] * EPS) for Z in Z2])
    assert be2.max() <= 10 and oe2.max() <= 10
    assert np.median(be2) <= 4 * max(np.median(be1), 0.01), (np.median(be1), np.median(be2))


def _hard_cases(rng):
    out = []
    for n in (4, 32, 100):
        J = np.diag(np.ones(n - 1), 1) + np.eye(n)
        out.append(J)  # Jordan block: defective, already triangular
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        out.append(Q @ J @ Q.T)  # the same, hidden by an orthogonal similarity
        out.append(Q)  # all |lambda| = 1
        d = np.repeat(rng.standard_normal((n + 2) // 3), 3)[:n]
        out.append(Q @ np.diag(d) @ Q.T)  # triple eigenvalues, normal
        out.append(np.zeros((n, n)))
        out.append(np.eye(n))
    for s in (1e-300, 1e-200, 1e200, 1e300):
        out.append(randn_matrix(rng, 50) * s)  # checked at unit scale (see _check)
    A = randn_matrix(rng, 60)
    A[:, 30:] = 0.0  # rank deficient, many zero eigenvalues
    out.append(A)
    comp = np.zeros((40, 40))  # companion matrix of z^40 - 1 (roots of unity)
    comp[1:, :-1] = np.eye(39)
    comp[0, -1] = 1.0
    out.append(comp)
    return out


def _check(A, T, Z, w):
    """The parity properties; at extreme scales (|A| ~ 1e+-200..300) the norms are taken
    at unit scale and, as in the FP64 path's extreme-scaling test, the eigenvalue/T
    consistency check is left out (scaled back to 1e-300, small entries of T are
    subnormal, so sqrt|b| sqrt|c| and the imaginary parts round differently)."""
    m = np.abs(A).max()
    if m > 0 and (m > 1e100 or m < 1e-100):
        n = A.shape[0]
        A1, T1 = A / m, T / m
        assert np.all(np.tril(T, -2) == 0)
        assert np.linalg.norm(A1 - Z @ T1 @ Z.T) / np.linalg.norm(A1) <= 20 * n * EPS
        assert np.linalg.norm(Z.T @ Z - np.eye(n)) <= 20 * n * EPS
        return
    assert_schur_real(A, T, Z, w, tol=20.0)


def test_mixed_hard_cases_fall_back(gs):
    """Inputs whose eigenvalues FP32 cannot separate (defective, repeated, clustered) or
    whose scale leaves FP32's range: every matrix still meets the FP64 bar, through the
    refinement or through the FP64 recomputation."""
    rng = np.random.default_rng(9)
    mats = _hard_cases(rng)
    Ts, Zs, ws, status = gs.gschur_batched(mats, mixed=True)
    assert np.all(status == 0)
    for A, T, Z, w in zip(mats, Ts, Zs, ws):
        _check(A, T, Z, w)


def test_mixed_no_fallback_reports(gs):
    """fallback=False: matrices the refinement cannot finish come back unconverged
    (and untouched); every matrix reported converged meets the bar."""
    rng = np.random.default_rng(9)
    mats = _hard_cases(rng) + [randn_matrix(rng, int(n)) for n in (20, 80, 128)]
    packed, ns, offs, woffs = gs.pack_batch(mats)
    T, Z, w, st = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, mixed=True, fallback=False,
                                    raise_on_failure=False)
    assert set(np.unique(st)) <= {0, 1}
    assert np.all(st[-3:] == 0)
    for b, A in enumerate(mats):
        n = A.shape[0]
        Tb = T[offs[b]:offs[b] + n * n].reshape((n, n), order="F")
        if st[b] == 0:
            _check(A, Tb, Z[offs[b]:offs[b] + n * n].reshape((n, n), order="F"), w[woffs[b]:woffs[b] + n])
        else:
            np.testing.assert_array_equal(Tb, A)


def test_mixed_graph_replay_matches(gs):
    rng = np.random.default_rng(5)
    mats = [randn_matrix(rng, int(n)) for n in rng.integers(8, 129, size=64)]
    packed, ns, offs, woffs = gs.pack_batch(mats)
    T1, Z1, w1, s1 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True, mixed=True)
    T2, Z2, w2, s2 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=True, mixed=True)
    T3, Z3, w3, s3 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, graph=False, mixed=True)
    np.testing.assert_array_equal(T1, T2)
    np.testing.assert_array_equal(T1, T3)
    np.testing.assert_array_equal(Z1, Z3)
    np.testing.assert_array_equal(w1, w3)


@pytest.mark.parametrize("bad_n", [129, -1])
def test_mixed_device_orders_out_of_range(gs, bad_n):
    """GS_DEVICE | GS_MIXED: an order outside [0, 128] gives that matrix GS_BADARG and
    leaves it untouched; the others are decomposed."""
    torch = pytest.importorskip("torch")
    from genericschur_gb300 import _capi
    rng = np.random.default_rng(78)
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
                                          _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE | _capi.GS_MIXED)
        assert rc == 0, ctx.last_error()
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
            np.testing.assert_array_equal(T[o:o + int(room[b])], packed[o:o + int(room[b])])
            continue
        assert status[b] == 0
        An = packed[o:o + n * n].reshape((n, n), order="F")
        assert_schur_real(An, T[o:o + n * n].reshape((n, n), order="F"), Zh[o:o + n * n].reshape((n, n), order="F"),
                          w[woffs[b]:woffs[b] + n])


def test_mixed_host_buffer_call_matches(gs):
    """A host-buffer call of 2048+ matrices (inputs copied in, the whole mixed sequence as one
    internally captured CUDA graph, outputs copied back) gives the results of the GS_GRAPH call
    bit for bit, and every 97th matrix passes the Schur checks."""
    rng = np.random.default_rng(61)
    mats = [randn_matrix(rng, int(n)) for n in rng.integers(4, 48, size=2300)]
    packed, ns, offs, woffs = gs.pack_batch(mats)
    T1, Z1, w1, s1 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, mixed=True)
    T2, Z2, w2, s2 = gs.gschur_batched(packed=packed, ns=ns, offs=offs, woffs=woffs, mixed=True, graph=True)
    assert np.all(s1 == 0) and np.all(s2 == 0)
    np.testing.assert_array_equal(T1, T2)
    np.testing.assert_array_equal(Z1, Z2)
    np.testing.assert_array_equal(w1, w2)
    for b in range(0, len(mats), 97):
        n = int(ns[b])
        o = int(offs[b])
        assert_schur_real(mats[b], T1[o:o + n * n].reshape((n, n), order="F"),
                          Z1[o:o + n * n].reshape((n, n), order="F"), w1[woffs[b]:woffs[b] + n])
