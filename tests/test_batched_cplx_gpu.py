"""GPU parity tests of the complex FP64 Schur kernels against the CPU oracle.

Criteria: T upper triangular, values == diag(T) (test/complex.jl:1-34),
||A - Z T Z^H||_F / ||A||_F <= 10 n eps, ||Z^H Z - I||_F <= 10 n eps, eigenvalues
matched to the oracle's within 1e2 n eps ||A||_F / s_i.
"""
import numpy as np
import pytest

from common import EPS, assert_schur_cplx, eig_tolerances, godunov, match_eigenvalues, randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 4, 5, 8, 16, 31, 32, 33, 64, 65, 96, 97, 112, 113, 127, 128]


@pytest.mark.parametrize("n", SIZES)
def test_single_random(gs, n):
    rng = np.random.default_rng(2000 + n)
    A = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, "worst err/tol %.3g" % worst


def test_batched_mixed_sizes(gs):
    rng = np.random.default_rng(5)
    ns = list(rng.integers(8, 129, size=120)) + [1, 2, 128, 0]
    mats = [randn_matrix(rng, int(n), cplx=True) for n in ns]
    Ts, Zs, ws, status = gs.gschur_batched(mats)
    assert np.all(status == 0)
    for A, T, Z, w in zip(mats, Ts, Zs, ws):
        if A.shape[0]:
            assert_schur_cplx(A, T, Z, w)
    for idx in range(0, len(mats), 13):
        A = mats[idx]
        if A.shape[0] == 0:
            continue
        w_ref, tol = eig_tolerances(A, po)
        ok, worst = match_eigenvalues(ws[idx], w_ref, tol)
        assert ok, "matrix %d: worst %.3g" % (idx, worst)


@pytest.mark.parametrize("n", [4, 32, 120])
def test_unitary_normal(gs, n):
    # random unitary: Schur form is diagonal (test/complex.jl:130-135)
    rng = np.random.default_rng(600 + n)
    Q, R = np.linalg.qr(randn_matrix(rng, n, cplx=True))
    U = Q @ np.diag(np.sign(np.diag(R)))
    S = gs.gschur(U)
    assert_schur_cplx(U, S.T, S.Z, S.values, tol=20.0)
    assert np.linalg.norm(np.triu(S.T, 1)) / (n * np.linalg.norm(U) * EPS) < 20


@pytest.mark.parametrize("n", [4, 32, 128])
def test_jordan(gs, n):
    A = (np.diag(np.ones(n - 1), 1) + np.eye(n)).astype(np.complex128)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values, tol=20.0)


@pytest.mark.parametrize("s", [1e-300, 1e300])
def test_extreme_scaling(gs, s):
    rng = np.random.default_rng(18)
    n = 20
    A0 = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(s * A0)
    be = np.linalg.norm(A0 - S.Z @ (S.T / s) @ S.Z.conj().T) / np.linalg.norm(A0)
    assert be <= 10 * n * EPS
    assert np.all(np.tril(S.T, -1) == 0)


def test_godunov_complex(gs):
    A, vals, econd = godunov()
    A = A.astype(np.complex128)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)
    w_ref, tol = eig_tolerances(A, po)
    ok, worst = match_eigenvalues(S.values, w_ref, tol)
    assert ok, worst


def test_real_input_as_complex(gs):
    rng = np.random.default_rng(19)
    A = rng.standard_normal((40, 40)).astype(np.complex128)
    S = gs.gschur(A)
    assert_schur_cplx(A, S.T, S.Z, S.values)


def test_unconverged_status(gs):
    rng = np.random.default_rng(20)
    A = randn_matrix(rng, 20, cplx=True)
    with pytest.raises(gs.UnconvergedException):
        gs.gschur(A, maxiter=3)


@pytest.mark.parametrize("bad_n", [129, -1])
def test_device_orders_out_of_range(gs, bad_n):
    """GS_DEVICE complex batches: an order outside [0, 128] read on the device gives
    that matrix status GS_BADARG and leaves it untouched; the others are decomposed."""
    torch = pytest.importorskip("torch")
    from genericschur_gb300 import _capi
    rng = np.random.default_rng(78)
    ns = np.array([16, bad_n, 128, 45], dtype=np.int32)
    room = np.maximum(ns, 0).astype(np.int64) ** 2
    offs = np.concatenate([[0], np.cumsum(room)[:-1]]).astype(np.int64)
    woffs = np.concatenate([[0], np.cumsum(np.maximum(ns, 0))[:-1]]).astype(np.int64)
    m = int(room.sum())
    packed = (rng.standard_normal(m) + 1j * rng.standard_normal(m)) / np.sqrt(2)
    dev = torch.device("cuda", 0)
    ctx = gs.get_context(0)
    stream = torch.cuda.Stream(dev)
    A = torch.from_numpy(packed.view(np.float64).copy()).to(dev)
    Z = torch.zeros_like(A)
    w = torch.zeros(2 * int(np.maximum(ns, 0).sum()), dtype=torch.float64, device=dev)
    st = torch.full((len(ns),), -1, dtype=torch.int32, device=dev)
    dns, doffs, dwoffs = (torch.from_numpy(x).to(dev) for x in (ns, offs, woffs))
    torch.cuda.synchronize()
    ctx.set_stream(stream.cuda_stream)
    try:
        rc = ctx.lib.gs_schur_batched_c64(ctx.handle, len(ns), dns.data_ptr(), doffs.data_ptr(), dwoffs.data_ptr(),
                                          A.data_ptr(), Z.data_ptr(), w.data_ptr(), st.data_ptr(),
                                          _capi.GS_WANTZ | _capi.GS_SCALE | _capi.GS_DEVICE)
        assert rc == 0
        stream.synchronize()
    finally:
        ctx.set_stream(None)
    status = st.cpu().numpy()
    T = A.cpu().numpy().view(np.complex128)
    Zh = Z.cpu().numpy().view(np.complex128)
    wh = w.cpu().numpy().view(np.complex128)
    for b, n in enumerate(ns):
        o = int(offs[b])
        if n < 0 or n > 128:
            assert status[b] == _capi.GS_BADARG
            np.testing.assert_array_equal(T[o:o + room[b]], packed[o:o + room[b]])
            continue
        assert status[b] == 0
        A0 = packed[o:o + n * n].reshape(n, n, order="F")
        q = int(woffs[b])
        assert_schur_cplx(A0, T[o:o + n * n].reshape(n, n, order="F"), Zh[o:o + n * n].reshape(n, n, order="F"),
                          wh[q:q + n])
