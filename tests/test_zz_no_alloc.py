"""GPU test of the allocation-free batched real Schur entry point.

Callers that cannot allocate device memory at call time (a host program or
framework that owns every device allocation, or a launch sequence being recorded
for replay) use gs_schur_batched_f64_noalloc, which keeps its work-queue scratch in
a static device array instead of allocating.  This test calls it through the C-ABI
twice in a row on device buffers and checks each result against the regular
entry point gs_schur_batched_f64, within the tolerances the other tests use.  It
lives in a file collected last so that a stop-at-first-failure run has already run
everything else, and it sets up everything it needs itself, so it also passes in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

from common import EPS, assert_schur_real

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point(gs):
    torch = pytest.importorskip("torch")
    from genericschur_gb300 import _capi
    from genericschur_gb300.workloads import batched_real

    lib = _capi.load()
    ctx = gs.get_context(0)
    packed, ns, offs, woffs = batched_real(count=300, seed=11)
    nw = int(ns.sum())
    dev = torch.device("cuda", 0)
    dA0 = torch.from_numpy(packed).to(dev)
    dns = torch.from_numpy(ns).to(dev)
    doffs = torch.from_numpy(offs).to(dev)
    dwoffs = torch.from_numpy(woffs).to(dev)
    stream = torch.cuda.Stream(dev)
    flags = _capi.GS_WANTZ | _capi.GS_SCALE

    def run(entry):
        A = dA0.clone()
        Z = torch.empty_like(A)
        wr = torch.empty(nw, dtype=torch.float64, device=dev)
        wi = torch.empty(nw, dtype=torch.float64, device=dev)
        st = torch.full((len(ns),), -1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        args = (len(ns), dns.data_ptr(), doffs.data_ptr(), dwoffs.data_ptr(), A.data_ptr(), Z.data_ptr(),
                wr.data_ptr(), wi.data_ptr(), st.data_ptr())
        if entry == "regular":
            ctx.set_stream(stream.cuda_stream)
            rc = lib.gs_schur_batched_f64(ctx.handle, *args, flags | _capi.GS_DEVICE)
            ctx.set_stream(None)
        else:
            free0 = torch.cuda.mem_get_info(dev)[0]
            rc = lib.gs_schur_batched_f64_noalloc(ctypes.c_void_p(stream.cuda_stream), *args, flags)
        assert rc == 0, (entry, rc)
        stream.synchronize()
        if entry != "regular":
            free_delta.append(free0 - torch.cuda.mem_get_info(dev)[0])
        return A.cpu().numpy(), Z.cpu().numpy(), wr.cpu().numpy() + 1j * wi.cpu().numpy(), st.cpu().numpy()

    free_delta = []

    T0, Z0, w0, s0 = run("regular")
    assert np.all(s0 == 0)
    for call in range(2):
        T1, Z1, w1, s1 = run("noalloc")
        assert np.all(s1 == 0), "call %d: status %s" % (call, np.unique(s1))
        for b in range(len(ns)):
            n = int(ns[b])
            o, q = int(offs[b]), int(woffs[b])
            A = packed[o:o + n * n].reshape(n, n, order="F")
            T = T1[o:o + n * n].reshape(n, n, order="F")
            Z = Z1[o:o + n * n].reshape(n, n, order="F")
            tol = 10 * n * EPS * np.linalg.norm(A)
            assert np.max(np.abs(T - T0[o:o + n * n].reshape(n, n, order="F"))) <= tol
            assert np.max(np.abs(Z - Z0[o:o + n * n].reshape(n, n, order="F"))) <= 10 * n * EPS
            assert np.max(np.abs(w1[q:q + n] - w0[q:q + n])) <= tol
            if b % 25 == 0:
                assert_schur_real(A, T, Z, w1[q:q + n])
    # The first call may load the code module that holds the static scratch array (the
    # memory every GPU that loads the library keeps); the second call must leave the
    # device's free memory exactly as it was: nothing is allocated on its behalf.
    assert free_delta[1] == 0, free_delta


def test_noalloc_rejects_oversized_batch(gs):
    from genericschur_gb300 import _capi
    lib = _capi.load()
    dummy = ctypes.c_void_p(1)
    rc = lib.gs_schur_batched_f64_noalloc(None, 65537, dummy, dummy, dummy, dummy, dummy, dummy, dummy, dummy, 0)
    assert rc == _capi.GS_BADARG


def test_noalloc_rejects_bad_orders_per_matrix(gs):
    """Orders are read on the device only: an order above 128 (or negative) gives that
    matrix GS_BADARG and leaves it untouched; the rest of the batch is decomposed."""
    torch = pytest.importorskip("torch")
    from genericschur_gb300 import _capi
    lib = _capi.load()
    gs.get_context(0)
    rng = np.random.default_rng(12)
    ns = np.array([30, 129, 100, -2, 8], dtype=np.int32)
    room = np.maximum(ns, 0).astype(np.int64) ** 2
    offs = np.concatenate([[0], np.cumsum(room)[:-1]]).astype(np.int64)
    woffs = np.concatenate([[0], np.cumsum(np.maximum(ns, 0))[:-1]]).astype(np.int64)
    packed = rng.standard_normal(int(room.sum()))
    dev = torch.device("cuda", 0)
    A = torch.from_numpy(packed).to(dev)
    Z = torch.zeros_like(A)
    nw = int(np.maximum(ns, 0).sum())
    wr = torch.zeros(nw, dtype=torch.float64, device=dev)
    wi = torch.zeros(nw, dtype=torch.float64, device=dev)
    st = torch.full((len(ns),), -1, dtype=torch.int32, device=dev)
    dns, doffs, dwoffs = (torch.from_numpy(x).to(dev) for x in (ns, offs, woffs))
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize()
    rc = lib.gs_schur_batched_f64_noalloc(ctypes.c_void_p(stream.cuda_stream), len(ns), dns.data_ptr(),
                                          doffs.data_ptr(), dwoffs.data_ptr(), A.data_ptr(), Z.data_ptr(),
                                          wr.data_ptr(), wi.data_ptr(), st.data_ptr(), _capi.GS_WANTZ | _capi.GS_SCALE)
    assert rc == 0
    stream.synchronize()
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
        q = int(woffs[b])
        assert_schur_real(packed[o:o + n * n].reshape(n, n, order="F"), T[o:o + n * n].reshape(n, n, order="F"),
                          Zh[o:o + n * n].reshape(n, n, order="F"), w[q:q + n])
