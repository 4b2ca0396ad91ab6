"""The batched kernels' tuning table (gs_set_tuning / gs_get_tuning) and the tuned
launch shapes.

CPU: the table parser accepts the tuner's format, rejects shapes that are not compiled
or do not fit in shared memory and bounds that do not increase to 128 (keeping the
previous shapes), and the committed table parses.  GPU: every compiled shape, in every
bin it fits, gives Schur forms that meet the parity rule of the other tests (for the
FP32 stage of the mixed form: after the refinement).
"""
import ctypes
import os

import numpy as np
import pytest

from common import assert_schur_cplx, assert_schur_real, eig_tolerances, match_eigenvalues, randn_matrix

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COMMITTED = os.path.join(ROOT, "genericschur.jl_gb300", "genericschur_gb300", "tuning", "sm_103a.tsv")
THREADS = [64, 96, 128, 160, 192, 256]


@pytest.fixture(scope="module")
def raw_ctx():
    """A context handle for the host-only calls (gs_create reports GS_CUDA without a
    GPU but still returns a handle on which gs_set_tuning / gs_get_tuning work)."""
    import build_lib
    build_lib.build()
    from genericschur_gb300 import _capi
    lib = _capi.load()
    h = ctypes.c_void_p()
    lib.gs_create(ctypes.byref(h), 0)
    assert h.value
    yield lib, h
    lib.gs_destroy(h)


def _text(lib, h):
    buf = ctypes.create_string_buffer(4096)
    assert lib.gs_get_tuning(h, buf, len(buf)) == 0
    return buf.value.decode()


def _rows(text):
    return [ln.split() for ln in text.splitlines() if ln and not ln.startswith("#")]


def test_defaults_and_roundtrip(raw_ctx, tmp_path):
    lib, h = raw_ctx
    assert lib.gs_set_tuning(h, None) == 0
    rows = _rows(_text(lib, h))
    assert len(rows) == 12
    assert rows[3] == ["real_f64", "3", "128", "128", "0", "0"]
    assert rows[11] == ["mixed_f32", "3", "128", "128", "0", "0"]
    p = tmp_path / "t.tsv"
    p.write_text("# comment\nreal_f64 3 128 160 0 0\nreal_f64 2 104 192 0 2\ncomplex_f64 0 32 96 1 0\n"
                 "mixed_f32 3 128 256 1 0\n")
    assert lib.gs_set_tuning(h, str(p).encode()) == 0
    rows = _rows(_text(lib, h))
    assert rows[3] == ["real_f64", "3", "128", "160", "0", "0"]
    assert rows[2] == ["real_f64", "2", "104", "192", "0", "2"]
    assert rows[4] == ["complex_f64", "0", "32", "96", "1", "0"]
    assert rows[11] == ["mixed_f32", "3", "128", "256", "1", "0"]
    # the active table is itself a valid table
    q = tmp_path / "q.tsv"
    q.write_text(_text(lib, h))
    assert lib.gs_set_tuning(h, str(q).encode()) == 0
    assert _rows(_text(lib, h)) == rows
    assert lib.gs_set_tuning(h, None) == 0


@pytest.mark.parametrize("line", [
    "real_f64 3 128 100 0 0",        # thread count that is not compiled
    "complex_f64 3 128 128 1 0",     # full complex 128 x 128 matrix does not fit in shared memory
    "real_f64 3 120 128 0 0",        # last bin must end at 128
    "real_f64 1 100 64 1 0",         # bounds must increase (bin 1 above bin 2's 96)
    "imag_f64 0 32 64 1 0",          # unknown kind
    "real_f64 4 128 128 0 0",        # bin out of range
    "real_f64 0 32 64",              # missing fields
    "real_f64 0 32 64 2 0",          # hsmem is 0 or 1
    "mixed_f32 2 100 128 0 0",       # the FP32 stage keeps the default bounds
    "mixed_f32 0 32 160 1 0",        # 160 threads are not compiled in FP32
])
def test_rejects_bad_tables(raw_ctx, tmp_path, line):
    lib, h = raw_ctx
    good = tmp_path / "g.tsv"
    good.write_text("real_f64 3 128 160 0 0\n")
    assert lib.gs_set_tuning(h, str(good).encode()) == 0
    before = _text(lib, h)
    bad = tmp_path / "b.tsv"
    bad.write_text(line + "\n")
    assert lib.gs_set_tuning(h, str(bad).encode()) == 2
    assert lib.gs_last_error(h)
    assert _text(lib, h) == before
    assert lib.gs_set_tuning(h, b"/nonexistent/table.tsv") == 2
    assert lib.gs_set_tuning(h, None) == 0


def test_committed_table_parses(raw_ctx):
    if not os.path.exists(COMMITTED):
        pytest.skip("no committed tuning table")
    lib, h = raw_ctx
    assert lib.gs_set_tuning(h, COMMITTED.encode()) == 0
    rows = _rows(_text(lib, h))
    assert int(rows[3][2]) == 128 and int(rows[7][2]) == 128
    assert lib.gs_set_tuning(h, None) == 0


def _batch(rng, cplx):
    ns = [1, 2, 5, 17, 32, 33, 50, 64, 65, 80, 96, 97, 110, 127, 128]
    return [randn_matrix(rng, n, cplx=cplx) for n in ns]


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["real_f64", "complex_f64", "mixed_f32"])
@pytest.mark.parametrize("nt", THREADS)
@pytest.mark.parametrize("hs", [0, 1])
def test_every_shape_parity(gs, tmp_path, kind, nt, hs):
    """Every compiled shape, placed in every default bin whose orders it can hold, gives
    Schur forms within the parity bounds (10 n eps backward and orthogonality errors,
    eigenvalues matched to the oracle's within 1e2 n eps ||A||_F / s_i)."""
    from oracle import pyoracle as po
    cplx = kind == "complex_f64"
    mixed = kind == "mixed_f32"
    if mixed and nt == 160:
        pytest.skip("160 threads are not compiled in FP32")
    lines = []
    for b, hi in enumerate([32, 64, 96, 128]):
        size = (16 if cplx else (4 if mixed else 8)) * ((hi * (hi | 1)) if hs else hi * hi // 2)
        if size < 200 * 1024:
            lines.append("%s %d %d %d %d 0" % (kind, b, hi, nt, hs))
    if not lines:
        pytest.skip("shape fits no bin")
    p = tmp_path / "shape.tsv"
    p.write_text("\n".join(lines) + "\n")
    ctx = gs.Context(0)
    ctx.set_tuning(str(p))
    try:
        mats = _batch(np.random.default_rng(31 + nt + hs), cplx)
        Ts, Zs, ws, st = gs.gschur_batched(mats, ctx=ctx, mixed=mixed)
        assert np.all(st == 0)
        for k, (A, T, Z, w) in enumerate(zip(mats, Ts, Zs, ws)):
            (assert_schur_cplx if cplx else assert_schur_real)(A, T, Z, w)
            if k % 3 == 0:
                w_ref, tol = eig_tolerances(A, po)
                ok, worst = match_eigenvalues(w, w_ref, tol)
                assert ok, "n=%d: worst err/tol %.3g" % (A.shape[0], worst)
    finally:
        ctx.close()
