"""CPU checks of the C-ABI boundary: the library builds, loads and exports every
entry point that include/gschur_gb300.h declares; host-side argument handling
raises the reference's exception types without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(HEADER_DIR):
        if fn.endswith(".h"):
            text = open(os.path.join(HEADER_DIR, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(gs_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_all_declared_symbols():
    import build_lib
    path = build_lib.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from genericschur_gb300 import _capi
    assert set(declared_symbols()) == set(_capi.SIGNATURES)


def test_version_call_needs_no_gpu():
    from genericschur_gb300 import _capi
    assert _capi.load().gs_version() >= 100


def test_non_square_raises_dimension_mismatch():
    # test/errors.jl:12-13
    import genericschur_gb300 as g
    with pytest.raises(g.DimensionMismatch):
        g.gschur(np.zeros((5, 4)))
    with pytest.raises(g.DimensionMismatch):
        g.gschur(np.zeros((5, 4), dtype=np.complex128))


def test_integer_input_rejected():
    # "letter of marque": no methods for integer element types (test/errors.jl:16-27)
    import genericschur_gb300 as g
    with pytest.raises(TypeError):
        g.gschur(np.arange(16).reshape(4, 4))


def test_pack_unpack_roundtrip():
    import genericschur_gb300 as g
    rng = np.random.default_rng(0)
    mats = [rng.standard_normal((n, n)) for n in (1, 3, 8, 0, 5)]
    packed, ns, offs, woffs = g.pack_batch(mats)
    back = g.unpack_batch(packed, ns, offs)
    for a, b in zip(mats, back):
        np.testing.assert_array_equal(a, b)
    assert list(woffs) == [0, 1, 4, 12, 12]


def test_algorithm_selection():
    """geigen!/geigvals!/_gschur! take QRIteration() (the default) or DivideAndConquer()
    (GenericSchur.jl:119-161); RobustRepresentations falls back to QRIteration with a warning
    (symtridiag.jl:12-26) and any other algorithm raises ArgumentError (symtridiag.jl:61-67)."""
    import warnings
    import genericschur_gb300 as gs
    assert gs._alg(None) == "QR" and gs._alg("QRIteration") == "QR"
    assert gs._alg("DivideAndConquer") == "DC"

    class DivideAndConquer:
        pass

    assert gs._alg(DivideAndConquer()) == "DC"
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        assert gs._alg("RobustRepresentations") == "QR"
        assert any("falling back to QRIteration" in str(x.message) for x in w)
    with pytest.raises(gs.ArgumentError):
        gs._alg("Jacobi")


def test_generalized_sylvester_shape_checks():
    """trsylvester!(A, B, C, D, E, F) checks its dimensions before any GPU work
    (gsylvester.jl:29-47)."""
    import genericschur_gb300 as gs
    with pytest.raises(gs.DimensionMismatch):
        gs.trsylvester(np.eye(3), np.eye(2), np.zeros((3, 2)), np.eye(2), np.eye(2), np.zeros((3, 2)),
                       ctx=object())
    with pytest.raises(gs.DimensionMismatch):
        gs.trsylvester(np.eye(3), np.eye(2), np.zeros((2, 2)), ctx=object())
