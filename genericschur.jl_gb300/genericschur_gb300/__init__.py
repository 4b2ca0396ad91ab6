"""GB300 dense Schur engine — Python host mirror of GenericSchur.jl's API.

Each function keeps the name, argument meaning and error behaviour of the
GenericSchur.jl function it replaces (Julia's trailing `!` becomes a trailing
underscore):

  gschur(A)  / gschur_(A)      GenericSchur.jl:343 / 805-835 (real), 350-372 (complex)
  schur(A)                      pirates.jl:8-10 (schur!) through the non-mutating wrapper
  eigvals(A)                    pirates.jl:17-27
  eigvecs(S; left) / geigvecs   pirates.jl:38-48 / vectors.jl:12-20
  eigen(A)                      pirates.jl:63-89 (without balancing)
  triangularize(S)              triang.jl:9-43
  hessenberg(A)                 pirates.jl:232 / hessenberg.jl:3-17, 150-166
  gschur_batched(...)           batched form, no reference counterpart
  geigvecs_batched(...)         batched eigenvectors, no reference counterpart
  eig_adjoint_batched(...)      eigenvalue adjoint (reverse-mode rule), no reference counterpart

Matrices are numpy arrays; they are handed to the C-ABI column-major (Julia's
layout).  All arithmetic runs in the CUDA library; nothing here computes a
decomposition, and there is no CPU fallback.
"""
from collections import namedtuple

import numpy as np

from . import _capi
from ._capi import (GS_BADARG, GS_CUDA, GS_DEVICE, GS_GRAPH, GS_OK, GS_SCALE, GS_UNCONVERGED, GS_WANTZ, Context,
                    GSError, get_context)

__all__ = ["Schur", "Eigen", "UnconvergedException", "DimensionMismatch", "ArgumentError", "gschur", "gschur_",
           "schur", "eigvals", "eigvecs", "geigvecs", "eigen", "triangularize", "gschur_batched", "geigvecs_batched",
           "eig_adjoint_batched", "hessenberg", "gschur_mixed", "balance", "balance_", "Balancer", "balancer_lmul",
           "balancer_ldiv", "enormalize", "gordschur", "ordschur", "rconde", "EigenFull", "eigvalscond",
           "subspacesep", "eigen_rcond", "Hermitian", "SymTridiagonal", "HermitianHessenberg", "geigen",
           "geigvals", "gschur_symtridiag", "hessenberg_hermitian", "GeneralizedSchur", "ggschur", "ggschur_batched", "ggeigvecs", "trsylvester", "adjtrsylvester",
           "get_context", "Context", "pack_batch", "unpack_batch"]

# LinearAlgebra.Eigen(values, vectors)
Eigen = namedtuple("Eigen", ["values", "vectors"])

# LinearAlgebra.Schur(T, Z, values)
Schur = namedtuple("Schur", ["T", "Z", "values"])


class UnconvergedException(RuntimeError):
    """Iteration limit reached (GenericSchur.jl:39-45)."""


class DimensionMismatch(ValueError):
    """Non-square input or mismatched Z (GenericSchur.jl:523-525, LinearAlgebra.checksquare)."""


class ArgumentError(ValueError):
    """Invalid argument (GenericSchur.jl:206-210)."""


def _raise(rc, ctx, what):
    msg = "%s: %s" % (what, ctx.last_error())
    if rc == GS_UNCONVERGED:
        raise UnconvergedException("Convergence failure; " + msg)
    if rc == GS_BADARG:
        raise ArgumentError(msg)
    raise GSError(rc, msg)


def _ptr(a):
    return a.ctypes.data if a is not None else None


def _checksquare(A):
    if A.ndim != 2 or A.shape[0] != A.shape[1]:
        raise DimensionMismatch("matrix is not square: dimensions are %s" % (A.shape,))
    return A.shape[0]


def gschur_(A, wantZ=True, scale=True, maxiter=None, maxinner=None, ctx=None):
    """Destructive Schur decomposition: A (Fortran-ordered float64/complex128 array)
    is overwritten by T.  Returns Schur(T, Z, values), T being A itself."""
    n = _checksquare(A)
    ctx = ctx or get_context()
    if not (A.flags.f_contiguous and A.dtype in (np.float64, np.float32, np.complex128)):
        raise ArgumentError("gschur_ needs a Fortran-ordered float64, float32 or complex128 array")
    flags = (GS_WANTZ if wantZ else 0) | (GS_SCALE if scale else 0)
    lib = ctx.lib
    if A.dtype == np.complex128:
        Z = np.zeros((n, n), dtype=np.complex128, order="F") if wantZ else None
        w = np.zeros(n, dtype=np.complex128)
        rc = lib.gs_schur_c64(ctx.handle, n, _ptr(A), max(n, 1), _ptr(Z), max(n, 1), _ptr(w), flags,
                              int(maxiter or 0), int(maxinner or 0))
        if rc != GS_OK:
            _raise(rc, ctx, "gschur")
        return Schur(A, Z if wantZ else np.zeros((0, 0), dtype=np.complex128), w)
    dt = A.dtype
    Z = np.zeros((n, n), dtype=dt, order="F") if wantZ else None
    wr = np.zeros(n, dtype=dt)
    wi = np.zeros(n, dtype=dt)
    fn = lib.gs_schur_f32 if dt == np.float32 else lib.gs_schur_f64
    rc = fn(ctx.handle, n, _ptr(A), max(n, 1), _ptr(Z), max(n, 1), _ptr(wr), _ptr(wi), flags, int(maxiter or 0))
    if rc != GS_OK:
        _raise(rc, ctx, "gschur")
    return Schur(A, Z if wantZ else np.zeros((0, 0), dtype=dt), wr + 1j * wi)


def gschur(A, **kw):
    """Schur decomposition of a copy of A (GenericSchur.jl:343)."""
    A = np.asarray(A)
    if A.dtype.kind in "iub":
        raise TypeError("gschur is defined for floating-point element types only")
    if np.iscomplexobj(A):
        dt = np.complex128
    else:
        dt = np.float32 if A.dtype == np.float32 else np.float64  # Float32 stays Float32, as in the reference
    return gschur_(np.array(A, dtype=dt, order="F", copy=True), **kw)


# LinearAlgebra.GeneralizedSchur(S, T, alpha, beta, Q, Z): A = Q S Z', B = Q T Z'
GeneralizedSchur = namedtuple("GeneralizedSchur", ["S", "T", "alpha", "beta", "Q", "Z"])


def _ggschur_real(A, B, wantQ, wantZ, scale, ctx):
    S = np.array(A, dtype=np.float64, order="F", copy=True)
    T = np.array(B, dtype=np.float64, order="F", copy=True)
    n = _checksquare(S)
    if _checksquare(T) != n:
        raise ArgumentError("matrices must have the same sizes")
    Q = np.zeros((n, n), order="F") if wantQ else None
    Z = np.zeros((n, n), order="F") if wantZ else None
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1))
    rc = ctx.lib.gs_ggschur_f64(ctx.handle, n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(al), _ptr(be),
                                _capi.GS_SCALE if scale else 0)
    if rc != GS_OK:
        _raise(rc, ctx, "ggschur!")
    return GeneralizedSchur(S, T, al[:n], be[:n], Q, Z)


def ggschur(A, B, wantQ=True, wantZ=True, scale=True, ctx=None):
    """ggschur!(A, B; wantQ, wantZ, scale) on copies, on the GPU: the generalized Schur form
    of the pencil (A, B).  Complex pencils (generalized.jl:21-80): S, T upper triangular.
    Real pencils (rgeneralized.jl:10-66): S quasi-triangular with 2 x 2 blocks for complex
    eigenvalue pairs, T upper triangular, alpha complex and beta real."""
    ctx = ctx or get_context()
    if not (np.iscomplexobj(A) or np.iscomplexobj(B)):
        return _ggschur_real(A, B, wantQ, wantZ, scale, ctx)
    S = np.array(A, dtype=np.complex128, order="F", copy=True)
    T = np.array(B, dtype=np.complex128, order="F", copy=True)
    n = _checksquare(S)
    if _checksquare(T) != n:
        raise ArgumentError("matrices must have the same sizes")
    Q = np.zeros((n, n), dtype=np.complex128, order="F") if wantQ else None
    Z = np.zeros((n, n), dtype=np.complex128, order="F") if wantZ else None
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1), dtype=np.complex128)
    rc = ctx.lib.gs_ggschur_c64(ctx.handle, n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(al), _ptr(be),
                                _capi.GS_SCALE if scale else 0)
    if rc != GS_OK:
        _raise(rc, ctx, "ggschur!")
    return GeneralizedSchur(S, T, al[:n], be[:n], Q, Z)


def ggschur_batched(As, Bs, wantQ=True, wantZ=True, scale=True, ctx=None):
    """ggschur! over a list of pencils in one launch (one CTA per pencil).  Returns a list
    of GeneralizedSchur and the per-pencil status.  All-real lists take the real QZ."""
    ctx = ctx or get_context()
    if not any(np.iscomplexobj(a) for a in list(As) + list(Bs)):
        return _ggschur_batched_real(As, Bs, wantQ, wantZ, scale, ctx)
    Ap, ns, offs, woffs = pack_batch(As, dtype=np.complex128)
    Bp, ns2, _, _ = pack_batch(Bs, dtype=np.complex128)
    if not np.array_equal(ns, ns2):
        raise ArgumentError("matrices must have the same sizes")
    plen = len(Ap)
    wlen = int(ns.sum())
    Qp = np.zeros(plen, dtype=np.complex128) if wantQ else None
    Zp = np.zeros(plen, dtype=np.complex128) if wantZ else None
    al = np.zeros(max(wlen, 1), dtype=np.complex128)
    be = np.zeros(max(wlen, 1), dtype=np.complex128)
    st = np.zeros(len(ns), dtype=np.int32)
    rc = ctx.lib.gs_ggschur_batched_c64(ctx.handle, len(ns), _ptr(ns), _ptr(offs), plen, _ptr(Ap), _ptr(Bp), _ptr(Qp),
                                        _ptr(Zp), _ptr(woffs), wlen, _ptr(al), _ptr(be), _ptr(st),
                                        _capi.GS_SCALE if scale else 0)
    if rc not in (GS_OK, GS_UNCONVERGED):
        _raise(rc, ctx, "ggschur! (batched)")
    out = []
    for k, n in enumerate(ns):
        n = int(n)
        o, w = int(offs[k]), int(woffs[k])
        sl = slice(o, o + n * n)
        out.append(GeneralizedSchur(Ap[sl].reshape(n, n, order="F"), Bp[sl].reshape(n, n, order="F"),
                                    al[w:w + n].copy(), be[w:w + n].copy(),
                                    Qp[sl].reshape(n, n, order="F") if wantQ else None,
                                    Zp[sl].reshape(n, n, order="F") if wantZ else None))
    return out, st


def _ggschur_batched_real(As, Bs, wantQ, wantZ, scale, ctx):
    Ap, ns, offs, woffs = pack_batch(As, dtype=np.float64)
    Bp, ns2, _, _ = pack_batch(Bs, dtype=np.float64)
    if not np.array_equal(ns, ns2):
        raise ArgumentError("matrices must have the same sizes")
    plen = len(Ap)
    wlen = int(ns.sum())
    Qp = np.zeros(plen) if wantQ else None
    Zp = np.zeros(plen) if wantZ else None
    al = np.zeros(max(wlen, 1), dtype=np.complex128)
    be = np.zeros(max(wlen, 1))
    st = np.zeros(len(ns), dtype=np.int32)
    rc = ctx.lib.gs_ggschur_batched_f64(ctx.handle, len(ns), _ptr(ns), _ptr(offs), plen, _ptr(Ap), _ptr(Bp), _ptr(Qp),
                                        _ptr(Zp), _ptr(woffs), wlen, _ptr(al), _ptr(be), _ptr(st),
                                        _capi.GS_SCALE if scale else 0)
    if rc not in (GS_OK, GS_UNCONVERGED):
        _raise(rc, ctx, "ggschur! (batched)")
    out = []
    for k, n in enumerate(ns):
        n = int(n)
        o, w = int(offs[k]), int(woffs[k])
        sl = slice(o, o + n * n)
        out.append(GeneralizedSchur(Ap[sl].reshape(n, n, order="F"), Bp[sl].reshape(n, n, order="F"),
                                    al[w:w + n].copy(), be[w:w + n].copy(),
                                    Qp[sl].reshape(n, n, order="F") if wantQ else None,
                                    Zp[sl].reshape(n, n, order="F") if wantZ else None))
    return out, st


def schur(A, B=None, **kw):
    """schur(A) (pirates.jl:8-10) or schur(A, B) -> ggschur (pirates.jl:11-15)."""
    if B is not None:
        return ggschur(A, B, **kw)
    return _schur1(A, **kw)


def _schur1(A, **kw):
    """LinearAlgebra.schur through the pirated schur! (pirates.jl:8-10)."""
    return gschur(A, **kw)


def _eigsortby(w):
    # LinearAlgebra.eigsortby: lexicographic by (real, imag)
    return np.lexsort((w.imag, w.real))


def eigvals(A, B=None, sortby="default", **kw):
    """Eigenvalues via gschur!(A; wantZ=false) (pirates.jl:17-27); for a Hermitian or
    SymTridiagonal argument, geigvals! with alg= (GenericSchur.jl:138-146, symtridiag.jl:51-57,
    pirates.jl:170-197); for a pencil (A, B), alpha ./ beta of ggschur! in the Schur form's
    order."""
    alg = kw.pop("alg", None)
    if B is not None:
        G = ggschur(A, B, wantQ=False, wantZ=False, ctx=kw.get("ctx"))
        with np.errstate(divide="ignore", invalid="ignore"):
            return G.alpha / G.beta
    if isinstance(A, Hermitian):
        return geigvals(A, alg=alg, sortby=sortby, **kw)
    if isinstance(A, SymTridiagonal):
        return _st_eig(A, False, sortby, kw.get("ctx"), alg)[0]
    if alg is not None:
        raise ArgumentError("alg applies to Hermitian and SymTridiagonal arguments")
    S = gschur(A, wantZ=False, **kw)
    w = S.values
    if sortby is None:
        return w
    if sortby == "default":
        return w[_eigsortby(w)]
    return w[np.argsort([sortby(x) for x in w], kind="stable")]


# ---------------------------------------------------------------------------
# batched form
# ---------------------------------------------------------------------------
def pack_batch(mats, dtype=np.float64):
    """Pack a list of square matrices column-major into one buffer.
    Returns (packed, ns int32, offs int64, woffs int64)."""
    ns = np.array([m.shape[0] for m in mats], dtype=np.int32)
    sq = ns.astype(np.int64) ** 2
    offs = np.zeros(len(mats), dtype=np.int64)
    if len(mats) > 1:
        offs[1:] = np.cumsum(sq)[:-1]
    woffs = np.zeros(len(mats), dtype=np.int64)
    if len(mats) > 1:
        woffs[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    packed = np.empty(int(sq.sum()), dtype=dtype)
    for m, o, n in zip(mats, offs, ns):
        packed[o:o + n * n] = np.asarray(m, dtype=dtype).ravel(order="F")
    return packed, ns, offs, woffs


def unpack_batch(packed, ns, offs):
    return [packed[o:o + n * n].reshape((n, n), order="F") for o, n in zip(offs, ns)]


def gschur_batched(mats=None, packed=None, ns=None, offs=None, woffs=None, wantZ=True, scale=True, graph=False,
                   ctx=None, raise_on_failure=True, mixed=False, fallback=True):
    """gschur! over a ragged batch (orders <= 128) in one launch sequence.

    Pass either `mats` (list of square arrays) or the packed form (packed, ns,
    offs, woffs) as produced by pack_batch.  Returns (T_list, Z_list, values_list,
    status) for `mats`, or (T_packed, Z_packed, w_packed, status) for packed input.
    mixed=True (real Float64 only): FP32 Schur pairs refined to FP64 accuracy by
    Newton steps; matrices the refinement cannot finish are recomputed in FP64, or,
    with fallback=False, reported as unconverged.
    """
    ctx = ctx or get_context()
    lists = mats is not None
    if lists:
        for m in mats:
            _checksquare(np.asarray(m))
        cplx = any(np.iscomplexobj(m) for m in mats)
        single = (not cplx) and all(np.asarray(m).dtype == np.float32 for m in mats) and len(mats) > 0
        packed, ns, offs, woffs = pack_batch(mats, np.complex128 if cplx else (np.float32 if single else np.float64))
    else:
        cplx = np.iscomplexobj(packed)
        single = (not cplx) and np.asarray(packed).dtype == np.float32
        packed = np.array(packed, copy=True)
    count = len(ns)
    ns = np.ascontiguousarray(ns, dtype=np.int32)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    woffs = np.ascontiguousarray(woffs, dtype=np.int64)
    nw = int(ns.sum()) if count else 0
    nw = max(nw, int((woffs + ns).max()) if count else 0)
    flags = (GS_WANTZ if wantZ else 0) | (GS_SCALE if scale else 0) | (GS_GRAPH if graph else 0)
    if mixed:
        if cplx or single:
            raise ArgumentError("gschur_batched: mixed=True applies to real Float64 batches")
        flags |= _capi.GS_MIXED | (0 if fallback else _capi.GS_NOFALLBACK)
    status = np.zeros(count, dtype=np.int32)
    Z = np.zeros_like(packed) if wantZ else None
    lib = ctx.lib
    if cplx:
        w = np.zeros(nw, dtype=np.complex128)
        rc = lib.gs_schur_batched_c64(ctx.handle, count, _ptr(ns), _ptr(offs), _ptr(woffs), _ptr(packed), _ptr(Z),
                                      _ptr(w), _ptr(status), flags)
    else:
        dt = np.float32 if single else np.float64
        wr = np.zeros(nw, dtype=dt)
        wi = np.zeros(nw, dtype=dt)
        fn = lib.gs_schur_batched_f32 if single else lib.gs_schur_batched_f64
        rc = fn(ctx.handle, count, _ptr(ns), _ptr(offs), _ptr(woffs), _ptr(packed), _ptr(Z), _ptr(wr), _ptr(wi),
                _ptr(status), flags)
        w = wr + 1j * wi
    if rc not in (GS_OK, GS_UNCONVERGED) or (rc == GS_UNCONVERGED and raise_on_failure):
        _raise(rc, ctx, "gschur_batched")
    if not lists:
        return packed, Z, w, status
    Ts = unpack_batch(packed, ns, offs)
    Zs = unpack_batch(Z, ns, offs) if wantZ else [None] * count
    ws = [w[o:o + n] for o, n in zip(woffs, ns)]
    return Ts, Zs, ws, status


# ---------------------------------------------------------------------------
# eigenvectors, triangularize, eigen
# ---------------------------------------------------------------------------
def _fc(a, dt):
    return np.array(a, dtype=dt, order="F", copy=True)


def ggeigvecs(G, left=False, ctx=None):
    """geigvecs(S::GeneralizedSchur; left) (vectors.jl:22-33) for a complex pencil: right
    eigenvectors v_k with beta_k A v_k = alpha_k B v_k (back-transformed by G.Z), or left
    eigenvectors (back-transformed by G.Q); columns scaled to max |re|+|im| = 1."""
    ctx = ctx or get_context()
    if not (np.iscomplexobj(G.S) or np.iscomplexobj(G.T)):
        # real pencil (vectors.jl:1040-1513): complex vectors, conjugate columns for a pair
        S = _fc(G.S, np.float64)
        T = _fc(G.T, np.float64)
        n = _checksquare(S)
        V = np.zeros((n, n), dtype=np.complex128, order="F")
        if n == 0:
            return V
        M = G.Q if left else G.Z
        M = _fc(M, np.float64) if M is not None else None
        Q, Z = (M, None) if left else (None, M)
        outR, outL = (None, V) if left else (V, None)
        rc = ctx.lib.gs_ggeigvecs_f64(ctx.handle, n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(outR), _ptr(outL), 0)
        if rc != GS_OK:
            _raise(rc, ctx, "geigvecs(GeneralizedSchur)")
        return V
    S = _fc(G.S, np.complex128)
    T = _fc(G.T, np.complex128)
    n = _checksquare(S)
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    if n == 0:
        return V
    M = G.Q if left else G.Z
    M = _fc(M, np.complex128) if M is not None else None
    Q, Z = (M, None) if left else (None, M)
    outR, outL = (None, V) if left else (V, None)
    rc = ctx.lib.gs_ggeigvecs_c64(ctx.handle, n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(outR), _ptr(outL), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "geigvecs(GeneralizedSchur)")
    return V


def geigvecs(S, left=False, normalize=True, ctx=None):
    """Eigenvectors from a Schur decomposition (vectors.jl:12-20): right, or left
    with left=True; columns ordered like S.values, unit 2-norm with the
    largest-modulus entry real.  A GeneralizedSchur goes to ggeigvecs (vectors.jl:22-33)."""
    if isinstance(S, GeneralizedSchur):
        return ggeigvecs(S, left=left, ctx=ctx)
    ctx = ctx or get_context()
    T = np.asarray(S.T)
    n = _checksquare(T)
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    if n == 0:
        return V
    Z = S.Z if (S.Z is not None and np.asarray(S.Z).size) else None
    flags = 0 if normalize else _capi.GS_RAW
    outR, outL = (None, V) if left else (V, None)
    if np.iscomplexobj(T):
        Tc = _fc(T, np.complex128)
        Zc = _fc(Z, np.complex128) if Z is not None else None
        rc = ctx.lib.gs_eigvecs_c64(ctx.handle, n, _ptr(Tc), _ptr(Zc), _ptr(outR), _ptr(outL), flags)
    else:
        Tr = _fc(T, np.float64)
        Zr = _fc(Z, np.float64) if Z is not None else None
        rc = ctx.lib.gs_eigvecs_f64(ctx.handle, n, _ptr(Tr), _ptr(Zr), _ptr(outR), _ptr(outL), flags)
    if rc != GS_OK:
        _raise(rc, ctx, "geigvecs")
    return V


def eigvecs(S, left=False, ctx=None):
    """LinearAlgebra.eigvecs(S::Schur; left) as pirated by the reference (pirates.jl:38-48)."""
    return geigvecs(S, left=left, ctx=ctx)


def triangularize(S, ctx=None):
    """Real standard-form Schur -> complex triangular Schur (triang.jl:9-43)."""
    ctx = ctx or get_context()
    T = _fc(S.T, np.float64)
    n = _checksquare(T)
    Z = _fc(S.Z, np.float64) if (S.Z is not None and np.asarray(S.Z).size) else None
    Tc = np.zeros((n, n), dtype=np.complex128, order="F")
    Zc = np.zeros((n, n), dtype=np.complex128, order="F") if Z is not None else None
    w = np.zeros(n, dtype=np.complex128)
    rc = ctx.lib.gs_triangularize_f64(ctx.handle, n, _ptr(T), _ptr(Z), _ptr(Tc), _ptr(Zc), _ptr(w), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "triangularize")
    return Schur(Tc, Zc if Zc is not None else np.zeros((0, 0), dtype=np.complex128), w)


Balancer = namedtuple("Balancer", ["ilo", "ihi", "prow_pcol", "D", "trivial"])


def balance_(A, scale=True, permute=True, ctx=None):
    """balance!(A; scale, permute) (balance.jl:33-185) on a Fortran-ordered float64 or
    complex128 array, in place.  Returns (A, Balancer)."""
    ctx = ctx or get_context()
    n = _checksquare(A)
    if not (A.flags.f_contiguous and A.dtype in (np.float64, np.complex128)):
        raise ArgumentError("balance_ needs a Fortran-ordered float64 or complex128 array")
    info = np.zeros(3, dtype=np.int64)
    sp = np.zeros(max(n, 1), dtype=np.int64)
    D = np.ones(max(n, 1))
    flags = (GS_SCALE if scale else 0) | (_capi.GS_BAL_PERMUTE if permute else 0)
    fn = ctx.lib.gs_balance_c64 if A.dtype == np.complex128 else ctx.lib.gs_balance_f64
    rc = fn(ctx.handle, n, _ptr(A), max(n, 1), flags, _ptr(info), _ptr(sp), _ptr(D))
    if rc != GS_OK:
        _raise(rc, ctx, "balance!")
    return A, Balancer(int(info[0]), int(info[1]), sp[:n].copy(), D[:n].copy(), bool(info[2]))


def balance(A, scale=True, permute=True, ctx=None):
    """balance! on a copy of A."""
    A = np.asarray(A)
    dt = np.complex128 if np.iscomplexobj(A) else np.float64
    return balance_(np.array(A, dtype=dt, order="F", copy=True), scale=scale, permute=permute, ctx=ctx)


def _balancer_apply(B, V, inverse, ctx):
    ctx = ctx or get_context()
    V = np.array(V, dtype=np.complex128, order="F", copy=True)
    n, m = V.shape
    info = np.array([B.ilo, B.ihi, int(B.trivial)], dtype=np.int64)
    sp = np.ascontiguousarray(B.prow_pcol, dtype=np.int64)
    D = np.ascontiguousarray(B.D, dtype=np.float64)
    rc = ctx.lib.gs_balancer_apply_c64(ctx.handle, n, m, _ptr(V), max(n, 1), _ptr(info), _ptr(sp), _ptr(D),
                                       int(inverse), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "Balancer")
    return V


def balancer_lmul(B, V, ctx=None):
    """lmul!(B, V): right eigenvectors of the balanced matrix -> of A (balance.jl:189-222)."""
    return _balancer_apply(B, V, False, ctx)


def balancer_ldiv(B, V, ctx=None):
    """ldiv!(B, V): left eigenvectors of the balanced matrix -> of A (balance.jl:226-261)."""
    return _balancer_apply(B, V, True, ctx)


def enormalize(V, ctx=None):
    """_enormalize! (util.jl:572-592) of the columns of V, on the GPU."""
    ctx = ctx or get_context()
    V = np.array(V, dtype=np.complex128, order="F", copy=True)
    n, m = V.shape
    rc = ctx.lib.gs_enormalize_c64(ctx.handle, n, m, _ptr(V), max(n, 1), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "_enormalize!")
    return V


def gordschur(S, select, ctx=None):
    """gordschur!(S, select) / ordschur (ordschur.jl:12-74, rordschur.jl:3-47) on a copy:
    the eigenvalues with select[k] true move to the leading positions, in their order.
    Returns the reordered Schur(T, Z, values).  Raises UnconvergedException if a block
    swap is rejected as ill-conditioned (the reference's IllConditionException).
    A complex GeneralizedSchur goes to gordschur! of the pencil (ordschur.jl:147-305)."""
    ctx = ctx or get_context()
    if isinstance(S, GeneralizedSchur):
        return _ggordschur(S, select, ctx)
    T = np.array(S.T, order="F", copy=True)
    n = _checksquare(T)
    sel = np.ascontiguousarray(np.asarray(select, dtype=bool).astype(np.int32))
    if len(sel) != n:
        raise DimensionMismatch("select must have length %d" % n)
    cplx = np.iscomplexobj(T)
    dt = np.complex128 if cplx else np.float64
    T = np.array(T, dtype=dt, order="F")
    Z = np.array(S.Z if (S.Z is not None and np.asarray(S.Z).size) else np.eye(n), dtype=dt, order="F", copy=True)
    if cplx:
        w = np.zeros(n, dtype=np.complex128)
        rc = ctx.lib.gs_ordschur_c64(ctx.handle, n, _ptr(T), _ptr(Z), _ptr(sel), _ptr(w), 0)
    else:
        wr = np.zeros(n)
        wi = np.zeros(n)
        rc = ctx.lib.gs_ordschur_f64(ctx.handle, n, _ptr(T), _ptr(Z), _ptr(sel), _ptr(wr), _ptr(wi), 0)
        w = wr + 1j * wi
    if rc != GS_OK:
        _raise(rc, ctx, "gordschur!")
    return Schur(T, Z, w)


def _ggordschur_real(G, select, ctx, scale):
    S = _fc(G.S, np.float64)
    T = _fc(G.T, np.float64)
    n = _checksquare(S)
    sel = np.ascontiguousarray(np.asarray(select, dtype=bool).astype(np.int32))
    if len(sel) != n:
        raise DimensionMismatch("select must have length %d" % n)
    Q = _fc(G.Q if G.Q is not None else np.eye(n), np.float64)
    Z = _fc(G.Z if G.Z is not None else np.eye(n), np.float64)
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1))
    rc = ctx.lib.gs_ggordschur_f64(ctx.handle, n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(sel), _ptr(al), _ptr(be),
                                   _capi.GS_SCALE if scale else 0)
    if rc != GS_OK:
        _raise(rc, ctx, "gordschur!(GeneralizedSchur)")
    return GeneralizedSchur(S, T, al[:n], be[:n], Q, Z)


def _ggordschur(G, select, ctx, scale=True):
    if not (np.iscomplexobj(G.S) or np.iscomplexobj(G.T)):
        return _ggordschur_real(G, select, ctx, scale)
    S = _fc(G.S, np.complex128)
    T = _fc(G.T, np.complex128)
    n = _checksquare(S)
    sel = np.ascontiguousarray(np.asarray(select, dtype=bool).astype(np.int32))
    if len(sel) != n:
        raise DimensionMismatch("select must have length %d" % n)
    Q = _fc(G.Q if G.Q is not None else np.eye(n), np.complex128)
    Z = _fc(G.Z if G.Z is not None else np.eye(n), np.complex128)
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1), dtype=np.complex128)
    rc = ctx.lib.gs_ggordschur_c64(ctx.handle, n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(sel), _ptr(al), _ptr(be),
                                   _capi.GS_SCALE if scale else 0)
    if rc != GS_OK:
        _raise(rc, ctx, "gordschur!(GeneralizedSchur)")
    return GeneralizedSchur(S, T, al[:n], be[:n], Q, Z)


ordschur = gordschur


EigenFull = namedtuple("EigenFull", ["values", "vectors", "vectorsl", "rconde", "rcondv"],
                       defaults=(np.zeros(0),))


def _cond_T(S):
    T = S.T if hasattr(S, "T") and not isinstance(S, np.ndarray) else S
    T = np.asarray(T)
    cplx = np.iscomplexobj(T)
    return np.array(T, dtype=np.complex128 if cplx else np.float64, order="F"), cplx


def _gpair(G):
    """S and T of a GeneralizedSchur as complex Fortran arrays.  A real pair runs through the
    complex path: on real triangular data every product, sum, quotient and modulus there has
    a zero imaginary part, so the arithmetic is the reference's real arithmetic."""
    S = np.array(G.S, dtype=np.complex128, order="F")
    T = np.array(G.T, dtype=np.complex128, order="F")
    n = _checksquare(S)
    if T.shape != S.shape:
        raise DimensionMismatch("S and T must have the same size")
    return S, T, n


def eigvalscond(S, nsub, ctx=None):
    """eigvalscond(S, nsub) (ordschur.jl:84-105): reciprocal condition number of the
    leading nsub eigenvalues of the Schur form S (a Schur tuple or its T), from one
    triangular Sylvester solve on the GPU.  Use gordschur to bring the eigenvalues of
    interest to the front first.

    For a GeneralizedSchur (gcondition.jl:121-165) returns (pl, pr), the reciprocal norms of
    the left and right projectors onto the deflating subspaces of the leading nsub block,
    from one generalized Sylvester solve."""
    ctx = ctx or get_context()
    if isinstance(S, GeneralizedSchur):
        Sc, Tc, n = _gpair(S)
        out = np.zeros(2)
        rc = ctx.lib.gs_geigvalscond_c64(ctx.handle, n, _ptr(Sc), max(n, 1), _ptr(Tc), max(n, 1), int(nsub),
                                         _ptr(out), 0)
        if rc != GS_OK:
            _raise(rc, ctx, "eigvalscond")
        return float(out[0]), float(out[1])
    T, cplx = _cond_T(S)
    n = _checksquare(T)
    out = np.zeros(1)
    fn = ctx.lib.gs_eigvalscond_c64 if cplx else ctx.lib.gs_eigvalscond_f64
    rc = fn(ctx.handle, n, _ptr(T), max(n, 1), int(nsub), _ptr(out), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "eigvalscond")
    return float(out[0])


def subspacesep(S, nsub, pnorm=None, ctx=None):
    """subspacesep(S, nsub) (ordschur.jl:107-140): estimated reciprocal condition of the
    invariant subspace of the leading nsub block (the separation of the two diagonal
    blocks, by the one-norm estimator over GPU Sylvester solves).  0 < nsub < n.

    For a GeneralizedSchur (gcondition.jl:169-260) returns [Difu, Difl]: with pnorm "F"
    (the default) the look-ahead estimates of _trgsep, with pnorm 1 the one-norm estimates
    over the generalized Sylvester operator and its adjoint."""
    ctx = ctx or get_context()
    if isinstance(S, GeneralizedSchur):
        if pnorm is None or pnorm in ("F", "Frobenius"):
            pn = 0
        elif pnorm == 1:
            pn = 1
        else:
            raise ArgumentError("pnorm must be :Frobenius or 1")
        Sc, Tc, n = _gpair(S)
        out = np.zeros(2)
        rc = ctx.lib.gs_gsubspacesep_c64(ctx.handle, n, _ptr(Sc), max(n, 1), _ptr(Tc), max(n, 1), int(nsub), pn,
                                         _ptr(out), 0)
        if rc != GS_OK:
            _raise(rc, ctx, "subspacesep")
        return out
    if pnorm is not None:
        raise ArgumentError("subspacesep of a Schur form takes no pnorm")
    T, cplx = _cond_T(S)
    n = _checksquare(T)
    out = np.zeros(1)
    fn = ctx.lib.gs_subspacesep_c64 if cplx else ctx.lib.gs_subspacesep_f64
    rc = fn(ctx.handle, n, _ptr(T), max(n, 1), int(nsub), _ptr(out), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "subspacesep")
    return float(out[0])


def _gtrsyl(A, B, C, D, E, F, adjoint, ctx):
    ctx = ctx or get_context()
    A_, B_, D_, E_ = (np.array(x, dtype=np.complex128, order="F") for x in (A, B, D, E))
    m, n = _checksquare(A_), _checksquare(B_)
    if D_.shape != (m, m) or E_.shape != (n, n):
        raise DimensionMismatch("dimensions of D and E must match A and B")
    R = np.array(C, dtype=np.complex128, order="F")
    L = np.array(F, dtype=np.complex128, order="F")
    if R.shape != (m, n) or L.shape != (m, n):
        raise DimensionMismatch("dimensions of C %s and F %s must match A, (%d,%d), and B, (%d,%d)"
                                % (R.shape, L.shape, m, m, n, n))
    sc = np.ones(1)
    pert = np.zeros(1, dtype=np.int32)
    rc = ctx.lib.gs_gtrsylvester_c64(ctx.handle, m, n, _ptr(A_), max(m, 1), _ptr(B_), max(n, 1), _ptr(R), max(m, 1),
                                     _ptr(D_), max(m, 1), _ptr(E_), max(n, 1), _ptr(L), max(m, 1), int(adjoint),
                                     _ptr(sc), _ptr(pert), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "adjtrsylvester" if adjoint else "trsylvester")
    return R, L, float(sc[0]), bool(pert[0])


def _trsyl(A, B, C, adjoint, possign, ctx):
    ctx = ctx or get_context()
    cplx = any(np.iscomplexobj(x) for x in (A, B, C))
    dt = np.complex128 if cplx else np.float64
    A_, B_ = np.array(A, dtype=dt, order="F"), np.array(B, dtype=dt, order="F")
    m, n = _checksquare(A_), _checksquare(B_)
    X = np.array(C, dtype=dt, order="F")
    if X.ndim == 1:
        X = X.reshape(-1, 1, order="F")
    if X.shape != (m, n):
        raise DimensionMismatch("dimensions of C %s must match A, (%d,%d), and B, (%d,%d)" % (X.shape, m, m, n, n))
    sc = np.ones(1)
    pert = np.zeros(1, dtype=np.int32)
    fn = ctx.lib.gs_trsylvester_c64 if cplx else ctx.lib.gs_trsylvester_f64
    rc = fn(ctx.handle, m, n, _ptr(A_), max(m, 1), _ptr(B_), max(n, 1), _ptr(X), max(m, 1), int(adjoint),
            int(bool(possign)), _ptr(sc), _ptr(pert), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "adjtrsylvester!" if adjoint else "trsylvester!")
    return X, float(sc[0]), bool(pert[0])


def trsylvester(A, B, C, D=None, E=None, F=None, possign=False, ctx=None):
    """trsylvester!(A, B, C; possign) (sylvester.jl:11-75): A X - X B = s C (A X + X B with
    possign) for upper triangular A, B; returns (X, s, perturbed).
    trsylvester!(A, B, C, D, E, F) (gsylvester.jl:23-99): A R - L B = s C, D R - L E = s F for
    complex upper triangular A, D (m x m) and B, E (n x n); returns (R, L, s, perturbed).
    On the GPU; the inputs are not modified."""
    if D is None and E is None and F is None:
        return _trsyl(A, B, C, False, possign, ctx)
    return _gtrsyl(A, B, C, D, E, F, False, ctx)


def adjtrsylvester(A, B, C, D=None, E=None, F=None, possign=False, ctx=None):
    """adjtrsylvester!(A, B, C; possign) (sylvester.jl:80-139): A^H X - X B^H = s C;
    adjtrsylvester!(A, B, C, D, E, F) (gsylvester.jl:103-155): A^H R + D^H L = s C,
    R B^H + L E^H = -s F."""
    if D is None and E is None and F is None:
        return _trsyl(A, B, C, True, possign, ctx)
    return _gtrsyl(A, B, C, D, E, F, True, ctx)


def eigen_rcond(S, want_rconde=True, want_rcondv=True, ctx=None):
    """The per-eigenvalue loop of eigen!(A; jcv = true) (pirates.jl:136-153): for each j,
    eigenvalue j moved to the front of a copy of T by ordschur!, then eigvalscond(., 1)
    and subspacesep(., 1).  Returns (rconde, rcondv) (None for the ones not asked for)."""
    ctx = ctx or get_context()
    T, cplx = _cond_T(S)
    n = _checksquare(T)
    e = np.zeros(n) if want_rconde else None
    v = np.zeros(n) if want_rcondv else None
    fn = ctx.lib.gs_eigen_rcond_c64 if cplx else ctx.lib.gs_eigen_rcond_f64
    rc = fn(ctx.handle, n, _ptr(T), _ptr(e), _ptr(v), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "eigen (jcv)")
    return e, v


def rconde(VL, VR, ctx=None):
    """Reciprocal eigenvalue condition numbers |vl_j^H vr_j| / (|vl_j| |vr_j|)
    (pirates.jl:107-113), on the GPU."""
    ctx = ctx or get_context()
    VL = _fc(VL, np.complex128)
    VR = _fc(VR, np.complex128)
    n = _checksquare(VR)
    out = np.zeros(n)
    rc = ctx.lib.gs_rconde_c64(ctx.handle, n, _ptr(VL), _ptr(VR), _ptr(out), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "rconde")
    return out


# LinearAlgebra.Hermitian(data, uplo) / Symmetric: the triangle `uplo` of data is read.
Hermitian = namedtuple("Hermitian", ["data", "uplo"], defaults=("U",))
# LinearAlgebra.SymTridiagonal(dv, ev)
SymTridiagonal = namedtuple("SymTridiagonal", ["dv", "ev"])
# hessenberg!(Hermitian(A, uplo)): the tridiagonal and the reflectors (hessenberg.jl:26-96)
HermitianHessenberg = namedtuple("HermitianHessenberg", ["factors", "tau", "dv", "ev", "uplo"])


_ALGS = {"QRIteration": "QR", "QR": "QR", "DivideAndConquer": "DC", "DC": "DC"}


def _alg(alg):
    """QRIteration() (the default) or DivideAndConquer() (GenericSchur.jl:119-136);
    RobustRepresentations falls back to QRIteration with a warning (symtridiag.jl:12-26)."""
    if alg is None:
        return "QR"
    name = alg if isinstance(alg, str) else type(alg).__name__
    if name == "RobustRepresentations":
        import warnings
        warnings.warn("GenericSchur does not currently provide alg=RobustRepresentations (LinearAlgebra "
                      "default); falling back to QRIteration.")
        return "QR"
    if name not in _ALGS:
        raise ArgumentError("Unsupported algorithm %s" % (name,))
    return _ALGS[name]


def _heev(H, wantv, ctx, alg=None):
    ctx = ctx or get_context()
    A = np.asarray(H.data)
    n = _checksquare(A)
    cplx = np.iscomplexobj(A)
    dt = np.complex128 if cplx else np.float64
    A = np.array(A, dtype=dt, order="F")
    w = np.zeros(max(n, 1))
    V = np.zeros((n, n), dtype=dt, order="F") if wantv else None
    fn = ctx.lib.gs_heev_c64 if cplx else ctx.lib.gs_heev_f64
    uplo = str(H.uplo).upper()[:1]
    flags = (_capi.GS_WANTZ if wantv else 0) | (_capi.GS_DC if _alg(alg) == "DC" else 0)
    rc = fn(ctx.handle, n, _ptr(A), max(n, 1), ord(uplo), _ptr(w), _ptr(V), max(n, 1), flags)
    if rc != GS_OK:
        _raise(rc, ctx, "geigen!")
    return w[:n], V


def _sorted(w, V, sortby):
    if sortby == "default" or sortby is None:
        return w, V
    p = np.argsort([sortby(x) for x in w], kind="stable")
    return w[p], (V[:, p] if V is not None else None)


def geigen(H, alg=None, sortby="default", ctx=None):
    """geigen!(Hermitian(A, uplo), alg) (GenericSchur.jl:126-136) and geigen!(::SymTridiagonal,
    alg) (symtridiag.jl:43-49) on the GPU: Eigen(values ascending, orthonormal vectors).
    alg: "QRIteration" (default) or "DivideAndConquer" (symtri_dc.jl)."""
    if isinstance(H, SymTridiagonal):
        w, V = _st_eig(H, True, sortby, ctx, alg)
        return Eigen(w, V)
    w, V = _heev(H, True, ctx, alg)
    w, V = _sorted(w, V, sortby)
    return Eigen(w, V)


def geigvals(H, alg=None, sortby="default", ctx=None):
    """geigvals!(Hermitian(A, uplo), alg) (GenericSchur.jl:138-146)."""
    if isinstance(H, SymTridiagonal):
        return _st_eig(H, False, sortby, ctx, alg)[0]
    w, _ = _heev(H, False, ctx, alg)
    return _sorted(w, None, sortby)[0]


def gschur_symtridiag(T, Z=None, alg=None, ctx=None):
    """_gschur!(SymTridiagonal(dv, ev), alg, Z): with QRIteration (symtridiag.jl:79-183) or
    DivideAndConquer (symtri_dc.jl:6-104); the eigenvalues in the algorithm's order, Z
    multiplied from the right by the eigenvectors (when given).  Returns (d, e, Z)."""
    ctx = ctx or get_context()
    d = np.array(T.dv, dtype=np.float64)
    n = len(d)
    e = np.zeros(max(n - 1, 1))
    e[:max(n - 1, 0)] = np.asarray(T.ev, dtype=np.float64)[:max(n - 1, 0)]
    Zc = np.array(Z, dtype=np.float64, order="F", copy=True) if Z is not None else None
    fn = ctx.lib.gs_stedc_f64 if _alg(alg) == "DC" else ctx.lib.gs_steqr_f64
    rc = fn(ctx.handle, n, _ptr(d), _ptr(e), _ptr(Zc), max(n, 1), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "_gschur!(SymTridiagonal)")
    return d, e[:max(n - 1, 0)], Zc


def _st_eig(T, wantv, sortby, ctx, alg=None):
    n = len(T.dv)
    d, _, Z = gschur_symtridiag(T, np.eye(n) if wantv else None, alg=alg, ctx=ctx)
    p = np.argsort(d, kind="stable") if sortby == "default" else \
        (np.arange(n) if sortby is None else np.argsort([sortby(x) for x in d], kind="stable"))
    return d[p], (Z[:, p] if wantv else None)


def hessenberg_hermitian(H, ctx=None):
    """hessenberg!(Hermitian(A, uplo)) (pirates.jl:236-238 -> hessenberg.jl:26-96) on a
    copy: HermitianHessenberg(factors, tau, dv, ev, uplo)."""
    ctx = ctx or get_context()
    A = np.asarray(H.data)
    n = _checksquare(A)
    cplx = np.iscomplexobj(A)
    dt = np.complex128 if cplx else np.float64
    A = np.array(A, dtype=dt, order="F", copy=True)
    d = np.zeros(max(n, 1))
    e = np.zeros(max(n - 1, 1))
    tau = np.zeros(max(n - 1, 1), dtype=dt)
    uplo = str(H.uplo).upper()[:1]
    fn = ctx.lib.gs_hetrd_c64 if cplx else ctx.lib.gs_hetrd_f64
    rc = fn(ctx.handle, n, _ptr(A), max(n, 1), ord(uplo), _ptr(d), _ptr(e), _ptr(tau), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "hessenberg!(Hermitian)")
    return HermitianHessenberg(A, tau[:max(n - 1, 0)], d[:n], e[:max(n - 1, 0)], uplo)


def eigen(A, permute=True, scale=True, sortby="default", jvr=True, jvl=False, jce=False, jcv=False, ctx=None,
          alg=None):
    """Eigen decomposition (pirates.jl:63-160): balance! (permute/scale, as the reference's
    defaults), Schur form, triangularize for real input, right eigenvectors (and left
    ones with jvl or jce), the Balancer's lmul!/ldiv!, _enormalize!, sort.  With jce the
    reciprocal eigenvalue condition numbers are computed from the balanced form's
    vectors, as the reference does.  With jcv, every eigenvalue is moved to the front of
    a copy of the Schur form and its subspacesep (and, with jce as well, its
    eigvalscond, which then replaces the vector-based value) is computed, as the
    reference's (expensive) loop does.  Returns Eigen(values, vectors), or, when jvl, jce
    or jcv is asked for, EigenFull(values, vectors, vectorsl, rconde, rcondv).
    For a Hermitian or SymTridiagonal argument, geigen! with alg (QRIteration by default,
    or DivideAndConquer; pirates.jl:162-184)."""
    if isinstance(A, (Hermitian, SymTridiagonal)):
        # eigen!(::Hermitian; alg) / eigen!(::SymTridiagonal; alg) (pirates.jl:162-184)
        return geigen(A, alg=alg, sortby=sortby, ctx=ctx)
    if alg is not None:
        raise ArgumentError("alg applies to Hermitian and SymTridiagonal arguments")
    A = np.asarray(A)
    B = None
    if permute or scale:
        A, B = balance(A, scale=scale, permute=permute, ctx=ctx)
    S = gschur(A, ctx=ctx)
    if not np.iscomplexobj(S.T):
        S = triangularize(S, ctx=ctx)
    full = jvl or jce or jcv
    w = S.values
    if not full:
        if B is not None:
            V = geigvecs(S, normalize=False, ctx=ctx)
            V = balancer_lmul(B, V, ctx=ctx)
            V = enormalize(V, ctx=ctx)
        else:
            V = geigvecs(S, ctx=ctx)
        if sortby is None:
            return Eigen(w, V)
        p = _eigsortby(w) if sortby == "default" else np.argsort([sortby(x) for x in w], kind="stable")
        return Eigen(w[p], V[:, p])
    n = S.T.shape[0]
    V = geigvecs(S, normalize=False, ctx=ctx) if (jvr or jce) else np.zeros((0, 0), dtype=np.complex128)
    VL = geigvecs(S, left=True, normalize=False, ctx=ctx)
    rce = rconde(VL, V, ctx=ctx) if jce else np.zeros(0)
    if jvr:
        if B is not None:
            V = balancer_lmul(B, V, ctx=ctx)
        V = enormalize(V, ctx=ctx)
    else:
        V = np.zeros((0, 0), dtype=np.complex128)
    if jvl:
        if B is not None:
            VL = balancer_ldiv(B, VL, ctx=ctx)
        VL = enormalize(VL, ctx=ctx)
    else:
        VL = np.zeros((0, 0), dtype=np.complex128)
    rcv = np.zeros(0)
    if jcv:
        e_j, rcv = eigen_rcond(S, want_rconde=jce, want_rcondv=True, ctx=ctx)
        if jce:
            rce = e_j
    if sortby is None:
        return EigenFull(w, V, VL, rce, rcv)
    p = _eigsortby(w) if sortby == "default" else np.argsort([sortby(x) for x in w], kind="stable")
    return EigenFull(w[p], V[:, p] if V.size else V, VL[:, p] if VL.size else VL, rce[p] if rce.size else rce,
                     rcv[p] if rcv.size else rcv)


def geigvecs_batched(T_packed, Z_packed, ns, offs, woffs=None, left=False, normalize=True, ctx=None):
    """Eigenvectors for a packed batch of Schur pairs (orders <= 128).  Returns the
    packed complex eigenvector matrices."""
    ctx = ctx or get_context()
    ns = np.ascontiguousarray(ns, dtype=np.int32)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    count = len(ns)
    plen = len(T_packed)
    V = np.zeros(plen, dtype=np.complex128)
    outR, outL = (None, V) if left else (V, None)
    flags = 0 if normalize else _capi.GS_RAW
    if np.iscomplexobj(T_packed):
        T = np.ascontiguousarray(T_packed, dtype=np.complex128)
        Z = np.ascontiguousarray(Z_packed, dtype=np.complex128) if Z_packed is not None else None
        rc = ctx.lib.gs_eigvecs_batched_c64(ctx.handle, count, _ptr(ns), _ptr(offs), plen, _ptr(T), _ptr(Z), _ptr(outR),
                                            _ptr(outL), flags)
    else:
        if woffs is None:
            woffs = np.zeros(count, dtype=np.int64)
            woffs[1:] = np.cumsum(ns.astype(np.int64))[:-1]
        woffs = np.ascontiguousarray(woffs, dtype=np.int64)
        wlen = int((woffs + ns).max()) if count else 0
        T = np.ascontiguousarray(T_packed, dtype=np.float64)
        Z = np.ascontiguousarray(Z_packed, dtype=np.float64) if Z_packed is not None else None
        rc = ctx.lib.gs_eigvecs_batched_f64(ctx.handle, count, _ptr(ns), _ptr(offs), _ptr(woffs), plen, wlen, _ptr(T),
                                            _ptr(Z), _ptr(outR), _ptr(outL), flags)
    if rc != GS_OK:
        _raise(rc, ctx, "geigvecs_batched")
    return V


def eig_adjoint_batched(T_packed, Z_packed, ns, offs, woffs, gbar, ctx=None):
    """Reverse-mode rule of A -> eigenvalues(A) for a packed batch of complex Schur
    pairs: returns grad = dL/dRe(A) + i dL/dIm(A) (packed like T) given the
    cotangents gbar = dL/dRe(l) + i dL/dIm(l) of the eigenvalues, ordered like
    S.values.  Eigenvectors are recomputed on the GPU from (T, Z)."""
    ctx = ctx or get_context()
    ns = np.ascontiguousarray(ns, dtype=np.int32)
    offs = np.ascontiguousarray(offs, dtype=np.int64)
    woffs = np.ascontiguousarray(woffs, dtype=np.int64)
    T = np.ascontiguousarray(T_packed, dtype=np.complex128)
    Z = np.ascontiguousarray(Z_packed, dtype=np.complex128)
    g = np.ascontiguousarray(gbar, dtype=np.complex128)
    count = len(ns)
    G = np.zeros(len(T), dtype=np.complex128)
    wlen = int((woffs + ns).max()) if count else 0
    rc = ctx.lib.gs_eig_adjoint_batched_c64(ctx.handle, count, _ptr(ns), _ptr(offs), _ptr(woffs), len(T), wlen,
                                            _ptr(T), _ptr(Z), _ptr(g), _ptr(G), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "eig_adjoint_batched")
    return G


def hessenberg(A, ctx=None):
    """Householder Hessenberg reduction (hessenberg.jl:3-17) and Q (hessenberg.jl:150-166).
    Returns (Hpacked, tau, Q): Hpacked holds H on and above the first subdiagonal and
    the reflectors below it, as the reference's Hessenberg object stores them."""
    ctx = ctx or get_context()
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    n = _checksquare(A)
    tau = np.zeros(max(n - 1, 1))
    Q = np.zeros((n, n), order="F")
    rc = ctx.lib.gs_hessenberg_f64(ctx.handle, n, _ptr(A), max(n, 1), _ptr(tau), _ptr(Q), max(n, 1), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "hessenberg")
    return A, tau[:max(n - 1, 0)], Q


def gemm_f64_tc(A, B, transA=False, ctx=None):
    """FP64 product op(A) @ B on the BF16 tensor cores by exact splitting (the product the
    mixed-precision refinement uses for Z^T A Z and Z^T Z).  No counterpart in the
    reference; accuracy at least that of an FP64 GEMM relative to the row maxima of op(A)
    and column maxima of B."""
    ctx = ctx or get_context()
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    if A.ndim != 2 or B.ndim != 2:
        raise DimensionMismatch("gemm_f64_tc: matrices expected")
    m, q = (A.shape[1], A.shape[0]) if transA else A.shape
    if B.shape[0] != q:
        raise DimensionMismatch("gemm_f64_tc: inner dimensions %d and %d" % (q, B.shape[0]))
    p = B.shape[1]
    C = np.zeros((m, p), order="F")
    rc = ctx.lib.gs_gemm_f64_tc(ctx.handle, m, p, q, _ptr(A), max(A.shape[0], 1), 1 if transA else 0, _ptr(B),
                                max(q, 1), _ptr(C), max(m, 1), 0)
    if rc != GS_OK:
        _raise(rc, ctx, "gemm_f64_tc")
    return C


def gschur_mixed(A, scale=True, maxiter=None, ctx=None, return_info=False, fallback=True):
    """Real Schur decomposition computed in FP32 on the GPU and refined to FP64
    accuracy (Newton refinement of the Schur pair).  Same outputs as gschur.
    When FP32 does not separate the eigenvalues well enough for the refinement, the
    decomposition is recomputed in FP64 (info["iterations"] == -1); with
    fallback=False an UnconvergedException is raised instead."""
    ctx = ctx or get_context()
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    n = _checksquare(A)
    Z = np.zeros((n, n), order="F")
    wr = np.zeros(n)
    wi = np.zeros(n)
    info = np.zeros(4)
    flags = GS_WANTZ | (GS_SCALE if scale else 0) | (0 if fallback else _capi.GS_NOFALLBACK)
    rc = ctx.lib.gs_schur_mixed_f64(ctx.handle, n, _ptr(A), max(n, 1), _ptr(Z), max(n, 1), _ptr(wr), _ptr(wi), flags,
                                    int(maxiter or 0), _ptr(info))
    if rc != GS_OK:
        _raise(rc, ctx, "gschur_mixed")
    S = Schur(A, Z, wr + 1j * wi)
    if return_info:
        return S, {"iterations": int(info[0]), "residual": float(info[1]), "fp32_ms": float(info[2]),
                   "refine_ms": float(info[3])}
    return S
