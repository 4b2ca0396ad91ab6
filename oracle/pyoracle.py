"""numpy front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the shipped library never does.  Matrices are numpy arrays in Fortran
(column-major) order, like Julia's.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_i = ctypes.c_int
_ll = ctypes.c_longlong
_p = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        sig = {
            "or_gschur_d": [_i, _p, _i, _p, _i, _p, _p, _i, _i, _ll],
            "or_gschur_s": [_i, _p, _i, _p, _i, _p, _p, _i, _i, _ll],
            "or_gschur_z": [_i, _p, _i, _p, _i, _p, _i, _i, _ll, _ll],
            "or_gschur_hess_z": [_i, _p, _i, _p, _i, _p, _ll],
            "or_gschur_hess_d": [_i, _p, _i, _p, _i, _p, _p, _ll],
            "or_hessenberg_d": [_i, _p, _i, _p, _p, _i],
            "or_hessenberg_z": [_i, _p, _i, _p, _p, _i],
            "or_gschur_q": [_i, _p, _p, _p, _p, _p, _p],
            "or_gschur_zq": [_i, _p, _p, _p, _p, _p],
            "or_eigvecs_d": [_i, _p, _p, _p, _i, _i],
            "or_eigvecs_z": [_i, _p, _p, _p, _i, _i],
            "or_triangularize_d": [_i, _p, _p, _p, _p, _p],
            "or_gs2x2_d": [_p, _p, _p, _p],
            "or_reflector_d": [_p, _i, _p],
            "or_gschur_batched_d": [_i, _p, _p, _p, _p, _p, _p, _p, _p, _i],
            "or_gschur_batched_z": [_i, _p, _p, _p, _p, _p, _p, _p, _i],
            "or_balance_d": [_i, _p, _i, _i, _i, _p, _p, _p],
            "or_balance_z": [_i, _p, _i, _i, _i, _p, _p, _p],
            "or_balancer_apply_z": [_i, _i, _p, _i, _i, _i, _p, _p, _i, _i],
            "or_trsylv_d": [_i, _i, _i, _p, _i, _p, _i, _p, _i, _p],
            "or_trsylv_z": [_i, _i, _i, _p, _i, _p, _i, _p, _i, _p],
            "or_econd_d": [_i, _p, _i, _i, _p],
            "or_econd_z": [_i, _p, _i, _i, _p],
            "or_heev_d": [_i, _p, _i, _i, _i, _p, _p],
            "or_heev_z": [_i, _p, _i, _i, _i, _p, _p],
            "or_hetrd_d": [_i, _p, _i, _i, _p, _p, _p],
            "or_hetrd_z": [_i, _p, _i, _i, _p, _p, _p],
            "or_steqr_d": [_i, _p, _p, _p, _i],
            "or_stedc_d": [_i, _p, _p, _p, _i],
            "or_ggschur_z": [_i, _p, _p, _p, _p, _p, _p, _i],
            "or_ggevc_z": [_i, _p, _p, _p, _p, _i],
            "or_ggschur_d": [_i, _p, _p, _p, _p, _p, _p, _p, _i],
            "or_rgevc_d": [_i, _p, _p, _p, _p, _i],
            "or_ggordschur_z": [_i, _p, _p, _p, _p, _p, _i, _p, _p],
            "or_gtrsyl_z": [_i, _i, _p, _p, _p, _p, _p, _p, _i],
            "or_ggordschur_d": [_i, _p, _p, _p, _p, _p, _i, _p, _p],
            "or_gcond_z": [_i, _p, _p, _i, _p, _i],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _i
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f(a, dtype):
    return np.array(a, dtype=dtype, order="F", copy=True)


class Unconverged(RuntimeError):
    pass


def gschur_real(A, wantZ=True, scale=True, maxiter=0, dtype=np.float64):
    """Real Schur form (GenericSchur.jl:805-835).  Returns (T, Z, w)."""
    A = _f(A, dtype)
    n = A.shape[0]
    Z = np.zeros((n, n), dtype=dtype, order="F")
    wr = np.zeros(n, dtype=dtype)
    wi = np.zeros(n, dtype=dtype)
    fn = lib().or_gschur_d if dtype == np.float64 else lib().or_gschur_s
    st = fn(n, _ptr(A), max(n, 1), _ptr(Z), max(n, 1), _ptr(wr), _ptr(wi), int(wantZ), int(scale), maxiter)
    if st == 1:
        raise Unconverged("iteration limit reached")
    return A, (Z if wantZ else None), wr + 1j * wi


def gschur_cplx(A, wantZ=True, scale=True, maxiter=0, maxinner=0):
    """Complex Schur form (GenericSchur.jl:350-372).  Returns (T, Z, w)."""
    A = _f(A, np.complex128)
    n = A.shape[0]
    Z = np.zeros((n, n), dtype=np.complex128, order="F")
    w = np.zeros(n, dtype=np.complex128)
    st = lib().or_gschur_z(n, _ptr(A), max(n, 1), _ptr(Z), max(n, 1), _ptr(w), int(wantZ), int(scale),
                           maxiter, maxinner)
    if st == 1:
        raise Unconverged("iteration limit reached")
    return A, (Z if wantZ else None), w


def gschur(A, **kw):
    if np.iscomplexobj(A):
        return gschur_cplx(A, **kw)
    return gschur_real(A, **kw)


def gschur_hess_cplx(H, Z=None, maxiter=0):
    """Complex Hessenberg QR with the subdiagonal check (GenericSchur.jl:194-335)."""
    H = _f(H, np.complex128)
    n = H.shape[0]
    Zc = None if Z is None else _f(Z, np.complex128)
    w = np.zeros(n, dtype=np.complex128)
    st = lib().or_gschur_hess_z(n, _ptr(H), n, _ptr(Zc), n, _ptr(w), maxiter)
    return st, H, Zc, w


def hessenberg(A):
    """Hessenberg reduction and Q (hessenberg.jl:3-17, 150-166).  Returns (Hfull, tau, Q)."""
    cplx = np.iscomplexobj(A)
    dt = np.complex128 if cplx else np.float64
    A = _f(A, dt)
    n = A.shape[0]
    tau = np.zeros(max(n - 1, 1), dtype=dt)
    Q = np.zeros((n, n), dtype=dt, order="F")
    fn = lib().or_hessenberg_z if cplx else lib().or_hessenberg_d
    fn(n, _ptr(A), n, _ptr(tau), _ptr(Q), n)
    return A, tau[: max(n - 1, 0)], Q


def gschur_quad(A):
    """Real Schur in 113-bit arithmetic.  Returns (T, Z, w, (backward_err, orth_err))."""
    A = _f(A, np.float64)
    n = A.shape[0]
    T = np.zeros((n, n), order="F")
    Z = np.zeros((n, n), order="F")
    wr = np.zeros(n)
    wi = np.zeros(n)
    res = np.zeros(2)
    st = lib().or_gschur_q(n, _ptr(A), _ptr(T), _ptr(Z), _ptr(wr), _ptr(wi), _ptr(res))
    if st:
        raise Unconverged("iteration limit reached")
    return T, Z, wr + 1j * wi, tuple(res)


def gschur_cplx_quad(A):
    A = _f(A, np.complex128)
    n = A.shape[0]
    T = np.zeros((n, n), dtype=np.complex128, order="F")
    Z = np.zeros((n, n), dtype=np.complex128, order="F")
    w = np.zeros(n, dtype=np.complex128)
    res = np.zeros(2)
    st = lib().or_gschur_zq(n, _ptr(A), _ptr(T), _ptr(Z), _ptr(w), _ptr(res))
    if st:
        raise Unconverged("iteration limit reached")
    return T, Z, w, tuple(res)


_mplib = None


def mplib():
    """The 256-bit MPFR instance (oracle/_build/liboracle_mpfr.so), built on demand."""
    global _mplib
    if _mplib is None:
        path = _build.build_mpfr()
        if path is None:
            raise OSError("the 256-bit oracle needs libmpfr.so.6")
        _mplib = ctypes.CDLL(path)
        for name in ("or_gschur_mp", "or_gschur_zmp"):
            getattr(_mplib, name).restype = ctypes.c_int
    return _mplib


def gschur_mp(A):
    """Real Schur in 256-bit arithmetic (BigFloat precision).  Returns (T, Z, w,
    (backward_err, orth_err)) with T, Z, w rounded to FP64."""
    A = _f(A, np.float64)
    n = A.shape[0]
    T = np.zeros((n, n), order="F")
    Z = np.zeros((n, n), order="F")
    wr = np.zeros(n)
    wi = np.zeros(n)
    res = np.zeros(2)
    st = mplib().or_gschur_mp(ctypes.c_int(n), _ptr(A), _ptr(T), _ptr(Z), _ptr(wr), _ptr(wi), _ptr(res))
    if st:
        raise Unconverged("iteration limit reached")
    return T, Z, wr + 1j * wi, tuple(res)


def gschur_cplx_mp(A):
    """Complex Schur in 256-bit arithmetic (BigFloat precision)."""
    A = _f(A, np.complex128)
    n = A.shape[0]
    T = np.zeros((n, n), dtype=np.complex128, order="F")
    Z = np.zeros((n, n), dtype=np.complex128, order="F")
    w = np.zeros(n, dtype=np.complex128)
    res = np.zeros(2)
    st = mplib().or_gschur_zmp(ctypes.c_int(n), _ptr(A), _ptr(T), _ptr(Z), _ptr(w), _ptr(res))
    if st:
        raise Unconverged("iteration limit reached")
    return T, Z, w, tuple(res)


def eigvecs(T, Z, left=False, normalize=True):
    """Eigenvectors from a Schur pair (vectors.jl:12-20 -> _geigvecs!/_gleigvecs!)."""
    n = T.shape[0]
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    if np.iscomplexobj(T):
        lib().or_eigvecs_z(n, _ptr(_f(T, np.complex128)), _ptr(_f(Z, np.complex128)), _ptr(V), int(left),
                           int(normalize))
    else:
        lib().or_eigvecs_d(n, _ptr(_f(T, np.float64)), _ptr(_f(Z, np.float64)), _ptr(V), int(left),
                           int(normalize))
    return V


def triangularize(T, Z):
    """Real standard-form Schur -> complex triangular Schur (triang.jl:9-43)."""
    n = T.shape[0]
    Tc = np.zeros((n, n), dtype=np.complex128, order="F")
    Zc = np.zeros((n, n), dtype=np.complex128, order="F")
    w = np.zeros(n, dtype=np.complex128)
    lib().or_triangularize_d(n, _ptr(_f(T, np.float64)), _ptr(_f(Z, np.float64)), _ptr(Tc), _ptr(Zc), _ptr(w))
    return Tc, Zc, w


def gs2x2(B):
    """_gs2x2! (GenericSchur.jl:716-803) on a 2x2 block; returns (std block, cs, sn, w1, w2)."""
    h = np.array([B[0, 0], B[0, 1], B[1, 0], B[1, 1]], dtype=np.float64)
    cs = np.zeros(1)
    sn = np.zeros(1)
    w = np.zeros(4)
    lib().or_gs2x2_d(_ptr(h), _ptr(cs), _ptr(sn), _ptr(w))
    return np.array([[h[0], h[1]], [h[2], h[3]]]), cs[0], sn[0], w[0] + 1j * w[1], w[2] + 1j * w[3]


def gschur_batched_real(mats, nthreads=1):
    """Reference algorithm over a list of real matrices, OpenMP over the batch."""
    ns = np.array([m.shape[0] for m in mats], dtype=np.int32)
    offs = np.zeros(len(mats), dtype=np.int64)
    offs[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
    woffs = np.zeros(len(mats), dtype=np.int64)
    woffs[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    a = np.concatenate([np.asarray(m, dtype=np.float64).ravel(order="F") for m in mats])
    z = np.zeros_like(a)
    wr = np.zeros(int(ns.sum()))
    wi = np.zeros_like(wr)
    st = np.zeros(len(mats), dtype=np.int32)
    lib().or_gschur_batched_d(len(mats), _ptr(offs), _ptr(ns), _ptr(a), _ptr(z), _ptr(wr), _ptr(wi), _ptr(woffs),
                              _ptr(st), nthreads)
    return a, z, wr, wi, st, offs, woffs


def gschur_batched_packed_real(count, offs, ns, a, z, wr, wi, woffs, status, nthreads):
    """Same as gschur_batched_real on caller-owned packed buffers (no copies)."""
    return lib().or_gschur_batched_d(count, _ptr(offs), _ptr(ns), _ptr(a), _ptr(z), _ptr(wr), _ptr(wi),
                                     _ptr(woffs), _ptr(status), nthreads)


def gschur_batched_packed_cplx(count, offs, ns, a, z, w, woffs, status, nthreads):
    return lib().or_gschur_batched_z(count, _ptr(offs), _ptr(ns), _ptr(a), _ptr(z), _ptr(w), _ptr(woffs),
                                     _ptr(status), nthreads)


def balance(A, scale=True, permute=True):
    """balance!(A; scale, permute) (balance.jl:33-185).  Returns (Abal, (ilo, ihi, sp, D,
    trivial)) with sp the 1-based permutation record and D the scale factors."""
    cplx = np.iscomplexobj(A)
    A = _f(A, np.complex128 if cplx else np.float64)
    n = A.shape[0]
    out = np.zeros(3, dtype=np.int32)
    sp = np.zeros(max(n, 1), dtype=np.int32)
    D = np.ones(max(n, 1))
    fn = lib().or_balance_z if cplx else lib().or_balance_d
    rc = fn(n, _ptr(A), max(n, 1), int(scale), int(permute), _ptr(out), _ptr(sp), _ptr(D))
    if rc:
        raise ValueError("NaN encountered while balancing")
    return A, (int(out[0]), int(out[1]), sp[:n].copy(), D[:n].copy(), bool(out[2]))


def balancer_apply(V, B, inverse=False):
    """lmul!(B, V) (right eigenvectors) or ldiv!(B, V) (left eigenvectors) on complex V."""
    ilo, ihi, sp, D, trivial = B
    V = _f(V, np.complex128)
    n, m = V.shape
    lib().or_balancer_apply_z(n, m, _ptr(V), max(n, 1), ilo, ihi, _ptr(np.ascontiguousarray(sp, dtype=np.int32)),
                              _ptr(np.ascontiguousarray(D, dtype=np.float64)), int(trivial), int(inverse))
    return V


def trsylvester(A, B, C, adjoint=False, possign=False):
    """trsylvester!(A, B, C; possign) (A X -+ X B = scale C) or adjtrsylvester!(A, B, C;
    possign) (A^H X -+ X B^H = scale C), sylvester.jl:11-139.  Returns (X, scale, perturbed)."""
    cplx = np.iscomplexobj(A) or np.iscomplexobj(B) or np.iscomplexobj(C)
    dt = np.complex128 if cplx else np.float64
    A, B, X = _f(A, dt), _f(B, dt), _f(C, dt)
    m, p = X.shape
    out = np.zeros(2)
    fn = lib().or_trsylv_z if cplx else lib().or_trsylv_d
    fn(int(adjoint) | (2 if possign else 0), m, p, _ptr(A), max(m, 1), _ptr(B), max(p, 1), _ptr(X), max(m, 1),
       _ptr(out))
    return X, float(out[0]), bool(out[1])


def condition(T, nsub):
    """(eigvalscond(S, nsub), subspacesep(S, nsub)) of the Schur factor T
    (ordschur.jl:84-140)."""
    cplx = np.iscomplexobj(T)
    T = _f(T, np.complex128 if cplx else np.float64)
    n = T.shape[0]
    out = np.zeros(2)
    fn = lib().or_econd_z if cplx else lib().or_econd_d
    fn(n, _ptr(T), max(n, 1), int(nsub), _ptr(out))
    return float(out[0]), float(out[1])


def heev(A, uplo="U", wantv=True):
    """geigen!(Hermitian(A, uplo)) / geigvals! (GenericSchur.jl:126-146) with the default
    QRIteration: (w ascending, V or None, status)."""
    cplx = np.iscomplexobj(A)
    dt = np.complex128 if cplx else np.float64
    A = _f(A, dt)
    n = A.shape[0]
    w = np.zeros(max(n, 1))
    V = np.zeros((n, n), dtype=dt, order="F") if wantv else None
    fn = lib().or_heev_z if cplx else lib().or_heev_d
    st = fn(n, _ptr(A), max(n, 1), int(uplo == "U"), int(wantv), _ptr(w), _ptr(V))
    return w[:n], V, st


def hetrd(A, uplo="L"):
    """_hehessenberg!(Hermitian(A, uplo)) (hessenberg.jl:26-96): (d, e, tau, factors)."""
    cplx = np.iscomplexobj(A)
    dt = np.complex128 if cplx else np.float64
    A = _f(A, dt)
    n = A.shape[0]
    d = np.zeros(max(n, 1))
    e = np.zeros(max(n - 1, 1))
    tau = np.zeros(max(n - 1, 1), dtype=dt)
    fn = lib().or_hetrd_z if cplx else lib().or_hetrd_d
    fn(n, _ptr(A), max(n, 1), int(uplo == "U"), _ptr(d), _ptr(e), _ptr(tau))
    return d[:n], e[:max(n - 1, 0)], tau[:max(n - 1, 0)], A


def steqr(d, e, wantz=True):
    """_gschur!(SymTridiagonal(d, e), QRIteration(), Z = I) (symtridiag.jl:79-183):
    (eigenvalues in the iteration's order, Z, status)."""
    d = np.array(d, dtype=np.float64)
    n = len(d)
    e = np.array(np.concatenate([e, [0.0]]) if n else [0.0], dtype=np.float64)
    Z = np.asfortranarray(np.eye(n)) if wantz else None
    st = lib().or_steqr_d(n, _ptr(d), _ptr(e), _ptr(Z), int(wantz))
    return d, Z, st


def stedc(d, e, Z=None, wantz=True):
    """_gschur!(SymTridiagonal(d, e), DivideAndConquer(), Z) (symtri_dc.jl:6-104): the
    eigenvalues in the algorithm's order, Z times the eigenvectors (Z = I when not given),
    and the status (1: a secular equation did not converge)."""
    d = np.array(d, dtype=np.float64)
    e = np.array(e, dtype=np.float64)
    n = d.shape[0]
    if Z is None:
        Z = np.eye(n, order="F")
    else:
        Z = np.array(Z, dtype=np.float64, order="F")
    ee = np.zeros(max(n, 1))
    ee[:max(n - 1, 0)] = e[:max(n - 1, 0)]
    st = lib().or_stedc_d(n, _ptr(d), _ptr(ee), _ptr(Z), int(wantz))
    return d, (Z if wantz else None), st


def ggschur(A, B, scale=True):
    """ggschur!(A, B) for a complex pencil (generalized.jl:21-80): (S, T, alpha, beta, Q, Z,
    status)."""
    S = _f(A, np.complex128)
    T = _f(B, np.complex128)
    n = S.shape[0]
    Q = np.zeros((n, n), dtype=np.complex128, order="F")
    Z = np.zeros((n, n), dtype=np.complex128, order="F")
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1), dtype=np.complex128)
    st = lib().or_ggschur_z(n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(al), _ptr(be), int(scale))
    return S, T, al[:n], be[:n], Q, Z, st


def ggeigvecs(S, T, X=None, left=False):
    """Eigenvectors of a complex generalized Schur pair (vectors.jl:723-1038): right
    (back-transformed by X = Z) or left (X = Q); columns scaled to max |re|+|im| = 1."""
    Sf = _f(S, np.complex128)
    Tf = _f(T, np.complex128)
    n = Sf.shape[0]
    Xf = _f(X, np.complex128) if X is not None else None
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    lib().or_ggevc_z(n, _ptr(Sf), _ptr(Tf), _ptr(Xf), _ptr(V), int(left))
    return V


def ggschur_real(A, B, scale=True):
    """ggschur!(A, B) for a real pencil (rgeneralized.jl:10-66): (S quasi-triangular, T,
    alpha (complex), beta (real), Q, Z, status)."""
    S = _f(A, np.float64)
    T = _f(B, np.float64)
    n = S.shape[0]
    Q = np.zeros((n, n), order="F")
    Z = np.zeros((n, n), order="F")
    alr = np.zeros(max(n, 1))
    ali = np.zeros(max(n, 1))
    be = np.zeros(max(n, 1))
    st = lib().or_ggschur_d(n, _ptr(S), _ptr(T), _ptr(Q), _ptr(Z), _ptr(alr), _ptr(ali), _ptr(be), int(scale))
    return S, T, (alr + 1j * ali)[:n], be[:n], Q, Z, st


def rgeigvecs(S, T, X=None, left=False):
    """Eigenvectors of a real generalized Schur pair (vectors.jl:1040-1513), complex
    columns (a complex pair's second column is the conjugate of the first)."""
    Sf = _f(S, np.float64)
    Tf = _f(T, np.float64)
    n = Sf.shape[0]
    Xf = _f(X, np.float64) if X is not None else None
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    lib().or_rgevc_d(n, _ptr(Sf), _ptr(Tf), _ptr(Xf), _ptr(V), int(left))
    return V


def ggordschur(S, T, Q, Z, select, scale=True):
    """gordschur!(S, T, Q, Z, select) for a complex generalized Schur form (ordschur.jl:
    147-305): (S, T, alpha, beta, Q, Z, status), status 1 + j1 for a rejected swap."""
    Sf, Tf, Qf, Zf = (_f(x, np.complex128) for x in (S, T, Q, Z))
    n = Sf.shape[0]
    sel = np.ascontiguousarray(np.asarray(select, dtype=np.int32))
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1), dtype=np.complex128)
    st = lib().or_ggordschur_z(n, _ptr(Sf), _ptr(Tf), _ptr(Qf), _ptr(Zf), sel.ctypes.data_as(ctypes.c_void_p),
                               int(scale), _ptr(al), _ptr(be))
    return Sf, Tf, al[:n], be[:n], Qf, Zf, st


def ggordschur_real(S, T, Q, Z, select, scale=True):
    """gordschur!(S, T, Q, Z, select) for a real generalized Schur pair (rordschur.jl:542-627):
    (S, T, alpha, beta, Q, Z, status), status 1 + k when the block at k could not be moved."""
    Sf, Tf, Qf, Zf = (_f(x, np.float64) for x in (S, T, Q, Z))
    n = Sf.shape[0]
    sel = np.ascontiguousarray(np.asarray(select, dtype=np.int32))
    al = np.zeros(max(n, 1), dtype=np.complex128)
    be = np.zeros(max(n, 1))
    st = lib().or_ggordschur_d(n, _ptr(Sf), _ptr(Tf), _ptr(Qf), _ptr(Zf), sel.ctypes.data_as(ctypes.c_void_p),
                               int(scale), _ptr(al), _ptr(be))
    return Sf, Tf, al[:n], be[:n], Qf, Zf, st


def gtrsylvester(A, B, C, D, E, F, adjoint=False):
    """trsylvester!(A, B, C, D, E, F) / adjtrsylvester! (gsylvester.jl:23-155) for complex
    triangular matrices: (R, L, scale)."""
    A_, B_, D_, E_ = (_f(x, np.complex128) for x in (A, B, D, E))
    C_, F_ = _f(C, np.complex128), _f(F, np.complex128)
    m, n = C_.shape
    fn = lib().or_gtrsyl_z
    fn.restype = ctypes.c_double
    sc = fn(m, n, _ptr(A_), _ptr(B_), _ptr(C_), _ptr(D_), _ptr(E_), _ptr(F_), int(adjoint))
    return C_, F_, sc


def geigvalscond(S, T, nsub):
    """eigvalscond(S::GeneralizedSchur, nsub) (gcondition.jl:121-165): (pl, pr)."""
    Sf, Tf = _f(S, np.complex128), _f(T, np.complex128)
    out = np.zeros(2)
    lib().or_gcond_z(Sf.shape[0], _ptr(Sf), _ptr(Tf), int(nsub), _ptr(out), 0)
    return out[0], out[1]


def gsubspacesep(S, T, nsub):
    """subspacesep(S::GeneralizedSchur, nsub) with pnorm = :F (gcondition.jl:169-260)."""
    Sf, Tf = _f(S, np.complex128), _f(T, np.complex128)
    out = np.zeros(2)
    lib().or_gcond_z(Sf.shape[0], _ptr(Sf), _ptr(Tf), int(nsub), _ptr(out), 1)
    return out


def norm1est(apply, apply_h, N):
    """norm1est! (norm1est.jl:21-74) with apply / apply_h returning the operator (its adjoint)
    applied to a vector; _findamax (norm1est.jl:76-99) on abs2 for complex vectors."""
    tiny = np.finfo(np.float64).tiny
    x = apply(np.full(N, 1.0 / N, dtype=np.complex128))
    if N == 1:
        return abs(x[0])
    gamma = float(np.sum(np.abs(x)))

    def sign(v):
        a = np.abs(v)
        out = np.ones_like(v)
        big = a > tiny
        out[big] = v[big] / a[big]
        return out

    def findamax(v):
        k = v.real * v.real + v.imag * v.imag
        i0 = int(np.argmax(k))
        return float(np.sqrt(k[i0])), i0

    x = apply_h(sign(x))
    ax0, j0 = findamax(x)
    for _ in range(5):
        e = np.zeros(N, dtype=np.complex128)
        e[j0] = 1.0
        x = apply(e)
        old = gamma
        gamma = float(np.sum(np.abs(x)))
        if gamma <= old:
            break
        x = apply_h(sign(x))
        jlast = j0
        ax0, j0 = findamax(x)
        if abs(x[jlast]) == ax0:
            break
    v = np.array([(1.0 if i % 2 == 0 else -1.0) * (1.0 + i / (N - 1)) for i in range(N)], dtype=np.complex128)
    v = apply(v)
    t = 2.0 * float(np.sum(np.abs(v))) / (3 * N)
    return max(t, gamma)


def gsubspacesep1(S, T, nsub):
    """subspacesep(S::GeneralizedSchur, nsub; pnorm = 1) (gcondition.jl:169-260) with the
    Sylvester solves applied in place, as in the standard-form subspacesep
    (ordschur.jl:118-140): [1 / est_u, 1 / est_l]."""
    S = np.asarray(S, dtype=np.complex128)
    T = np.asarray(T, dtype=np.complex128)
    n = S.shape[0]
    n1, n2 = nsub, n - nsub
    out = []
    for A, B, D, E, m, q in ((S[:n1, :n1], S[n1:, n1:], T[:n1, :n1], T[n1:, n1:], n1, n2),
                             (S[n1:, n1:], S[:n1, :n1], T[n1:, n1:], T[:n1, :n1], n2, n1)):
        def op(adj, A=A, B=B, D=D, E=E, m=m, q=q):
            def f(x):
                R = x[:m * q].reshape((m, q), order="F")
                L = x[m * q:].reshape((m, q), order="F")
                R2, L2, _ = gtrsylvester(A, B, R, D, E, L, adjoint=adj)
                return np.concatenate([R2.ravel(order="F"), L2.ravel(order="F")])
            return f
        out.append(1.0 / norm1est(op(False), op(True), 2 * m * q))
    return np.array(out)
