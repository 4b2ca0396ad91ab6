"""ctypes binding of libgschur_gb300.so (declarations in include/gschur_gb300.h).

The library is the product: there is no CPU fallback.  If the shared object is
missing or cannot be loaded, every entry point raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libgschur_gb300.so")
# launch shapes of the batched kernels chosen by tune.py on a GB300 (sm_103a, the only
# target this library is built for)
DEFAULT_TUNING = os.path.join(HERE, "tuning", "sm_103a.tsv")

GS_OK = 0
GS_UNCONVERGED = 1
GS_BADARG = 2
GS_CUDA = 3

GS_WANTZ = 1
GS_SCALE = 2
GS_DEVICE = 4
GS_GRAPH = 8
GS_RAW = 16
GS_NOFALLBACK = 32
GS_BAL_PERMUTE = 64
GS_DC = 128
GS_MIXED = 256

_i = ctypes.c_int
_i64 = ctypes.c_int64
_u = ctypes.c_uint
_p = ctypes.c_void_p

# name -> (restype, argtypes); kept in sync with include/gschur_gb300.h
SIGNATURES = {
    "gs_version": (_i, []),
    "gs_create": (_i, [ctypes.POINTER(_p), _i]),
    "gs_destroy": (_i, [_p]),
    "gs_set_stream": (_i, [_p, _p]),
    "gs_last_error": (ctypes.c_char_p, [_p]),
    "gs_last_kernel_ms": (ctypes.c_float, [_p]),
    "gs_host_alloc": (_i, [_p, ctypes.POINTER(_p), ctypes.c_size_t]),
    "gs_host_free": (_i, [_p, _p]),
    "gs_set_tuning": (_i, [_p, ctypes.c_char_p]),
    "gs_get_tuning": (_i, [_p, ctypes.c_char_p, ctypes.c_size_t]),
    "gs_schur_f64": (_i, [_p, _i64, _p, _i64, _p, _i64, _p, _p, _u, _i64]),
    "gs_schur_f32": (_i, [_p, _i64, _p, _i64, _p, _i64, _p, _p, _u, _i64]),
    "gs_schur_c64": (_i, [_p, _i64, _p, _i64, _p, _i64, _p, _u, _i64, _i64]),
    "gs_schur_batched_f64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _p, _p, _u]),
    "gs_mixed_batched_info": (_i, [_p, _p]),
    "gs_schur_batched_f32": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _p, _p, _u]),
    "gs_schur_batched_c64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _p, _u]),
    "gs_eigvecs_c64": (_i, [_p, _i64, _p, _p, _p, _p, _u]),
    "gs_eigvecs_f64": (_i, [_p, _i64, _p, _p, _p, _p, _u]),
    "gs_triangularize_f64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _u]),
    "gs_eigvecs_batched_c64": (_i, [_p, _i64, _p, _p, _i64, _p, _p, _p, _p, _u]),
    "gs_eigvecs_batched_f64": (_i, [_p, _i64, _p, _p, _p, _i64, _i64, _p, _p, _p, _p, _u]),
    "gs_eig_adjoint_batched_c64": (_i, [_p, _i64, _p, _p, _p, _i64, _i64, _p, _p, _p, _p, _u]),
    "gs_hessenberg_f64": (_i, [_p, _i64, _p, _i64, _p, _p, _i64, _u]),
    "gs_schur_mixed_f64": (_i, [_p, _i64, _p, _i64, _p, _i64, _p, _p, _u, _i64, _p]),
    "gs_balance_f64": (_i, [_p, _i64, _p, _i64, _u, _p, _p, _p]),
    "gs_balance_c64": (_i, [_p, _i64, _p, _i64, _u, _p, _p, _p]),
    "gs_balancer_apply_c64": (_i, [_p, _i64, _i64, _p, _i64, _p, _p, _p, _i, _u]),
    "gs_enormalize_c64": (_i, [_p, _i64, _i64, _p, _i64, _u]),
    "gs_rconde_c64": (_i, [_p, _i64, _p, _p, _p, _u]),
    "gs_ordschur_f64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _u]),
    "gs_ordschur_c64": (_i, [_p, _i64, _p, _p, _p, _p, _u]),
    "gs_eigvalscond_f64": (_i, [_p, _i64, _p, _i64, _i64, _p, _u]),
    "gs_eigvalscond_c64": (_i, [_p, _i64, _p, _i64, _i64, _p, _u]),
    "gs_subspacesep_f64": (_i, [_p, _i64, _p, _i64, _i64, _p, _u]),
    "gs_subspacesep_c64": (_i, [_p, _i64, _p, _i64, _i64, _p, _u]),
    "gs_eigen_rcond_f64": (_i, [_p, _i64, _p, _p, _p, _u]),
    "gs_eigen_rcond_c64": (_i, [_p, _i64, _p, _p, _p, _u]),
    "gs_heev_f64": (_i, [_p, _i64, _p, _i64, _i, _p, _p, _i64, _u]),
    "gs_heev_c64": (_i, [_p, _i64, _p, _i64, _i, _p, _p, _i64, _u]),
    "gs_hetrd_f64": (_i, [_p, _i64, _p, _i64, _i, _p, _p, _p, _u]),
    "gs_hetrd_c64": (_i, [_p, _i64, _p, _i64, _i, _p, _p, _p, _u]),
    "gs_steqr_f64": (_i, [_p, _i64, _p, _p, _p, _i64, _u]),
    "gs_stedc_f64": (_i, [_p, _i64, _p, _p, _p, _i64, _u]),
    "gs_ggschur_c64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _u]),
    "gs_ggschur_f64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _u]),
    "gs_ggschur_batched_f64": (_i, [_p, _i64, _p, _p, _i64, _p, _p, _p, _p, _p, _i64, _p, _p, _p, _u]),
    "gs_ggeigvecs_f64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _u]),
    "gs_ggordschur_c64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _p, _u]),
    "gs_ggordschur_f64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _p, _u]),
    "gs_trsylvester_f64": (_i, [_p, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _i, _i, _p, _p, _u]),
    "gs_trsylvester_c64": (_i, [_p, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _i, _i, _p, _p, _u]),
    "gs_gtrsylvester_c64": (_i, [_p, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _i, _p,
                                 _p, _u]),
    "gs_geigvalscond_c64": (_i, [_p, _i64, _p, _i64, _p, _i64, _i64, _p, _u]),
    "gs_gsubspacesep_c64": (_i, [_p, _i64, _p, _i64, _p, _i64, _i64, _i, _p, _u]),
    "gs_ggeigvecs_c64": (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _u]),
    "gs_gemm_f64_tc": (_i, [_p, _i64, _i64, _i64, _p, _i64, _i, _p, _i64, _p, _i64, _u]),
    "gs_ggschur_batched_c64": (_i, [_p, _i64, _p, _p, _i64, _p, _p, _p, _p, _p, _i64, _p, _p, _p, _u]),
}
# allocation-free entry point (include/gschur_gb300_noalloc.h)
SIGNATURES["gs_schur_batched_f64_noalloc"] = (_i, [_p, _i64, _p, _p, _p, _p, _p, _p, _p, _p, _u])

_lib = None
_lock = threading.Lock()


def load(path=None):
    """Load the shared library (once) and attach the C signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError(
                "libgschur_gb300.so not found at %s; build it with genericschur.jl_gb300/build_lib.py" % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


class GSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class Context:
    """A library context on one CUDA device (owns a stream and a workspace arena)."""

    def __init__(self, device=0):
        self.lib = load()
        h = _p()
        rc = self.lib.gs_create(ctypes.byref(h), int(device))
        self.handle = h
        if rc != GS_OK:
            msg = self.last_error()
            raise GSError(rc, "gs_create failed: %s" % msg)
        self.device = device
        # the committed table of tuned launch shapes (GS_TUNING overrides; "" keeps the defaults)
        path = os.environ.get("GS_TUNING", DEFAULT_TUNING)
        if path and os.path.exists(path):
            self.set_tuning(path)

    def last_error(self):
        s = self.lib.gs_last_error(self.handle)
        return s.decode() if s else ""

    def set_tuning(self, path):
        """Load a batched-kernel tuning table (None: the built-in shapes)."""
        rc = self.lib.gs_set_tuning(self.handle, path.encode() if path else None)
        if rc != GS_OK:
            raise GSError(rc, self.last_error())

    def tuning(self):
        """The active tuning table as text."""
        buf = ctypes.create_string_buffer(4096)
        self.lib.gs_get_tuning(self.handle, buf, ctypes.c_size_t(len(buf)))
        return buf.value.decode()

    def set_stream(self, stream_ptr):
        self.lib.gs_set_stream(self.handle, _p(stream_ptr) if stream_ptr else None)

    def last_kernel_ms(self):
        return float(self.lib.gs_last_kernel_ms(self.handle))

    def mixed_info(self):
        """Counters of the last GS_MIXED batched call: refined, handed back to FP64, Newton
        steps, FLOPs of the refinement's FP64-accurate (tensor-core) products, refinement and
        FP32-stage device times in us (-1 if not timed)."""
        info = (ctypes.c_int64 * 6)()
        rc = self.lib.gs_mixed_batched_info(self.handle, info)
        if rc != GS_OK:
            raise RuntimeError("gs_mixed_batched_info: %s" % self.last_error())
        keys = ("refined", "handed_back", "newton_steps", "product_flops", "refine_us", "fp32_us")
        return dict(zip(keys, (int(x) for x in info)))

    def host_alloc(self, nbytes):
        p = _p()
        rc = self.lib.gs_host_alloc(self.handle, ctypes.byref(p), ctypes.c_size_t(nbytes))
        if rc != GS_OK:
            raise GSError(rc, self.last_error())
        return p.value

    def host_free(self, ptr):
        self.lib.gs_host_free(self.handle, _p(ptr))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gs_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ctx = {}


def get_context(device=0):
    """Process-wide default context per device."""
    c = _ctx.get(device)
    if c is None:
        c = Context(device)
        _ctx[device] = c
    return c
