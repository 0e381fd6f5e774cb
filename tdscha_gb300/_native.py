"""ctypes binding of libtdscha_gb300.so (the C ABI in include/tdscha_gb300.h).

There is no fallback: if the library is missing or the GPU is unavailable
every call raises.  Build it with `python -m tdscha_gb300.build`.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtdscha_gb300.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NAN, ERR_STATE, ERR_TIMEOUT = -1, -2, -3, -4, -5
PREC_FP64, PREC_MIXED = 0, 1

# every symbol the public header declares
EXPORTS = [
    "tdscha_last_error", "tdscha_version", "tdscha_get_perturb_average_sym",
    "tdscha_ctx_create", "tdscha_ctx_destroy", "tdscha_ctx_set_options",
    "tdscha_perturb_averages", "tdscha_apply_full_L", "tdscha_lanczos_run",
    "tdscha_continued_fraction", "tdscha_ctx_profile", "tdscha_ctx_profile_read",
    "tdscha_perturb_averages_noalloc",
]


class TdschaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("tdscha_gb300 error %d: %s" % (code, msg))
        self.code = code


_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_c_int, _c_double = ctypes.c_int, ctypes.c_double


def load():
    """Load the library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libtdscha_gb300.so not found at %s; run `python -m tdscha_gb300.build`"
                          % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    lib.tdscha_last_error.restype = ctypes.c_char_p
    lib.tdscha_version.restype = ctypes.c_char_p
    lib.tdscha_get_perturb_average_sym.argtypes = [
        _c_int, _c_int, _d, _d, _d, _d, _d, _d, _c_double, _c_int, _c_int, _c_int, _i, _i, _d, _i,
        _d, _d]
    lib.tdscha_ctx_create.argtypes = [
        ctypes.POINTER(_vp), _c_int, _c_int, _d, _d, _d, _d, _c_double, _c_int, _c_int, _i, _i,
        _d, _i, _c_int]
    lib.tdscha_ctx_destroy.argtypes = [_vp]
    lib.tdscha_ctx_set_options.argtypes = [_vp, _c_int, _c_int, _c_int, _c_int, _c_int, _c_double]
    lib.tdscha_perturb_averages.argtypes = [_vp, _vp, _vp, _c_int, _c_int, _vp, _vp, _c_int, _vp]
    lib.tdscha_apply_full_L.argtypes = [_vp, _vp, _vp, _c_int, _c_int, _vp]
    lib.tdscha_lanczos_run.argtypes = [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_int, _c_int,
                                       _c_int, _d, _i, _i, _vp]
    lib.tdscha_continued_fraction.argtypes = [
        _d, _c_int, _d, _c_int, _d, _c_int, _d, _c_int, _c_int, _c_double, _c_int, _c_double,
        _c_int, _c_int, _c_double, _c_int, _d]
    lib.tdscha_ctx_profile.argtypes = [_vp, _c_int]
    lib.tdscha_ctx_profile_read.argtypes = [_vp, _c_int, _d, _i]
    lib.tdscha_perturb_averages_noalloc.argtypes = [
        _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _c_double, _c_int, _vp, _vp, _vp]
    for name in EXPORTS:
        fn = getattr(lib, name)
        if name not in ("tdscha_last_error", "tdscha_version"):
            fn.restype = ctypes.c_int
    _lib = lib
    return lib


def check(rc):
    if rc != OK:
        msg = load().tdscha_last_error().decode(errors="replace")
        raise TdschaError(rc, msg)


def dp(a):
    return a.ctypes.data_as(_d)


def ip(a):
    return a.ctypes.data_as(_i)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.intc)


def flatten_symmetries(symmetries, degenerate_space):
    """Per-block lists (as the reference passes them) -> flat C-ABI tables."""
    n_deg = np.array([len(b) for b in degenerate_space], dtype=np.intc)
    deg = i32(np.concatenate([np.asarray(b, dtype=np.intc).ravel() for b in degenerate_space]))
    sym = f64(np.concatenate([np.asarray(s, dtype=np.float64).ravel() for s in symmetries]))
    n_syms = int(np.asarray(symmetries[0]).shape[0])
    for s, b in zip(symmetries, degenerate_space):
        s = np.asarray(s)
        if s.ndim != 3 or s.shape[0] != n_syms or s.shape[1] != len(b) or s.shape[2] != len(b):
            raise ValueError("symmetry block of shape %s does not match its degenerate space "
                             "of size %d and %d images" % (s.shape, len(b), n_syms))
    return n_deg, deg, sym, n_syms


class Context:
    """Owns a tdscha_ctx: the ensemble resident on the GPU."""

    def __init__(self, X, Y, w, rho, T, symmetries, degenerate_space, blocks_ids,
                 with_mixed=False):
        lib = load()
        X, Y, w, rho = f64(X), f64(Y), f64(w), f64(rho)
        if X.ndim != 2 or Y.shape != X.shape:
            raise ValueError("X and Y must be (N, M) arrays of the same shape")
        N, M = X.shape
        if w.shape != (M,):
            raise ValueError("N_modes from X is %d, while len(w) = %d" % (M, w.shape[0]))
        if rho.shape != (N,):
            raise ValueError("len(rho) = %d does not match N = %d" % (rho.shape[0], N))
        n_deg, deg, sym, n_syms = flatten_symmetries(symmetries, degenerate_space)
        bid = i32(blocks_ids)
        self.M, self.N, self.S = M, N, n_syms
        self.P = M + M * (M + 1)
        self.with_mixed = bool(with_mixed)
        h = _vp()
        check(lib.tdscha_ctx_create(ctypes.byref(h), M, N, dp(X), dp(Y), dp(w), dp(rho), float(T),
                                    n_syms, len(n_deg), ip(n_deg), ip(deg), dp(sym), ip(bid),
                                    1 if with_mixed else 0))
        self.handle = h
        self._opts = None

    def set_options(self, use_wigner, ignore_harmonic, ignore_v3, ignore_v4, reverse_L, shift):
        opts = (int(bool(use_wigner)), int(bool(ignore_harmonic)), int(bool(ignore_v3)),
                int(bool(ignore_v4)), int(bool(reverse_L)), float(shift))
        if opts != self._opts:
            check(load().tdscha_ctx_set_options(self.handle, *opts))
            self._opts = opts

    def close(self):
        if getattr(self, "handle", None):
            load().tdscha_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
