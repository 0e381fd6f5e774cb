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
    "tdscha_qctx_create", "tdscha_qctx_destroy", "tdscha_qctx_set_pert",
    "tdscha_qperturb_averages", "tdscha_qapply_full_L", "tdscha_qlanczos_run",
    "tdscha_static_L", "tdscha_ctx_sync", "tdscha_static_hessian_expand",
    "tdscha_static_hessian_collect", "tdscha_qkpm_run", "tdscha_lanczos_run_hostbuf",
    "tdscha_project_modes", "tdscha_project_bloch", "tdscha_ctx_set_translations",
    "tdscha_lanczos_run_batch", "tdscha_mlp_create", "tdscha_mlp_destroy",
    "tdscha_mlp_num_params", "tdscha_mlp_set_params", "tdscha_mlp_get_params",
    "tdscha_mlp_forward", "tdscha_mlp_loss_grad", "tdscha_mlp_train_step",
    "tdscha_release_cached_memory", "tdscha_ctx_layout", "tdscha_ctx_tuning",
    "tdscha_qctx_set_precision", "tdscha_ctx_set_basis_ld",
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
    lib.tdscha_ctx_set_basis_ld.argtypes = [_vp, ctypes.c_longlong]
    lib.tdscha_continued_fraction.argtypes = [
        _d, _c_int, _d, _c_int, _d, _c_int, _d, _c_int, _c_int, _c_double, _c_int, _c_double,
        _c_int, _c_int, _c_double, _c_int, _d]
    lib.tdscha_ctx_profile.argtypes = [_vp, _c_int]
    lib.tdscha_ctx_profile_read.argtypes = [_vp, _c_int, _d, _i]
    lib.tdscha_perturb_averages_noalloc.argtypes = [
        _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _c_double, _c_int, _vp, _vp, _vp]
    lib.tdscha_qctx_create.argtypes = [
        ctypes.POINTER(_vp), _c_int, _c_int, _c_int, _d, _d, _d, _i, _d, _c_double, _c_int, _i,
        _i, _d]
    lib.tdscha_qctx_destroy.argtypes = [_vp]
    lib.tdscha_qctx_set_pert.argtypes = [_vp, _c_int, _i, _c_int, _c_int, _c_int,
                                         ctypes.POINTER(ctypes.c_long), _i]
    lib.tdscha_qperturb_averages.argtypes = [_vp, _vp, _vp, _c_int, _vp, _vp, _c_int, _vp]
    lib.tdscha_qapply_full_L.argtypes = [_vp, _vp, _vp, _vp]
    lib.tdscha_qlanczos_run.argtypes = [_vp, _vp, _vp, _c_int, _c_int, _c_int, _c_int, _d, _i,
                                        _i, _vp]
    lib.tdscha_static_L.argtypes = [_vp, _c_int, _vp, _vp, _c_int, _c_double, _c_int, _vp]
    lib.tdscha_ctx_sync.argtypes = [_vp, _vp]
    lib.tdscha_ctx_layout.argtypes = [_vp, _i, ctypes.POINTER(ctypes.c_longlong)]
    lib.tdscha_ctx_tuning.argtypes = [_vp, _i, _i, _d]
    lib.tdscha_qctx_set_precision.argtypes = [_vp, _c_int]
    lib.tdscha_release_cached_memory.argtypes = [_vp]
    lib.tdscha_static_hessian_expand.argtypes = [_vp, _vp, _vp, _vp]
    lib.tdscha_lanczos_run_hostbuf.argtypes = [_vp, _d, _d, _c_int, _c_int, _c_int, _c_int, _c_int,
                                               _c_int, _d, _i, _i]
    lib.tdscha_project_modes.argtypes = [_c_int, _c_int, _c_int, _d, _d, _d, _d, _d, _c_double,
                                         _c_double, _d, _d]
    lib.tdscha_project_bloch.argtypes = [_c_int, _c_int, _c_int, _c_int, _d, _d, _d, _d, _d,
                                         _c_double, _c_double, _d, _d]
    lib.tdscha_ctx_set_translations.argtypes = [_vp, _c_int, _d, _c_int, _i]
    lib.tdscha_lanczos_run_batch.argtypes = [_vp, _c_int]
    _f = ctypes.POINTER(ctypes.c_float)
    lib.tdscha_mlp_create.argtypes = [ctypes.POINTER(_vp), _c_int, _c_int, _c_int]
    lib.tdscha_mlp_destroy.argtypes = [_vp]
    lib.tdscha_mlp_num_params.argtypes = [_vp]
    lib.tdscha_mlp_set_params.argtypes = [_vp, _f]
    lib.tdscha_mlp_get_params.argtypes = [_vp, _f]
    lib.tdscha_mlp_forward.argtypes = [_vp, _f, _c_int, _c_int, _f]
    lib.tdscha_mlp_loss_grad.argtypes = [_vp, _f, _f, _c_int, _f, _f]
    lib.tdscha_mlp_train_step.argtypes = [_vp, _vp, _vp, _c_int, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_float, _c_int, _f, _vp]
    lib.tdscha_qkpm_run.argtypes = [_vp, _vp, _vp, _vp, _c_int, _c_int, _c_double, _c_double, _vp,
                                    _i, _vp]
    lib.tdscha_static_hessian_collect.argtypes = [_vp, _vp, _vp, _vp]
    for name in EXPORTS:
        fn = getattr(lib, name)
        if name not in ("tdscha_last_error", "tdscha_version"):
            fn.restype = ctypes.c_int
    lib.tdscha_mlp_num_params.restype = ctypes.c_long
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
    s0 = symmetries[0] if len(symmetries) else None
    if (isinstance(s0, np.ndarray) and s0.ndim == 3 and s0.shape[1:] == (1, 1)
            and len(symmetries) == len(degenerate_space)
            and all(s is s0 for s in symmetries) and all(len(b) == 1 for b in degenerate_space)):
        # one-mode blocks sharing one image table (the unsymmetrised layout):
        # the same tables without a Python step per block
        nb = len(degenerate_space)
        deg = i32(np.concatenate(degenerate_space).astype(np.intc, copy=False).ravel())
        sym = f64(np.tile(np.asarray(s0, dtype=np.float64).ravel(), nb))
        return np.ones(nb, dtype=np.intc), deg, sym, int(s0.shape[0])
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
        # with_mixed: False (float64 only), True (float64 and mixed operands) or
        # "fp32" (mixed operands only, the float64 rows released after building them)
        if with_mixed not in (False, True, 0, 1, "fp32"):
            raise ValueError("with_mixed must be False, True or 'fp32', got %r" % (with_mixed,))
        code = 2 if with_mixed == "fp32" else (1 if with_mixed else 0)
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
        self.with_mixed = code != 0
        self.fp64_storage = code != 2
        h = _vp()
        check(lib.tdscha_ctx_create(ctypes.byref(h), M, N, dp(X), dp(Y), dp(w), dp(rho), float(T),
                                    n_syms, len(n_deg), ip(n_deg), ip(deg), dp(sym), ip(bid),
                                    code))
        self.handle = h
        self._opts = None

    def layout(self):
        """(images applied on the perturbation side, resident ensemble rows)."""
        j, rows = ctypes.c_int(0), ctypes.c_longlong(0)
        check(load().tdscha_ctx_layout(self.handle, ctypes.byref(j), ctypes.byref(rows)))
        return j.value, rows.value

    def tuning(self):
        """(stage A one-accumulator kernel, stage B splits, tuned application ms)."""
        a, n, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
        check(load().tdscha_ctx_tuning(self.handle, ctypes.byref(a), ctypes.byref(n),
                                       ctypes.byref(ms)))
        return a.value, n.value, ms.value

    def basis_ld(self):
        """Row stride used for Lanczos basis buffers: P rounded up to 32 doubles
        (256-byte rows, so that the re-biorthogonalisation reads element pairs)."""
        return (self.P + 31) // 32 * 32

    def set_basis_ld(self, ld):
        check(load().tdscha_ctx_set_basis_ld(self.handle, int(ld)))

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


def csr_symmetries(symmetries, L):
    """q-space symmetry matrices (dense or scipy.sparse, (L, L) complex) -> the
    C-ABI CSR tables: row pointers (n_syms x (L + 1)) into one shared column /
    value list."""
    rowptr, cols, vals = [], [], []
    base = 0
    for S in symmetries:
        if hasattr(S, "tocsr"):
            S = S.tocsr()
            S.sort_indices()
            rp, ci, v = S.indptr, S.indices, S.data
        else:
            S = np.asarray(S)
            nz = [np.nonzero(S[a])[0] for a in range(S.shape[0])]
            rp = np.concatenate([[0], np.cumsum([len(z) for z in nz])])
            ci = np.concatenate(nz) if len(nz) else np.zeros(0, dtype=int)
            v = np.concatenate([S[a, z] for a, z in enumerate(nz)]) if len(nz) else np.zeros(0)
        if S.shape != (L, L):
            raise ValueError("symmetry matrix of shape %s, expected (%d, %d)" % (S.shape, L, L))
        rowptr.append(np.asarray(rp, dtype=np.int64) + base)
        cols.append(np.asarray(ci, dtype=np.int64))
        vals.append(np.asarray(v, dtype=np.complex128))
        base += len(ci)
    if base >= 2 ** 31:
        raise ValueError("symmetry tables too large")
    return (i32(np.concatenate(rowptr)), i32(np.concatenate(cols) if cols else np.zeros(1)),
            f64(np.concatenate(vals).view(np.float64) if vals else np.zeros(2)))


class QContext:
    """Owns a tdscha_qctx: the Bloch-transformed ensemble resident on the GPU."""

    def __init__(self, X_q, Y_q, w_q, rho, T, valid=None, symmetries=None):
        lib = load()
        X_q = np.ascontiguousarray(X_q, dtype=np.complex128)
        Y_q = np.ascontiguousarray(Y_q, dtype=np.complex128)
        if X_q.ndim != 3 or Y_q.shape != X_q.shape:
            raise ValueError("X_q and Y_q must be (n_q, N, n_bands) arrays of the same shape")
        n_q, N, nb = X_q.shape
        w_q = f64(w_q)
        if w_q.shape != (nb, n_q):
            raise ValueError("w_q must be (n_bands, n_q) = (%d, %d), got %s" % (nb, n_q, w_q.shape))
        rho = f64(rho)
        if rho.shape != (N,):
            raise ValueError("len(rho) = %d does not match N = %d" % (rho.shape[0], N))
        vptr = None
        if valid is not None:
            valid = i32(np.asarray(valid).astype(np.intc))
            if valid.shape != (nb, n_q):
                raise ValueError("valid must be (n_bands, n_q)")
            vptr = ip(valid)
        n_syms, rp, ci, sv = 0, None, None, None
        if symmetries is not None and len(symmetries) > 0:
            rp, ci, sv = csr_symmetries(symmetries, n_q * nb)
            n_syms = len(symmetries)
        self.n_q, self.N, self.nb = n_q, N, nb
        self.n_syms = max(1, n_syms)
        h = _vp()
        Xf, Yf = X_q.view(np.float64), Y_q.view(np.float64)
        check(lib.tdscha_qctx_create(ctypes.byref(h), n_q, nb, N, dp(Xf), dp(Yf), dp(w_q), vptr,
                                     dp(rho), float(T), n_syms,
                                     ip(rp) if rp is not None else None,
                                     ip(ci) if ci is not None else None,
                                     dp(sv) if sv is not None else None))
        self.handle = h
        self.P = None
        self.n_pairs = None

    def set_precision(self, precision):
        """"fp64" (default) or "mixed": fp32 averages on the CUDA cores."""
        code = {"fp64": PREC_FP64, "mixed": PREC_MIXED}.get(precision)
        if code is None:
            raise ValueError("precision must be 'fp64' or 'mixed', got %r" % (precision,))
        if getattr(self, "_precision", None) != code:
            check(load().tdscha_qctx_set_precision(self.handle, code))
            self._precision = code

    def set_pert(self, iq_pert, q_pair_map, ignore_harmonic=False, ignore_v3=False,
                 ignore_v4=False):
        qm = i32(q_pair_map)
        if qm.shape != (self.n_q,):
            raise ValueError("q_pair_map must have n_q = %d entries" % self.n_q)
        P = ctypes.c_long()
        npairs = ctypes.c_int()
        check(load().tdscha_qctx_set_pert(self.handle, int(iq_pert), ip(qm), int(bool(ignore_harmonic)),
                                          int(bool(ignore_v3)), int(bool(ignore_v4)),
                                          ctypes.byref(P), ctypes.byref(npairs)))
        self.P, self.n_pairs = int(P.value), int(npairs.value)
        return self.P

    def close(self):
        if getattr(self, "handle", None):
            load().tdscha_qctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
