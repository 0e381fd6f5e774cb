"""The C-ABI library loads and exports what include/tdscha_gb300.h declares;
argument validation fails with error codes before any device work."""
import ctypes
import os
import re

import numpy as np
import pytest

from tdscha_gb300 import build, _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return nat.load()


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(tdscha_\w+)\s*\(", src))
    return sorted(names)


def test_header_symbols_exported(lib):
    names = declared_symbols()
    assert "tdscha_perturb_averages" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(nat.EXPORTS) | set(names)


def test_version(lib):
    assert b"sm_103a" in lib.tdscha_version()


def _tables(M):
    return (np.ones(M, dtype=np.intc), np.arange(M, dtype=np.intc), np.ones(M),
            np.arange(M, dtype=np.intc))


def _create(lib, M=4, N=3, **over):
    X = np.zeros((N, M)); Y = np.zeros((N, M)); w = np.full(M, 1e-3); rho = np.ones(N)
    n_deg, deg, sym, bid = _tables(M)
    args = dict(M=M, N=N, X=X, Y=Y, w=w, rho=rho, T=300.0, S=1, nb=M, n_deg=n_deg, deg=deg,
                sym=sym, bid=bid, mixed=0)
    args.update(over)
    h = ctypes.c_void_p()
    rc = lib.tdscha_ctx_create(ctypes.byref(h), args["M"], args["N"], nat.dp(args["X"]),
                               nat.dp(args["Y"]), nat.dp(args["w"]), nat.dp(args["rho"]),
                               args["T"], args["S"], args["nb"], nat.ip(args["n_deg"]),
                               nat.ip(args["deg"]), nat.dp(args["sym"]), nat.ip(args["bid"]),
                               args["mixed"])
    return rc, h


def test_create_rejects_bad_sizes(lib):
    rc, h = _create(lib, M=0)
    assert rc == nat.ERR_ARG and not h.value
    assert b"bad sizes" in lib.tdscha_last_error()


@pytest.mark.gpu
def test_create_rejects_nan_input(gpu_lib):
    # the ensemble is checked for non-finite entries on the device, while its
    # images are formed
    X = np.zeros((3, 4)); X[1, 2] = np.nan
    rc, h = _create(gpu_lib, X=X)
    assert rc == nat.ERR_NAN and not h.value
    assert b"non-finite X/Y at 6" in gpu_lib.tdscha_last_error()
    Y = np.zeros((3, 4)); Y[2, 0] = np.inf
    rc, h = _create(gpu_lib, Y=Y)
    assert rc == nat.ERR_NAN and b"at 8" in gpu_lib.tdscha_last_error()


def test_create_rejects_bad_storage_mode(lib):
    for mode in (-1, 3):
        rc, h = _create(lib, mixed=mode)
        assert rc == nat.ERR_ARG and not h.value and b"with_mixed" in lib.tdscha_last_error()
    with pytest.raises(ValueError):
        nat.Context(np.zeros((3, 4)), np.zeros((3, 4)), np.full(4, 1e-3), np.ones(3), 300.0,
                    None, None, None, with_mixed="fp16")


def test_create_rejects_bad_blocks(lib):
    bid = np.arange(4, dtype=np.intc); bid[2] = 7
    rc, _ = _create(lib, bid=bid)
    assert rc == nat.ERR_ARG and b"blocks_ids" in lib.tdscha_last_error()
    deg = np.array([0, 1, 2, 9], dtype=np.intc)
    rc, _ = _create(lib, deg=deg)
    assert rc == nat.ERR_ARG


def test_create_rejects_nonpositive_frequency(lib):
    rc, _ = _create(lib, w=np.array([1e-3, 0.0, 1e-3, 1e-3]))
    assert rc == nat.ERR_ARG


def test_one_shot_rejects_bad_apply_d4(lib):
    M, N = 3, 2
    n_deg, deg, sym, bid = _tables(M)
    z = np.zeros((N, M)); f = np.zeros(M); d2v = np.zeros((M, M))
    rc = lib.tdscha_get_perturb_average_sym(M, N, nat.dp(z), nat.dp(z), nat.dp(np.ones(M)),
                                            nat.dp(np.ones(N)), nat.dp(np.zeros(M)),
                                            nat.dp(np.zeros((M, M))), 300.0, 2, 1, M,
                                            nat.ip(n_deg), nat.ip(deg), nat.dp(sym), nat.ip(bid),
                                            nat.dp(f), nat.dp(d2v))
    assert rc == nat.ERR_ARG and b"apply_D4" in lib.tdscha_last_error()


def test_null_context_calls(lib):
    assert lib.tdscha_perturb_averages(None, None, None, 1, 0, None, None, 0, None) == nat.ERR_ARG
    assert lib.tdscha_apply_full_L(None, None, None, 0, 0, None) == nat.ERR_ARG
    i = ctypes.c_int()
    assert lib.tdscha_lanczos_run(None, None, None, 1, 0, 1, 0, 0, 0, None, ctypes.byref(i),
                                  ctypes.byref(i), None) == nat.ERR_ARG
    assert lib.tdscha_ctx_destroy(None) == nat.OK


def test_continued_fraction_rejects_bad_args(lib):
    g = np.zeros(2)
    a = np.ones(1)
    rc = lib.tdscha_continued_fraction(nat.dp(a), 0, nat.dp(a), 0, nat.dp(a), 0, nat.dp(a), 1,
                                       0, 1.0, 0, 0.0, 1, 1, 0.0, 0, nat.dp(g))
    assert rc == nat.ERR_ARG


# entry points whose first argument is a context / network handle: NULL is rejected
# with TDSCHA_ERR_ARG before any CUDA call (destroy of NULL is a no-op)
_HANDLE_FIRST = [
    "tdscha_ctx_layout", "tdscha_ctx_profile", "tdscha_ctx_profile_read", "tdscha_ctx_set_basis_ld",
    "tdscha_ctx_set_options", "tdscha_ctx_set_translations", "tdscha_ctx_sync", "tdscha_ctx_tuning",
    "tdscha_lanczos_run", "tdscha_lanczos_run_hostbuf", "tdscha_apply_full_L",
    "tdscha_perturb_averages", "tdscha_static_L", "tdscha_static_hessian_expand",
    "tdscha_static_hessian_collect", "tdscha_qapply_full_L", "tdscha_qctx_set_pert",
    "tdscha_qctx_set_precision", "tdscha_qkpm_run", "tdscha_qlanczos_run",
    "tdscha_qperturb_averages", "tdscha_mlp_forward", "tdscha_mlp_get_params",
    "tdscha_mlp_set_params", "tdscha_mlp_loss_grad", "tdscha_mlp_train_step",
    # no handle, but null output / input pointers
    "tdscha_ctx_create", "tdscha_qctx_create", "tdscha_mlp_create", "tdscha_project_modes",
    "tdscha_project_bloch", "tdscha_perturb_averages_noalloc", "tdscha_lanczos_run_batch"]


def _null_args(fn):
    args = []
    for t in fn.argtypes:
        if t in (ctypes.c_double, ctypes.c_float):
            args.append(0.0)
        elif t in (ctypes.c_int, ctypes.c_long, ctypes.c_longlong, ctypes.c_uint,
                   ctypes.c_ulong, ctypes.c_ulonglong, ctypes.c_size_t):
            args.append(0)
        else:
            args.append(None)
    return args


@pytest.mark.parametrize("name", _HANDLE_FIRST)
def test_null_handles_and_pointers_rejected(lib, name):
    fn = getattr(lib, name)
    args = _null_args(fn)
    if name == "tdscha_lanczos_run_batch":
        args[1] = -1          # a negative run count with no runs
    assert fn(*args) == nat.ERR_ARG, name
    assert lib.tdscha_last_error()


def test_null_destroy_is_noop(lib):
    for name in ("tdscha_ctx_destroy", "tdscha_qctx_destroy", "tdscha_mlp_destroy"):
        assert getattr(lib, name)(None) == nat.OK
