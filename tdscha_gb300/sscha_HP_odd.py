"""Drop-in for the reference's compiled module `sscha_HP_odd` on the fast path
(`GetPerturbAverageSym`, and `GetPerturbAverage` without symmetry images).

`GetPerturbAverageSym` keeps the reference's positional arguments
(CModules/odd_corr_module.c:491-634, call site
Modules/DynamicalLanczos.py:3114-3116) and writes the outputs in place:
`f_out` is overwritten, `d2v_out` is overwritten with the D3 term and the D4
term is added when apply_D4 == 1.  The computation runs in float64 on the GPU
through the C ABI (tdscha_get_perturb_average_sym); errors raise instead of
terminating the interpreter (the reference calls exit(EXIT_FAILURE),
odd_corr_module.c:535-547).
"""
import numpy as np

from . import _native as nat


def GetPerturbAverageSym(X, Y, w, rho, R1, Y1, T, apply_D4, N_syms, sym_list, n_deg,
                         sym_basis_list, blocks_ids, f_out, d2v_out):
    lib = nat.load()
    X, Y, w, rho = nat.f64(X), nat.f64(Y), nat.f64(w), nat.f64(rho)
    R1, Y1 = nat.f64(R1), nat.f64(Y1)
    N, M = X.shape
    if M != w.shape[0]:
        raise ValueError("N_modes from X is %d, while len(w) = %d" % (M, w.shape[0]))
    if apply_D4 not in (0, 1):
        raise ValueError("the apply_D4 value passed must be either 0 or 1 (got %r)" % apply_D4)
    for name, arr, shape in (("f_out", f_out, (M,)), ("d2v_out", d2v_out, (M, M))):
        if not (isinstance(arr, np.ndarray) and arr.dtype == np.float64 and arr.shape == shape
                and arr.flags.c_contiguous):
            raise ValueError("%s must be a C-contiguous float64 array of shape %s" % (name, shape))
    ndeg_flat, deg, sym, s = nat.flatten_symmetries(sym_list, sym_basis_list)
    if int(N_syms) != s:
        raise ValueError("N_syms=%d but the symmetry blocks hold %d images" % (N_syms, s))
    if not np.array_equal(np.asarray(n_deg, dtype=np.intc), ndeg_flat):
        raise ValueError("n_deg does not match the degenerate spaces")
    bid = nat.i32(blocks_ids)
    nat.check(lib.tdscha_get_perturb_average_sym(
        M, N, nat.dp(X), nat.dp(Y), nat.dp(w), nat.dp(rho), nat.dp(R1), nat.dp(Y1), float(T),
        int(apply_D4), s, len(ndeg_flat), nat.ip(ndeg_flat), nat.ip(deg), nat.dp(sym),
        nat.ip(bid), nat.dp(f_out), nat.dp(d2v_out)))
    return None


def GetPerturbAverage(X, Y, w, rho, R1, Y1, T, apply_D4, f_out, d2v_out):
    """The module's form without symmetry images (CModules/odd_corr_module.c:408-487,
    LanczosFunctions.c:1731-1905): same outputs and in-place convention.  Y1 enters
    those loops only through x^T Y1 x and x^T Y1 f, i.e. through its symmetric part,
    so this is GetPerturbAverageSym with one-mode identity blocks on (Y1 + Y1^T) / 2
    (the reference's two functions agree to rounding on such inputs)."""
    X = nat.f64(X)
    if X.ndim != 2:
        raise ValueError("X must be an (N, n_modes) array")
    M = X.shape[1]
    Y1 = nat.f64(Y1)
    if Y1.shape != (M, M):
        raise ValueError("Y1 must have shape (%d, %d), got %s" % (M, M, Y1.shape))
    one = np.ones((1, 1, 1))
    return GetPerturbAverageSym(X, Y, w, rho, R1, 0.5 * (Y1 + Y1.T), T, apply_D4, 1, [one] * M,
                                np.ones(M, dtype=np.intc),
                                [np.array([i], dtype=np.intc) for i in range(M)],
                                np.arange(M, dtype=np.intc), f_out, d2v_out)
