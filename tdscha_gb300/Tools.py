"""Linear solvers of the static response (Modules/Tools.py).

`minimum_residual_algorithm` and `minimum_residual_algorithm_precond` keep the
reference's interface (an operator with `.matvec`, numpy or torch vectors) and
its iteration (Tools.py:265-474).  `batched_minimum_residual` runs the same
iteration for many right-hand sides at once on device tensors (one row per
system): every row follows its own scalars and stops updating once its
residual is below the threshold, exactly as independent runs would; the
operator is applied to the still-active rows only.
"""
import time

import numpy as np


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _dot(a, b):
    if _is_torch(a):
        return float((a * b).sum())
    return float(a.dot(b))


def _copy(a):
    return a.clone() if _is_torch(a) else a.copy()


def _matvec(A, x):
    return A.matvec(x) if hasattr(A, "matvec") else A(x)


def minimum_residual_algorithm(A, b, x0, precond=None, verbose=True, max_iters=100,
                               conv_thr=1e-6, callback=None):
    """Solve A x = b by the minimal-residual iteration (Tools.py:265-414)."""
    if verbose:
        print()
        print("Minimal residual algorithm")
        print("--------------------------")
        print()
        print("Initialization...")
    r1 = b - _matvec(A, x0)
    if precond is not None:
        r1 = _matvec(precond, r1)
    b_prec = _copy(b)
    if precond is not None:
        b_prec = _matvec(precond, b)
    if verbose:
        print("Starting residual: {}".format(np.sqrt(_dot(r1, r1))))
    r1_bar = _matvec(A, r1)
    if precond is not None:
        r1_bar = _matvec(precond, r1_bar)
    z1 = _copy(r1)
    p1 = _copy(r1)
    p1_bar = _copy(r1_bar)
    x = _copy(x0)
    b_norm = np.sqrt(_dot(b_prec, b_prec))
    iters = 1
    converged = False
    r_norm = np.inf
    while iters < max_iters and not converged:
        t1 = time.time()
        if verbose:
            print("Iteration: {}".format(iters))
        Ap = p1_bar
        Ap_bar = _matvec(A, p1_bar)
        if precond is not None:
            Ap_bar = _matvec(precond, Ap_bar)
        alpha = _dot(r1_bar, z1) / _dot(p1_bar, Ap)
        x = x + alpha * p1
        if callback is not None:
            callback(x, iters)
        r = r1 - alpha * Ap
        rbar = r1_bar - alpha * Ap_bar
        r_norm = np.sqrt(_dot(r, r)) / b_norm
        if verbose:
            print("    residual = {}".format(r_norm))
            print("    time to perform the step: {} s".format(time.time() - t1))
        beta = _dot(rbar, r) / _dot(r1_bar, z1)
        p1 = r + beta * p1
        p1_bar = rbar + beta * p1_bar
        r1, r1_bar, z1 = r, rbar, r
        converged = r_norm < conv_thr
        iters += 1
    if not converged:
        print("WARNING: cg did not converge after {} iterations.".format(max_iters))
        print("         residual = {}".format(r_norm))
    return x


def minimum_residual_algorithm_precond(A, b, precond_half, **kwargs):
    """Solve A x = b as (P A P) y = P b, x = P y with P ~ A^-1/2 (Tools.py:417-474)."""
    if precond_half is None:
        return minimum_residual_algorithm(A, b, _copy(b), precond=None, **kwargs)

    class _Tilde:
        def matvec(self, x):
            return _matvec(precond_half, _matvec(A, _matvec(precond_half, x)))

    b_tilde = _matvec(precond_half, b)
    if "x0" not in kwargs:
        kwargs["x0"] = _copy(b_tilde)
    x_tilde = minimum_residual_algorithm(_Tilde(), b_tilde, precond=None, **kwargs)
    return _matvec(precond_half, x_tilde)


def batched_minimum_residual(apply_A, B, X0, max_iters=100, conv_thr=1e-6, verbose=False):
    """The minimal-residual iteration for the rows of B (torch, n_sys x n).

    apply_A maps a (k, n) tensor of rows to A applied to each row.  Returns
    (X, iterations per row, converged per row)."""
    import torch
    R1 = B - apply_A(X0)
    bn = torch.sqrt((B * B).sum(1))
    R1b = apply_A(R1)
    Z1 = R1.clone()
    P1 = R1.clone()
    P1b = R1b.clone()
    X = X0.clone()
    n = B.shape[0]
    active = torch.ones(n, dtype=torch.bool, device=B.device)
    iters = torch.ones(n, dtype=torch.int64, device=B.device)
    it = 1
    while it < max_iters:
        idx = torch.nonzero(active).flatten()
        if idx.numel() == 0:
            break
        full = idx.numel() == n
        p1b = P1b if full else P1b[idx]
        r1b = R1b if full else R1b[idx]
        z1 = Z1 if full else Z1[idx]
        r1 = R1 if full else R1[idx]
        p1 = P1 if full else P1[idx]
        Apb = apply_A(p1b)
        alpha = (r1b * z1).sum(1) / (p1b * p1b).sum(1)
        r = r1 - alpha[:, None] * p1b
        rb = r1b - alpha[:, None] * Apb
        rn = torch.sqrt((r * r).sum(1)) / bn[idx]
        beta = (rb * r).sum(1) / (r1b * z1).sum(1)
        newx = (X if full else X[idx]) + alpha[:, None] * p1
        newp = r + beta[:, None] * p1
        newpb = rb + beta[:, None] * p1b
        if full:
            X, P1, P1b, R1, R1b, Z1 = newx, newp, newpb, r, rb, r.clone()
        else:
            X[idx], P1[idx], P1b[idx] = newx, newp, newpb
            R1[idx], R1b[idx], Z1[idx] = r, rb, r
        conv = rn < conv_thr
        it += 1
        iters[idx] = it
        active[idx[conv]] = False
        if verbose:
            print("iteration %d: %d of %d systems active, max residual %.3e"
                  % (it - 1, int(active.sum()), n, float(rn.max())))
    return X, iters.cpu().numpy(), (~active).cpu().numpy()
