"""Many independent Lanczos runs advanced together on one GPU.

`run_batch([lanc_1, lanc_2, ...], n_iter)` takes prepared Lanczos and
QSpaceLanczos objects (each with its own ensemble context and perturbation:
IR / Raman polarisations, separate perturbations, q-points) and advances all
of them by n_iter steps through tdscha_lanczos_run_batch: every run on its own
stream, up to 16 steps of every run launched before any read-back, so small
runs fill the GPU together instead of one after the other.  The coefficients
land in each object exactly as run_FT would put them there.
"""
import ctypes

import numpy as np

from . import _native as nat
from .DynamicalLanczos import _torch
from .QSpaceLanczos import QSpaceLanczos


class _Run(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("ctx", ctypes.c_void_p), ("basis_Q", ctypes.c_void_p),
                ("basis_P", ctypes.c_void_p), ("capacity", ctypes.c_int),
                ("start_step", ctypes.c_int), ("n_iter", ctypes.c_int), ("run_simm", ctypes.c_int),
                ("precision", ctypes.c_int), ("reorth", ctypes.c_int),
                ("hist", ctypes.POINTER(ctypes.c_double)), ("steps_done", ctypes.c_int),
                ("converged", ctypes.c_int), ("status", ctypes.c_int)]


def run_batch(runs, n_iter, reorth=None, verbose=False):
    """Advance every object in `runs` by n_iter Lanczos steps together.

    reorth: None keeps each object's own choice (full_reorth for Lanczos,
    True -- the reference default -- for QSpaceLanczos); True / False forces it."""
    torch = _torch()
    if len({id(r) for r in runs}) != len(runs):
        raise ValueError("run_batch: every run must be a distinct object")
    lib = nat.load()
    descs = (_Run * len(runs))()
    setups = []
    for i, lz in enumerate(runs):
        if not lz.initialized:
            lz.prepare_symmetrization()
        if isinstance(lz, QSpaceLanczos):
            ro = True if reorth is None else bool(reorth)
            if lz._psi_size is None or lz.psi is None or len(lz.psi) != lz._psi_size:
                raise ValueError("run %d: prepare a perturbation first (prepare_mode_q)" % i)
            setup = lz._ft_setup(n_iter, 1 if ro else 0)
        else:
            ro = bool(lz.full_reorth) if reorth is None else bool(reorth)
            psi = np.asarray(lz.psi)
            if psi.size == 0 or not np.any(psi):
                raise ValueError("run %d: prepare a perturbation first" % i)
            setup = lz._ft_setup(n_iter, lz.use_wigner, 1 if ro else 0)
        setups.append(setup)
        d = descs[i]
        d.kind = setup["kind"]
        d.ctx = setup["ctx"].value if hasattr(setup["ctx"], "value") else setup["ctx"]
        d.basis_Q = lz._Qd.data_ptr()
        d.basis_P = lz._Pd.data_ptr()
        d.capacity = setup["cap"]
        d.start_step = setup["start"]
        d.n_iter = n_iter
        d.run_simm = setup["run_simm"]
        d.precision = setup["precision"]
        d.reorth = setup["reorth"]
        d.hist = nat.dp(setup["hist"])
    torch.cuda.synchronize()        # the basis rows written above are on torch's stream
    rc = lib.tdscha_lanczos_run_batch(descs, len(runs))
    for i, lz in enumerate(runs):
        d = descs[i]
        lz._ft_collect(setups[i]["hist"], setups[i]["start"], d.steps_done, bool(d.converged))
        if verbose:
            print("run %d: %d steps%s" % (i, d.steps_done, ", converged" if d.converged else ""))
    nat.check(rc)
    return [(d.steps_done, bool(d.converged), d.status) for d in descs]
