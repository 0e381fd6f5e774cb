"""Import the reference `tdscha.DynamicalLanczos` without its physics deps.

Fixture-generation helper (test infrastructure only). It is used by
`make_golden.py` in a checkout that has the reference tree; nothing on the
product path, in `smoke()` or in `bench.py` imports it.

The reference module imports cellconstructor, sscha and spglib at module
level (Modules/DynamicalLanczos.py:22-35) and `sscha_HP_odd` (the compiled
C kernels, CModules/odd_corr_module.c). The stubs below provide only the
names the Lanczos driver touches on the perturbation-average path; the
C module is the reference's own, compiled from source by oracle/build_ref.sh.
"""
import contextlib
import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
# the reference checkout: $TDSCHA_REFERENCE_ROOT, else "reference" beside this repository
REF_ROOT = os.environ.get("TDSCHA_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(REPO), "reference"))


def _stub(name, **attrs):
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def _go_parallel(func, items, reduce_op=None):
    res = [func(x) for x in items]
    if reduce_op == "+":
        out = res[0]
        for r in res[1:]:
            out = out + r
        return out
    return res


def load_reference():
    """Return the reference `tdscha.DynamicalLanczos` module (stubbed deps)."""
    if "tdscha.DynamicalLanczos" in sys.modules:
        return sys.modules["tdscha.DynamicalLanczos"]
    if not os.path.isdir(os.path.join(REF_ROOT, "Modules")):
        raise ImportError("reference tree not found at %s" % REF_ROOT)

    ref_so_dir = os.path.join(REPO, "oracle", "_ref")
    if ref_so_dir not in sys.path:
        sys.path.insert(0, ref_so_dir)
    importlib.import_module("sscha_HP_odd")

    settings = _stub(
        "cellconstructor.Settings",
        GetNProc=lambda: 1,
        am_i_the_master=lambda: True,
        barrier=lambda: None,
        broadcast=lambda x: x,
        GoParallel=_go_parallel,
    )
    cc = _stub("cellconstructor", Settings=settings)
    cc.Units = _stub("cellconstructor.Units", RY_TO_CM=109691.40235)
    cc.Phonons = _stub("cellconstructor.Phonons", __EPSILON_W__=1e-8)
    cc.symmetries = _stub("cellconstructor.symmetries")
    cc.Methods = _stub("cellconstructor.Methods")
    sscha = _stub("sscha")
    sscha.Ensemble = _stub("sscha.Ensemble", Bohr=1.889725989)
    sscha.Parallel = _stub("sscha.Parallel", pprint=lambda *a, **k: None,
                           am_i_the_master=lambda: True)
    _stub("spglib")

    pkg = types.ModuleType("tdscha")
    pkg.__path__ = [os.path.join(REF_ROOT, "Modules")]
    sys.modules["tdscha"] = pkg
    par = importlib.import_module("tdscha.Parallel")
    par.pprint = lambda *a, **k: None
    return importlib.import_module("tdscha.DynamicalLanczos")


def make_reference_lanczos(ens, use_wigner, mode=1):
    """Build a bare reference `Lanczos` from a synthetic ensemble dict.

    Mirrors what `Lanczos.__init__` + `init()` leave behind
    (Modules/DynamicalLanczos.py:300-483, :694-732 and :795-836).
    """
    import scipy.sparse.linalg

    DL = load_reference()
    lanc = DL.Lanczos()
    M = int(ens["X"].shape[1])
    lanc.T = float(ens["T"])
    lanc.w = np.ascontiguousarray(ens["w"], dtype=np.float64)
    lanc.n_modes = M
    lanc.N = int(ens["X"].shape[0])
    lanc.rho = np.ascontiguousarray(ens["rho"], dtype=np.float64)
    lanc.N_eff = float(np.sum(lanc.rho))
    lanc.X = np.ascontiguousarray(ens["X"], dtype=np.float64)
    lanc.Y = np.ascontiguousarray(ens["Y"], dtype=np.float64)
    lanc.m = np.ones(M, dtype=np.float64)
    lanc.pols = np.eye(M)
    lanc.use_wigner = bool(use_wigner)
    lanc.mode = mode
    lanc.verbose = False
    lanc.psi = np.zeros(M + M * (M + 1), dtype=np.float64)
    syms = ens.get("symmetries")
    if syms is None:
        lanc.symmetries = [np.ones((1, 1, 1), dtype=np.double)] * M
        lanc.N_degeneracy = np.ones(M, dtype=np.intc)
        lanc.degenerate_space = [np.array([i], dtype=np.intc) for i in range(M)]
        lanc.sym_block_id = np.arange(M).astype(np.intc)
    else:
        lanc.symmetries = [np.ascontiguousarray(s, dtype=np.double) for s in syms]
        lanc.degenerate_space = [np.array(b, dtype=np.intc) for b in ens["degenerate_space"]]
        lanc.N_degeneracy = np.array([len(b) for b in lanc.degenerate_space], dtype=np.intc)
        lanc.sym_block_id = np.ascontiguousarray(ens["sym_block_id"], dtype=np.intc)
    lanc.n_syms = lanc.symmetries[0].shape[0]
    lanc.initialized = True

    def L_transp(psi):
        return lanc.apply_full_L(psi, transpose=True)

    lanc.L_linop = scipy.sparse.linalg.LinearOperator(
        shape=(len(lanc.psi), len(lanc.psi)),
        matvec=lanc.apply_full_L, rmatvec=L_transp, dtype=np.double)
    return lanc


@contextlib.contextmanager
def static_adapter(lanc):
    """Route the reference's static-response call to its own C module.

    apply_anharmonic_static (Modules/DynamicalLanczos.py:3369-3430) still passes
    the 13-argument form (..., T, apply_d4, symmetries, N_degeneracy,
    deg_space, f, d2v) while GetPerturbAverageSym parses 15 arguments
    (CModules/odd_corr_module.c:519-521: ..., T, apply_D4, N_syms, symmetries,
    n_deg, degenerate_space, blocks_ids, f, d2v), so the reference's static path
    raises TypeError as shipped.  Inside this context (fixture generation only)
    13-argument calls are forwarded with the lanczos object's block tables and
    15-argument calls pass through, so the rest of the reference's static path
    -- apply_L1_static, the Y1 scaling, the output repack,
    Tools.minimum_residual_algorithm, run_hessian_calculation and StaticHessian
    -- runs unchanged.  Valid for one-mode blocks (identity symmetries), the
    only layout whose deg_space loop (:3398-3409) works."""
    import sscha_HP_odd as real
    DL = load_reference()

    class _Adapter:
        @staticmethod
        def GetPerturbAverageSym(*args):
            if len(args) == 15:
                return real.GetPerturbAverageSym(*args)
            X, Y, w, rho, R1, Y1, T, apply_d4, symmetries, n_deg, deg_space, f, d2v = args
            return real.GetPerturbAverageSym(X, Y, w, rho, R1, Y1, T, apply_d4,
                                             int(symmetries[0].shape[0]), symmetries, n_deg,
                                             lanc.degenerate_space, lanc.sym_block_id, f, d2v)

    mods = [DL] + [m for n, m in sys.modules.items() if n == "tdscha.StaticHessian"]
    saved = [m.sscha_HP_odd for m in mods]
    for m in mods:
        m.sscha_HP_odd = _Adapter
    try:
        yield DL
    finally:
        for m, v in zip(mods, saved):
            m.sscha_HP_odd = v
