"""Static response on the GPU (csrc/static.cu, Lanczos.apply_*_static,
run_hessian_calculation, StaticHessian) against the reference's own static
path (tests/golden/static_m12_n800.npz) and the oracle."""
import numpy as np
import pytest

import oracle
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.StaticHessian import StaticHessian
from tdscha_gb300.synthetic import make_ensemble

pytestmark = pytest.mark.gpu


def _lanczos(d, precision="fp64", syms=None):
    lz = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), precision=precision)
    if syms is None:
        lz.init(use_symmetries=False)
    else:
        lz.init(symmetries=syms)
    return lz


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(b).max()


def test_static_parts_match_reference(gpu_lib, golden):
    d = golden("static_m12_n800.npz")
    lz = _lanczos(d)
    psi = d["psi_s"]
    assert _rel(lz.apply_L1_static(psi), d["L1"]) < 1e-15
    assert _rel(lz.apply_L1_static(psi, inverse=True, power=0.5), d["L1_inv_half"]) < 1e-14
    lz.psi = psi.copy()
    assert _rel(lz.apply_anharmonic_static(), d["anh"]) < 1e-11
    lz.ignore_v4 = True
    lz.psi = psi.copy()
    assert _rel(lz.apply_anharmonic_static(), d["anh_nod4"]) < 1e-11
    with pytest.raises(AssertionError):
        lz.apply_L1_static(psi[:-1])


def test_run_hessian_calculation_matches_reference(gpu_lib, golden):
    d = golden("static_m12_n800.npz")
    lz = _lanczos(d)
    H = lz.run_hessian_calculation(verbose=False)
    assert _rel(H, d["hessian"]) < 1e-8
    H2 = lz.run_hessian_calculation(verbose=False, use_preconditioning=False)
    assert _rel(H2, d["hessian_noprec"]) < 1e-8


def test_static_hessian_matches_reference(gpu_lib, golden):
    d = golden("static_m12_n800.npz")
    sh = StaticHessian()
    sh.lanczos = _lanczos(d)
    sh.init(verbose=False)
    sh.run(int(d["sh_steps"]), threshold=1e-8, algorithm="cg-prec")
    assert _rel(sh.vector, d["sh_vector"]) < 1e-8
    assert _rel(sh.retrieve_hessian(noq=True), d["sh_hessian"]) < 1e-8


def test_static_hessian_apply_matches_loops(gpu_lib, golden):
    """apply_L through the expand / batched operator / collect kernels equals
    the per-row loop of StaticHessian.apply_L written out with the oracle."""
    d = golden("static_m12_n800.npz")
    sh = StaticHessian()
    sh.lanczos = _lanczos(d)
    sh.init(verbose=False)
    M = sh.lanczos.n_modes
    rng = np.random.default_rng(5)
    v = rng.standard_normal(len(sh.vector))
    got = sh.apply_L(v)
    ol = oracle.OracleLanczos(dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"])))
    G, W = sh.get_G_W(v)
    iu = np.triu_indices(M)
    for i in range(M):
        row = np.concatenate([G[i, :], W[i][iu]])
        out = oracle.static_L1(d["w"], float(d["T"]), row) + oracle.static_anharmonic(ol, row)
        G[i, :] = out[:M]
        W[i] = 0
        W[i][iu] = out[M:]
        W[i].T[iu] = out[M:]
    ref = sh.get_vector(G, W)
    assert _rel(got, ref) < 1e-11
    pre = sh.apply_L(v, preconditioner=True)
    G, W = sh.get_G_W(v)
    for i in range(M):
        row = np.concatenate([G[i, :], W[i][iu]])
        out = oracle.static_L1(d["w"], float(d["T"]), row, inverse=True, power=0.5)
        G[i, :] = out[:M]
        W[i][iu] = out[M:]
        W[i].T[iu] = out[M:]
    assert _rel(pre, sh.get_vector(G, W)) < 1e-14


def test_static_symmetric_and_mixed(gpu_lib):
    ens = make_ensemble(12, 400, seed=8, n_syms=48, rho_sigma=0.1, w_min_cm=40000.0,
                        w_max_cm=110000.0)
    syms = (ens["symmetries"], ens["degenerate_space"])
    lz = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"])
    lz.init(symmetries=syms)
    ol = oracle.OracleLanczos(ens)
    rng = np.random.default_rng(9)
    psi = rng.standard_normal(12 + 78)
    lz.psi = psi.copy()
    got = lz.apply_anharmonic_static()
    ref = oracle.static_anharmonic(ol, psi)
    assert _rel(got, ref) < 1e-11
    # tensor-core averages
    lz.precision = "mixed"
    lz.psi = psi.copy()
    assert _rel(lz.apply_anharmonic_static(), ref) < 2e-5
