"""GPU KPM (tdscha_qkpm_run via QSpaceKPM) against the oracle."""
import numpy as np
import pytest

import oracle.qspace as oq
from tdscha_gb300.QSpaceKPM import QSpaceKPM
from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
from tdscha_gb300.synthetic import make_qspace_ensemble

pytestmark = pytest.mark.gpu


def _setup(dims=(3, 1, 1), nb=3, N=200, iq=0, seed=5):
    e = make_qspace_ensemble(dims, nb, N, seed=seed, T=250.0, dispersion=0.3, rho_sigma=0.2)
    k = QSpaceKPM.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], q_points=e["q"])
    k.init(use_symmetries=False)
    k.prepare_mode_q(iq, 1)
    o = oq.OracleQSpaceLanczos(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], k.q_pair_map, iq)
    return e, k, o


@pytest.mark.parametrize("n_moments", [2, 3, 40, 41])
def test_kpm_moments_match_oracle(gpu_lib, n_moments):
    e, k, o = _setup()
    k.run_KPM(n_moments, verbose=False)
    psi = np.zeros(o.P, complex)
    psi[1] = 1
    lmin, lmax = oq.kpm_bounds(e["w_q"], np.ones_like(e["w_q"], bool), 1.2)
    mom, norm, vm, v = oq.kpm_moments(o.apply_full_L, psi, o.mask_dot_wigner(), n_moments,
                                      lmin, lmax)
    np.testing.assert_allclose(k.kpm_moments, mom, atol=1e-11)
    np.testing.assert_allclose(k.kpm_chebyshev_v, v, atol=1e-10 * np.abs(v).max())
    np.testing.assert_allclose(k.kpm_chebyshev_vm, vm, atol=1e-10 * np.abs(vm).max())
    w = np.linspace(0, 3e-3, 200)
    np.testing.assert_allclose(k.get_spectral_function_KPM(w),
                               oq.kpm_spectral(w, mom, norm, lmin, lmax), rtol=1e-8, atol=1e-6)


@pytest.mark.parametrize("first", [1, 20, 21])
def test_kpm_continuation(gpu_lib, tmp_path, first):
    e, k, o = _setup((2, 2, 1), 3, 150, iq=3)
    k.run_KPM(first, verbose=False)
    k.save_status(str(tmp_path / "kpm"))
    k2 = QSpaceKPM.from_qspace_lanczos(k)
    k2.load_status(str(tmp_path / "kpm"))
    k2.run_KPM(44, verbose=False)
    k3 = QSpaceKPM.from_qspace_lanczos(k)
    k3.run_KPM(44, verbose=False)
    np.testing.assert_allclose(k2.kpm_moments, k3.kpm_moments, atol=1e-11)


def test_kpm_single_q_point_reference_pin(gpu_lib, golden):
    """One q-point: GPU moments equal those of the reference's own 50-step
    Wigner Lanczos tridiagonal (tests/golden/runft_m21_n1000.npz)."""
    d = golden("runft_m21_n1000.npz")
    X, Y, w, rho, T, R1 = d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), d["R1"]
    k = QSpaceKPM.from_arrays(X[None].astype(complex), Y[None].astype(complex), w[:, None], rho, T)
    k.init(use_symmetries=False)
    k.build_q_pair_map(0)
    k.reset_q()
    k.psi[:len(R1)] = R1
    k.run_KPM(90, verbose=False)
    lmin, lmax = oq.kpm_bounds(w[:, None], np.ones((len(w), 1), bool))
    ref = oq.moments_from_tridiagonal(d["wigner/a"], d["wigner/b"], d["wigner/c"], 90, lmin, lmax)
    np.testing.assert_allclose(k.kpm_moments, ref, atol=1e-12)


def test_from_qspace_lanczos_shares_data(gpu_lib):
    e, k, o = _setup()
    ql = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], q_points=e["q"])
    ql.init(use_symmetries=False)
    ql.prepare_mode_q(0, 1)
    k2 = QSpaceKPM.from_qspace_lanczos(ql)
    k2.run_KPM(12, verbose=False)
    k.run_KPM(12, verbose=False)
    np.testing.assert_allclose(k2.kpm_moments, k.kpm_moments, atol=1e-13)
    assert k.estimate_kpm_steps(5.0) >= 8
