"""KPM oracle (oracle/qspace.py) pinned against the reference's own Lanczos
run, and the host-side KPM logic of tdscha_gb300.QSpaceKPM (no GPU)."""
import numpy as np

import oracle.qspace as oq
from tdscha_gb300.QSpaceKPM import QSpaceKPM


def test_kpm_moments_equal_reference_lanczos_tridiagonal(golden):
    """mu_n = e0^T T_n(T~) e0 of the reference's 50-step Wigner run_FT (one
    q-point, where the q-space operator is the reference's Wigner operator)
    equals the oracle's Chebyshev recurrence for n <= 2*50."""
    d = golden("runft_m21_n1000.npz")
    X, Y, w, rho, T, R1 = d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), d["R1"]
    ol = oq.OracleQSpaceLanczos(X[None].astype(complex), Y[None].astype(complex), w[:, None],
                                rho, T, np.array([0]), 0)
    psi = np.zeros(ol.P, complex)
    psi[:len(R1)] = R1
    lmin, lmax = oq.kpm_bounds(w[:, None], np.ones((len(w), 1), bool))
    mom, norm, _, _ = oq.kpm_moments(ol.apply_full_L, psi, ol.mask_dot_wigner(), 90, lmin, lmax)
    ref = oq.moments_from_tridiagonal(d["wigner/a"], d["wigner/b"], d["wigner/c"], 90, lmin, lmax)
    np.testing.assert_allclose(mom, ref, atol=1e-13)
    np.testing.assert_allclose(norm, np.linalg.norm(R1), rtol=1e-15)


def test_spectral_function_and_io(tmp_path):
    k = QSpaceKPM()
    rng = np.random.default_rng(0)
    k.kpm_n_moments = 30
    k.kpm_moments = rng.standard_normal(30) * np.exp(-np.arange(30) / 10)
    k.kpm_moments[0] = 1.0
    k.kpm_vector_norm = 1.3
    k.kpm_lambda_min, k.kpm_lambda_max = -2e-4, 1e-5
    k.kpm_rescale_a = 0.5 * (k.kpm_lambda_max - k.kpm_lambda_min)
    k.kpm_rescale_b = 0.5 * (k.kpm_lambda_max + k.kpm_lambda_min)
    w = np.linspace(0, 0.015, 300)
    got = k.get_spectral_function_KPM(w)
    ref = oq.kpm_spectral(w, k.kpm_moments, 1.3, k.kpm_lambda_min, k.kpm_lambda_max)
    # the host sums the series by Clenshaw's recurrence, the oracle forward:
    # equal to rounding, relative to the largest value
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(QSpaceKPM._jackson_kernel(30), oq.jackson_kernel(30))
    f = str(tmp_path / "m.txt")
    k.save_kpm(f)
    k2 = QSpaceKPM()
    k2.load_kpm(f)
    np.testing.assert_allclose(k2.get_spectral_function_KPM(w), got, rtol=1e-12)
    g = k.get_spectral_function_KPM(w, regularization="none")
    assert np.all(np.isfinite(g))
