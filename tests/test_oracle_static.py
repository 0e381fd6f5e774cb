"""Static-response oracle (oracle/__init__.py: static_lambda, static_L1,
static_anharmonic, minimum_residual, run_hessian_calculation) pinned against
the reference's own static path (tests/golden/static_m12_n800.npz, generated
by make_golden.py through ref_harness.static_adapter)."""
import numpy as np

import oracle


def _ol(d, apply_d4=True):
    ens = dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"]))
    return oracle.OracleLanczos(ens, use_wigner=True, apply_d4=apply_d4)


def test_static_harmonic_matches_reference(golden):
    d = golden("static_m12_n800.npz")
    w, T, psi = d["w"], float(d["T"]), d["psi_s"]
    np.testing.assert_array_equal(oracle.static_L1(w, T, psi), d["L1"])
    np.testing.assert_allclose(oracle.static_L1(w, T, psi, inverse=True, power=0.5),
                               d["L1_inv_half"], rtol=1e-15, atol=0)


def test_static_anharmonic_matches_reference(golden):
    d = golden("static_m12_n800.npz")
    psi = d["psi_s"]
    np.testing.assert_allclose(oracle.static_anharmonic(_ol(d), psi), d["anh"], rtol=1e-13,
                               atol=1e-13 * np.abs(d["anh"]).max())
    np.testing.assert_allclose(oracle.static_anharmonic(_ol(d, apply_d4=False), psi),
                               d["anh_nod4"], rtol=1e-13, atol=1e-13 * np.abs(d["anh_nod4"]).max())


def test_run_hessian_calculation_matches_reference(golden):
    d = golden("static_m12_n800.npz")
    ol = _ol(d)
    H = oracle.run_hessian_calculation(ol)
    np.testing.assert_allclose(H, d["hessian"], rtol=1e-10, atol=1e-12)
    H2 = oracle.run_hessian_calculation(ol, use_preconditioning=False)
    np.testing.assert_allclose(H2, d["hessian_noprec"], rtol=1e-10, atol=1e-12)


def test_static_lambda_edge_cases():
    # equal frequencies: the derivative term is a (signed) zero at finite T
    w = np.array([0.01, 0.01, 0.02])
    lam = oracle.static_lambda(w, 300.0)
    assert np.all(np.isfinite(lam))
    lam0 = oracle.static_lambda(w, 0.0)
    iu_r, iu_c = np.triu_indices(3)
    np.testing.assert_allclose(lam0, 1 / (w[iu_c] + w[iu_r]) / (4 * w[iu_c] * w[iu_r]))
