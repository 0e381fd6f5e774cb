"""Host-side logic of the drop-in API that needs no GPU."""
import numpy as np
import pytest

from tdscha_gb300 import sscha_HP_odd
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.synthetic import make_ensemble, oh_group, random_R1


def test_shim_rejects_mode_mismatch():
    X = np.zeros((4, 3))
    with pytest.raises(ValueError, match="N_modes"):
        sscha_HP_odd.GetPerturbAverageSym(X, X, np.ones(4), np.ones(4), np.zeros(3),
                                          np.zeros((3, 3)), 300.0, 1, 1,
                                          [np.ones((1, 1, 1))] * 3, np.ones(3, np.intc),
                                          [np.array([i], np.intc) for i in range(3)],
                                          np.arange(3, dtype=np.intc), np.zeros(3),
                                          np.zeros((3, 3)))


def test_shim_rejects_bad_apply_d4():
    X = np.zeros((4, 3))
    with pytest.raises(ValueError, match="apply_D4"):
        sscha_HP_odd.GetPerturbAverageSym(X, X, np.ones(3), np.ones(4), np.zeros(3),
                                          np.zeros((3, 3)), 300.0, 3, 1,
                                          [np.ones((1, 1, 1))] * 3, np.ones(3, np.intc),
                                          [np.array([i], np.intc) for i in range(3)],
                                          np.arange(3, dtype=np.intc), np.zeros(3),
                                          np.zeros((3, 3)))


def test_run_rejects_zero_start_vector():
    ens = make_ensemble(6, 20, seed=1)
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"])
    lanc.init(use_symmetries=False)
    with pytest.raises(ValueError, match="perturbation"):
        lanc.run_FT(3)


def test_symmetric_lanczos_needs_wigner():
    ens = make_ensemble(6, 20, seed=1)
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"],
                               use_wigner=False)
    lanc.init(use_symmetries=False)
    lanc.prepare_perturbation(random_R1(6), masses_exp=0)
    with pytest.raises(NotImplementedError):
        lanc.run_FT(3, run_simm=True)


def test_prepare_perturbation_modulus():
    ens = make_ensemble(6, 20, seed=1)
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"])
    lanc.init(use_symmetries=False)
    v = random_R1(6) * 3
    lanc.prepare_perturbation(v, masses_exp=0)
    assert np.isclose(lanc.perturbation_modulus, v.dot(v))
    lanc.prepare_mode(2)
    assert lanc.psi[2] == 1 and lanc.perturbation_modulus == 1


def test_mask_dot_and_chi_match_oracle():
    import oracle
    ens = make_ensemble(5, 10, seed=2)
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"])
    ol = oracle.OracleLanczos(ens)
    np.testing.assert_array_equal(lanc.mask_dot_wigner(), ol.mask_dot_wigner())
    cm, cp = ol._chi_matrices()
    np.testing.assert_array_equal(lanc.get_chi_minus(), cm)
    np.testing.assert_array_equal(lanc.get_chi_plus(), cp)


def test_oh_group_closed():
    G = oh_group()
    assert len(G) == 48
    keys = {tuple(np.round(g, 6).ravel()) for g in G}
    for a in G:
        for b in G:
            assert tuple(np.round(a @ b, 6).ravel()) in keys


def test_synthetic_deterministic_and_tables():
    e1 = make_ensemble(12, 30, seed=5, n_syms=48, rho_sigma=0.1)
    e2 = make_ensemble(12, 30, seed=5, n_syms=48, rho_sigma=0.1)
    np.testing.assert_array_equal(e1["X"], e2["X"])
    np.testing.assert_array_equal(e1["Y"], e2["Y"])
    assert len(e1["symmetries"]) == 4 and e1["symmetries"][0].shape == (48, 3, 3)
    np.testing.assert_allclose(e1["symmetries"][0][0], np.eye(3))
    # the weighted mean force is removed
    np.testing.assert_allclose((e1["rho"][:, None] * e1["Y"]).sum(0), 0, atol=1e-10)


def test_save_load_status_roundtrip(tmp_path):
    ens = make_ensemble(4, 8, seed=3)
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"])
    lanc.init(use_symmetries=False)
    lanc.a_coeffs = [1.0, 2.0]
    lanc.b_coeffs = [0.5]
    lanc.c_coeffs = [0.25]
    lanc.s_norm = [1.0, 0.3]
    lanc.basis_Q = [np.ones(lanc.psi.size), np.zeros(lanc.psi.size)]
    lanc.basis_P = [np.ones(lanc.psi.size), np.zeros(lanc.psi.size)]
    f = str(tmp_path / "st")
    lanc.save_status(f)
    other = Lanczos()
    other.load_status(f)
    assert other.a_coeffs == [1.0, 2.0] and other.c_coeffs == [0.25]
    np.testing.assert_array_equal(other.X, lanc.X)
    assert len(other.basis_Q) == 2 and other.use_wigner is True
    # the reference's key set
    keys = set(np.load(f + ".npz", allow_pickle=True).files)
    for k in ("T", "nat", "m", "w", "pols", "n_modes", "ignore_v3", "ignore_v4", "N", "rho", "X",
              "Y", "psi", "a_coeffs", "b_coeffs", "c_coeffs", "basis_Q", "basis_P", "s_norm",
              "krilov_basis", "arnoldi_matrix", "reverse", "shift", "perturbation_modulus",
              "use_wigner", "ignore_small_w", "sym_julia", "deg_julia", "n_syms"):
        assert k in keys


def test_unsymmetrised_tables_match_general_path():
    """init(use_symmetries=False) and flatten_symmetries take a vectorised path
    for one-mode identity blocks; it must give the general path's tables."""
    from tdscha_gb300 import _native as nat
    M = 37
    e = make_ensemble(M, 50, seed=3)
    lz = Lanczos.from_arrays(e["X"], e["Y"], e["w"], e["rho"], e["T"], use_wigner=False)
    lz.init(use_symmetries=False)
    ref = Lanczos.from_arrays(e["X"], e["Y"], e["w"], e["rho"], e["T"], use_wigner=False)
    ref.set_symmetries([np.ones((1, 1, 1))] * M, [np.array([i], np.intc) for i in range(M)])
    np.testing.assert_array_equal(lz.N_degeneracy, ref.N_degeneracy)
    np.testing.assert_array_equal(lz.sym_block_id, ref.sym_block_id)
    assert lz.n_syms == ref.n_syms == 1
    fast = nat.flatten_symmetries(lz.symmetries, lz.degenerate_space)
    # general path: distinct (equal) block arrays, so the shared-table shortcut is not taken
    slow = nat.flatten_symmetries([np.ones((1, 1, 1)) for _ in range(M)], ref.degenerate_space)
    for a, b in zip(fast, slow):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
        assert np.asarray(a).dtype == np.asarray(b).dtype


def test_unsymmetrised_shim_errors():
    X = np.zeros((4, 3))
    with pytest.raises(ValueError, match="N_modes"):
        sscha_HP_odd.GetPerturbAverage(X, X, np.ones(4), np.ones(4), np.zeros(3),
                                       np.zeros((3, 3)), 300.0, 1, np.zeros(3), np.zeros((3, 3)))
    with pytest.raises(ValueError, match="apply_D4"):
        sscha_HP_odd.GetPerturbAverage(X, X, np.ones(3), np.ones(4), np.zeros(3),
                                       np.zeros((3, 3)), 300.0, 2, np.zeros(3), np.zeros((3, 3)))


def test_unsymmetrised_shim_against_reference(monkeypatch):
    """GetPerturbAverage forwards to GetPerturbAverageSym with one-mode identity
    blocks and the symmetric part of Y1; the forwarded call, evaluated by the
    oracle, equals the reference module's own GetPerturbAverage (run live where
    oracle/_ref is built) on a non-symmetric Y1."""
    import importlib
    import os
    import sys
    import oracle
    ref_dir = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                           "oracle", "_ref")
    if not os.path.isdir(ref_dir):
        pytest.skip("oracle/_ref not built (no reference tree here)")
    sys.path.insert(0, ref_dir)
    try:
        ref = importlib.import_module("sscha_HP_odd")
    except ImportError:
        pytest.skip("oracle/_ref holds no importable reference module")
    finally:
        sys.path.remove(ref_dir)
    M, N = 9, 30
    ens = make_ensemble(M, N, seed=5, rho_sigma=0.1)
    rng = np.random.default_rng(1)
    R1, Y1 = random_R1(M, 2), rng.standard_normal((M, M)) * 1e-3

    def forwarded(X, Y, w, rho, R1, Y1, T, d4, S, syms, n_deg, spaces, bid, f, d2v):
        assert S == 1 and np.array_equal(Y1, Y1.T)
        assert np.array_equal(n_deg, np.ones(M)) and np.array_equal(bid, np.arange(M))
        f[:], d2v[:] = oracle.perturb_averages(X, Y, w, rho, R1, Y1, T, d4, syms, spaces, bid)

    monkeypatch.setattr(sscha_HP_odd, "GetPerturbAverageSym", forwarded)
    for d4 in (0, 1):
        f, d2v = np.zeros(M), np.zeros((M, M))
        sscha_HP_odd.GetPerturbAverage(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                       ens["T"], d4, f, d2v)
        f_ref, d_ref = np.zeros(M), np.zeros((M, M))
        ref.GetPerturbAverage(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1, ens["T"], d4,
                              f_ref, d_ref)
        np.testing.assert_allclose(f, f_ref, rtol=0, atol=1e-14 * np.abs(f_ref).max())
        np.testing.assert_allclose(d2v, d_ref, rtol=0, atol=1e-14 * np.abs(d_ref).max())
