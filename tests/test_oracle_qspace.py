"""The q-space oracle (oracle/qspace.py) pinned against the reference, and the
host-side layout logic of tdscha_gb300.QSpaceLanczos (no GPU needed)."""
import numpy as np
import pytest

import oracle
import oracle.qspace as oq
from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
from tdscha_gb300.synthetic import make_qspace_ensemble, qgrid, translation_tables


def test_single_q_point_reproduces_reference_wigner_lanczos(golden):
    """With one q-point and real data the q-space operator is the real-space
    Wigner operator: the q-space Hermitian Lanczos (no re-orthogonalisation)
    must give the reference's own run_FT coefficients (50 steps)."""
    d = golden("runft_m21_n1000.npz")
    X, Y, w, rho, T, R1 = d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), d["R1"]
    ol = oq.OracleQSpaceLanczos(X[None].astype(complex), Y[None].astype(complex), w[:, None],
                                rho, T, np.array([0]), 0)
    ol.psi[:len(R1)] = R1
    ol.run_FT(50, reorthogonalize=False)
    for t in "abc":
        ref = d["wigner/" + t]
        got = np.array(getattr(ol, t + "_coeffs"))
        assert len(got) == len(ref)
        np.testing.assert_allclose(got, ref, rtol=1e-12)


def test_single_q_point_no_d4(golden):
    d = golden("runft_m21_n1000.npz")
    X, Y, w, rho, T, R1 = d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), d["R1"]
    ol = oq.OracleQSpaceLanczos(X[None].astype(complex), Y[None].astype(complex), w[:, None],
                                rho, T, np.array([0]), 0, apply_d4=False)
    ol.psi[:len(R1)] = R1
    ol.run_FT(50, reorthogonalize=False)
    np.testing.assert_allclose(ol.a_coeffs, d["wigner_nod4/a"], rtol=1e-12)
    np.testing.assert_allclose(ol.b_coeffs, d["wigner_nod4/b"], rtol=1e-12)


@pytest.mark.parametrize("dims,nb", [((3, 1, 1), 2), ((2, 2, 1), 2)])
def test_difference_pairing_equals_translation_averaged_real_space(dims, nb):
    """At Gamma the q-space operator with the pairing q2 - q1 = q_pert equals the
    real-space Wigner operator of the supercell averaged over all lattice
    translations (the reference's real-space oracle, pinned separately)."""
    e = make_qspace_ensemble(dims, nb, 300, seed=4)
    n_q = e["n_q"]
    blocks, spaces, bid = translation_tables(n_q, nb, e["cells"], e["dims"])
    ens = dict(X=e["X_real"], Y=e["Y_real"], w=e["w_real"], rho=e["rho"], T=e["T"],
               symmetries=blocks, degenerate_space=spaces, sym_block_id=bid)
    ol = oracle.OracleLanczos(ens, use_wigner=True)
    M = n_q * nb
    nu0 = 1
    R1 = np.zeros(M)
    R1[nu0 * n_q:(nu0 + 1) * n_q] = 1 / np.sqrt(n_q)
    ol.prepare_perturbation_R(R1)
    ol.run_FT(10)
    oql = oq.OracleQSpaceLanczos(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], np.arange(n_q), 0)
    oql.psi[nu0] = 1.0
    oql.run_FT(10, reorthogonalize=False)
    np.testing.assert_allclose(oql.a_coeffs, ol.a_coeffs, rtol=1e-10)
    np.testing.assert_allclose(oql.b_coeffs, ol.b_coeffs, rtol=1e-10)


def test_pair_maps():
    qs = qgrid((4, 1, 1))
    qsum = oq.q_pair_map_grid(qs, 0)
    np.testing.assert_array_equal(qsum, [0, 3, 2, 1])
    lz = QSpaceLanczos.from_arrays(np.zeros((4, 2, 1)), np.zeros((4, 2, 1)), np.ones((1, 4)),
                                   np.ones(2), 0.0, q_points=qs)
    lz.build_q_pair_map(0)
    np.testing.assert_array_equal(lz.q_pair_map, qsum)
    lz.build_q_pair_map(0, pairing="difference")
    np.testing.assert_array_equal(lz.q_pair_map, np.arange(4))
    lz.build_q_pair_map(2)   # q_pert = 1/2: sum rule q2 = 1/2 - q1
    np.testing.assert_array_equal(lz.q_pair_map, [2, 1, 0, 3])
    lz.build_q_pair_map(2, pairing="difference")   # q_pert = 1/2 is its own inverse
    np.testing.assert_array_equal(lz.q_pair_map, [2, 3, 0, 1])
    with pytest.raises(ValueError):
        lz.build_q_pair_map(1, pairing="difference")   # q1 -> q1 + 1/4 is no involution
    with pytest.raises(ValueError):
        lz.set_q_pair_map(0, [1, 2, 3, 0])   # not an involution


def _host_pair(dims=(3, 1, 1), nb=3, N=40, seed=3, pairing="sum", T=250.0):
    e = make_qspace_ensemble(dims, nb, N, seed=seed, T=T, dispersion=0.3)
    lz = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"],
                                   q_points=e["q"], pairing=pairing)
    valid = np.ones((nb, e["n_q"]), dtype=bool)
    valid[0, 0] = False
    lz.valid_modes_q = valid
    lz.build_q_pair_map(0)
    o = oq.OracleQSpaceLanczos(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], lz.q_pair_map, 0,
                               valid=valid)
    return e, lz, o


def test_host_layout_matches_oracle():
    e, lz, o = _host_pair()
    assert lz.get_psi_size() == o.P
    np.testing.assert_array_equal(lz.mask_dot_wigner(), o.mask_dot_wigner())
    rng = np.random.default_rng(0)
    psi = rng.standard_normal(o.P) + 1j * rng.standard_normal(o.P)
    lz.psi = psi.copy()
    o.psi = psi.copy()
    for p in range(len(lz.unique_pairs)):
        for s in "ab":
            np.testing.assert_array_equal(lz.get_block(p, s), o.get_block(p, s, psi))
            out = np.zeros_like(psi)
            lz.set_block_in_psi(p, lz.get_block(p, s), s, out)
            off = lz.get_block_offset(p, s)
            n = lz.get_block_size(p)
            np.testing.assert_array_equal(out[off:off + n], psi[off:off + n])
    np.testing.assert_allclose(lz.apply_L1_FT(), o.apply_L1_FT(psi), rtol=0, atol=0)
    for a, b in zip(lz.get_alpha1_beta1_wigner_q(True), o.alpha1_blocks(psi)):
        np.testing.assert_allclose(a, b, rtol=1e-15, atol=0)
