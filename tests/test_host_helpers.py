"""Host-side Lanczos helpers against the reference's own outputs
(tests/golden/host_helpers_m9.npz, written by make_golden.py from
Modules/DynamicalLanczos.py): the Wigner change of variables
(get_alpha1_beta1_wigner / get_a1_b1_wigner), the IR and Raman perturbation
builders, the Lanczos matrix and the static frequency.  No GPU: the static
frequency's continued fraction comes from the oracle here (the product
evaluates it on the GPU; tests/test_gpu_fp64.py covers that path)."""
import numpy as np
import pytest

import oracle
from tdscha_gb300.DynamicalLanczos import Lanczos


class _Dyn:
    """The members of a dynamical matrix the IR / Raman builders read."""

    def __init__(self, ec, raman, supercell):
        self.effective_charges = ec
        self.raman_tensor = raman
        self._sc = tuple(supercell)

    def GetSupercell(self):
        return self._sc

    def GetRamanVector(self, p_in, p_out):
        return np.einsum("abc,a,b->c", self.raman_tensor, p_in, p_out)


@pytest.fixture
def case(golden):
    d = golden("host_helpers_m9.npz")
    lanc = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), pols=d["pols"],
                               m=d["m"])
    return d, lanc


@pytest.mark.parametrize("tag", ["T", "T0"])
def test_wigner_change_of_variables(case, tag):
    d, lanc = case
    lanc.T = float(d["T"]) if tag == "T" else 0.0
    lanc.psi = d["psi"].copy()
    np.testing.assert_array_equal(lanc.get_alpha1_beta1_wigner(True), d["alpha1/" + tag])
    np.testing.assert_array_equal(lanc.get_alpha1_beta1_wigner(False), d["beta1/" + tag])
    np.testing.assert_array_equal(lanc.get_a1_b1_wigner(True), d["a1/" + tag])
    np.testing.assert_array_equal(lanc.get_a1_b1_wigner(False), d["b1/" + tag])


def _check(lanc, d, key):
    M = lanc.n_modes
    np.testing.assert_allclose(lanc.psi[:M], d["psi/" + key], rtol=1e-14, atol=0)
    np.testing.assert_allclose(lanc.perturbation_modulus, d["mod/" + key], rtol=1e-13)


@pytest.mark.parametrize("with_dyn", [True, False])
def test_ir_and_raman_builders(case, with_dyn):
    d, lanc = case
    ec, raman = d["ec"], d["raman"]
    e = np.eye(3)
    if with_dyn:
        lanc.dyn = _Dyn(ec, raman, d["supercell"])
        kw_ir, kw_r = {}, {}
    else:
        # no dynamical matrix: arrays, supercell size inferred from pols
        kw_ir, kw_r = {"effective_charges": ec}, {"raman_tensor": raman}
    lanc.prepare_ir(pol_vec=e[0], **kw_ir)
    _check(lanc, d, "ir_x")
    lanc.prepare_ir(effective_charges=2 * ec, pol_vec=np.array([0.3, -0.5, 0.8]))
    _check(lanc, d, "ir_mix")
    lanc.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[1], **kw_r)
    _check(lanc, d, "raman_xy")
    lanc.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[2], mixed=True, pol_in_2=e[1],
                       pol_out_2=e[1], **kw_r)
    _check(lanc, d, "raman_mixed")
    for k in range(7):
        lanc.prepare_raman(unpolarized=k, **kw_r)
        _check(lanc, d, "raman_unpol%d" % k)
        lanc.prepare_unpolarized_raman(index=k, **kw_r)
        _check(lanc, d, "unpol%d" % k)
        assert lanc.get_prefactors_unpolarized_raman(k) == d["prefactor%d" % k]


def test_raman_sum_components(case):
    """sum_components keeps every term the reference drops (its final
    prepare_perturbation overwrites the accumulated vector)."""
    d, lanc = case
    raman = d["raman"]
    e = np.eye(3)
    lanc.prepare_raman(unpolarized=0, raman_tensor=raman, sum_components=True)
    summed = lanc.psi[:lanc.n_modes].copy()
    # (xx + yy + zz) / 3 = the unpolarised component 0 of prepare_unpolarized_raman / 3
    lanc.prepare_unpolarized_raman(index=0, raman_tensor=raman)
    np.testing.assert_allclose(summed, lanc.psi[:lanc.n_modes] / 3, rtol=1e-12, atol=1e-300)
    lanc.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[2], mixed=True, pol_in_2=e[1],
                       pol_out_2=e[1], raman_tensor=raman, sum_components=True)
    both = lanc.psi[:lanc.n_modes].copy()
    lanc.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[2], raman_tensor=raman)
    xz = lanc.psi[:lanc.n_modes].copy()
    lanc.prepare_raman(pol_vec_in=e[1], pol_vec_out=e[1], raman_tensor=raman)
    np.testing.assert_allclose(both, xz + lanc.psi[:lanc.n_modes], rtol=1e-12, atol=1e-300)


def test_builder_errors(case):
    d, lanc = case
    with pytest.raises(AssertionError):
        lanc.prepare_ir()                       # no charges, no dynamical matrix
    with pytest.raises(AssertionError):
        lanc.prepare_raman()                    # no Raman tensor
    with pytest.raises(AssertionError):       # 2 atoms x 3 x 3 cells != n_modes + 3
        lanc.prepare_ir(effective_charges=np.zeros((2, 3, 3)), n_supercell=3)
    with pytest.raises(ValueError):           # 12 coordinates are not whole cells of 9
        lanc.prepare_ir(effective_charges=np.zeros((3, 3, 3)))
    with pytest.raises(ValueError):
        lanc.prepare_raman(unpolarized=7, raman_tensor=d["raman"])
    with pytest.raises(ValueError):
        lanc.get_prefactors_unpolarized_raman(9)
    with pytest.raises(ValueError):
        lanc.run(3)


@pytest.mark.parametrize("tag", ["bi", "sym", "bi_rev"])
def test_lanczos_matrix(case, tag):
    d, lanc = case
    lanc.a_coeffs = list(d["coef_a"])
    lanc.b_coeffs = list(d["coef_b"])
    lanc.c_coeffs = [] if tag == "sym" else list(d["coef_c"])
    lanc.reverse_L, lanc.shift_value = (True, 0.7) if tag == "bi_rev" else (False, 0.0)
    np.testing.assert_array_equal(lanc.build_lanczos_matrix_from_coeffs(), d["matrix/" + tag])


@pytest.mark.parametrize("tag,wig", [("bilanczos", False), ("wigner", True)])
def test_static_frequency(case, golden, monkeypatch, tag, wig):
    d, lanc = case
    run = golden("runft_m21_n1000.npz")
    lanc.use_wigner = wig
    lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs = (list(run[tag + "/a"]), list(run[tag + "/b"]),
                                                   list(run[tag + "/c"]))
    lanc.perturbation_modulus = float(d["wstatic_modulus"])

    def cf(w, use_terminator=True, smearing=0.0):
        return oracle.continued_fraction(lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs, w,
                                         lanc.use_wigner, lanc.perturbation_modulus,
                                         use_terminator=use_terminator, smearing=smearing)

    monkeypatch.setattr(lanc, "get_green_function_continued_fraction", cf)
    for k, sm in enumerate(d["wstatic_smearing"]):
        got = lanc.get_static_frequency(float(sm))
        np.testing.assert_allclose(got, d["wstatic/%s/%d" % (tag, k)], rtol=1e-12)


def _qspace(seed=3):
    from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
    rng = np.random.default_rng(seed)
    n_q, N, nb = 2, 4, 6
    X = rng.standard_normal((n_q, N, nb)) + 1j * rng.standard_normal((n_q, N, nb))
    w_q = rng.uniform(1e-3, 3e-3, (nb, n_q))
    q, _ = np.linalg.qr(rng.standard_normal((nb, nb)) + 1j * rng.standard_normal((nb, nb)))
    pols_q = np.stack([q, np.conj(q)], axis=2)
    m = np.repeat(rng.uniform(1e3, 1e5, nb // 3), 3)
    ql = QSpaceLanczos.from_arrays(X, X.copy(), w_q, np.ones(N), 100.0,
                                   q_points=np.array([[0, 0, 0], [0.5, 0, 0]]), pols_q=pols_q, m=m)
    return ql, pols_q, m, rng


def test_qspace_ir_and_raman_at_gamma():
    """The q-space builders project on the q = 0 modes (QSpaceLanczos.py:1205-1451):
    R1 = conj(pols_q[:, :, 0])^T (v sqrt(cells) / sqrt(m)), the unpolarised terms
    summed (the q-space reference keeps every term), cells = the q grid size."""
    ql, pols_q, m, rng = _qspace()
    ec = rng.standard_normal((2, 3, 3))
    raman = rng.standard_normal((3, 3, 6))
    e = np.eye(3)
    proj = lambda v: np.conj(pols_q[:, :, 0]).T @ (v * np.sqrt(2) / np.sqrt(m))
    pol = np.array([0.2, 0.9, -0.4])
    ql.prepare_ir(effective_charges=ec, pol_vec=pol)
    np.testing.assert_allclose(ql.psi[:6], proj(np.einsum("abc,b", ec, pol).ravel()),
                               rtol=1e-13)
    rv = lambda a, b: np.einsum("abc,a,b->c", raman, e[a], e[b])
    ql.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[2], mixed=True, pol_in_2=e[1],
                     pol_out_2=e[1], raman_tensor=raman)
    np.testing.assert_allclose(ql.psi[:6], proj(rv(0, 2) + rv(1, 1)), rtol=1e-13)
    for k, want in ((0, (rv(0, 0) + rv(1, 1) + rv(2, 2)) / 3),
                    (1, (rv(0, 0) - rv(1, 1)) / np.sqrt(2)),
                    (5, rv(1, 2) * np.sqrt(3))):
        ql.prepare_raman(unpolarized=k, raman_tensor=raman)
        np.testing.assert_allclose(ql.psi[:6], proj(want), rtol=1e-12, atol=1e-300)
    ql.prepare_unpolarized_raman(index=3, raman_tensor=raman)
    np.testing.assert_allclose(ql.psi[:6], proj(rv(1, 1) - rv(2, 2)), rtol=1e-12, atol=1e-300)
    # the rest of psi stays zero: a Gamma perturbation of the R sector only
    assert not np.any(ql.psi[6:])


@pytest.mark.parametrize("tag", ["T", "T0"])
def test_l1_inverse_matches_reference(golden, tag):
    d = golden("l1_inverse_m6.npz")
    M = d["w_low"].size
    lanc = Lanczos.from_arrays(np.zeros((2, M)), np.zeros((2, M)), d["w_low"], np.ones(2),
                               float(d["T_low"]) if tag == "T" else 0.0, use_wigner=False)
    np.testing.assert_array_equal(lanc.apply_L1_inverse_FT(d["psi_r"]), d["inv/" + tag])
    np.testing.assert_array_equal(lanc.apply_L1_inverse_FT(d["psi_r"], transpose=True),
                                  d["invT/" + tag])
    with pytest.raises(AssertionError):
        lanc.apply_L1_inverse_FT(d["psi_r"][:-1])


def test_biconjugate_gradient_matches_reference(golden):
    """run_biconjugate_gradient's solves through L_linop / M_linop, with the
    operator applied by the oracle (the product applies it on the GPU), against
    the reference's own run on the same ensemble."""
    d = golden("l1_inverse_m6.npz")
    ens = dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"]))
    lanc = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), use_wigner=False)
    lanc.initialized = True
    ol = oracle.OracleLanczos(ens, use_wigner=False)
    lanc._apply_dev = lambda psi, transpose, **kw: ol.apply_full_L(np.asarray(psi), transpose)
    G_inv = lanc.run_biconjugate_gradient(verbose=False, tol=1e-12, maxiter=3000)
    np.testing.assert_allclose(G_inv, d["G_inv/bicgstab"], rtol=1e-7, atol=1e-10)
    # the BFGS form stops where the reference's does (short of the bicgstab solution)
    G_min = lanc.run_biconjugate_gradient(verbose=False, tol=1e-10, maxiter=3000,
                                          algorithm="cg-minimize")
    np.testing.assert_allclose(G_min, d["G_inv/cg-minimize"], rtol=1e-6, atol=1e-9)
    with pytest.raises(ValueError):
        lanc.run_biconjugate_gradient(verbose=False, algorithm="gmres")


def test_ir_raman_modulus_real_space_equals_qspace():
    """The reference's test_qspace/test_ir_modulus.py and test_raman_modulus.py in
    synthetic form: a two-cell supercell whose modes are the Bloch combinations of
    the q = 0 and q = 1/2 modes (Gamma translations dropped); with charges and a
    Raman tensor obeying the acoustic sum rule, the real-space and q-space
    perturbations have the same modulus."""
    from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
    rng = np.random.default_rng(21)
    nat, ncell = 2, 2
    nb = 3 * nat
    m_at = rng.uniform(1e3, 1e5, nat)
    m = np.repeat(m_at, 3)
    trans = np.zeros((nb, 3))
    for d in range(3):
        trans[d::3, d] = np.sqrt(m_at)
    e0, _ = np.linalg.qr(np.hstack([trans, rng.standard_normal((nb, nb - 3))]))
    e1, _ = np.linalg.qr(rng.standard_normal((nb, nb)))
    pols_q = np.stack([e0, e1], axis=2).astype(np.complex128)
    sc = np.hstack([np.vstack([e0, e0])[:, 3:], np.vstack([e1, -e1])]) / np.sqrt(ncell)
    M = sc.shape[1]
    N = 4
    real = Lanczos.from_arrays(rng.standard_normal((N, M)), rng.standard_normal((N, M)),
                               rng.uniform(1e-3, 3e-3, M), np.ones(N), 100.0, pols=sc,
                               m=np.tile(m, ncell))
    Xq = rng.standard_normal((ncell, N, nb)) + 0j
    ql = QSpaceLanczos.from_arrays(Xq, Xq.copy(), rng.uniform(1e-3, 3e-3, (nb, ncell)),
                                   np.ones(N), 100.0, q_points=np.array([[0, 0, 0], [0.5, 0, 0]]),
                                   pols_q=pols_q, m=m)
    A = rng.standard_normal((3, 3))
    ec = np.stack([A, -A])                               # sum over atoms = 0
    R = rng.standard_normal((3, 3, nat, 3))
    R -= R.mean(axis=2, keepdims=True)                   # sum over atoms = 0
    R = R.reshape(3, 3, nb)
    for pol in (np.array([1.0, 0, 0]), np.array([0.3, -0.4, 0.8])):
        real.prepare_ir(effective_charges=ec, pol_vec=pol)
        ql.prepare_ir(effective_charges=ec, pol_vec=pol)
        np.testing.assert_allclose(real.perturbation_modulus, ql.perturbation_modulus, rtol=1e-12)
    e = np.eye(3)
    real.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[1], raman_tensor=R)
    ql.prepare_raman(pol_vec_in=e[0], pol_vec_out=e[1], raman_tensor=R)
    np.testing.assert_allclose(real.perturbation_modulus, ql.perturbation_modulus, rtol=1e-12)
    for k in range(7):
        real.prepare_unpolarized_raman(index=k, raman_tensor=R)
        ql.prepare_unpolarized_raman(index=k, raman_tensor=R)
        np.testing.assert_allclose(real.perturbation_modulus, ql.perturbation_modulus,
                                   rtol=1e-12)


def test_free_energy_curvature_from_continued_fractions(golden, monkeypatch, tmp_path):
    """GetFreeEnergyCurvatureFromContinuedFraction against the reference's own
    output on the same coefficient tables (runs of different lengths, with and
    without mode mixing); the continued fractions come from the oracle here."""
    import tdscha_gb300.DynamicalLanczos as DLg
    d = golden("curvature_m4.npz")

    def cf(self, w, use_terminator=True, last_average=1, smearing=0.0, smooth_ramp=0):
        return oracle.continued_fraction(list(self.a_coeffs), list(self.b_coeffs),
                                         list(self.c_coeffs), w, self.use_wigner,
                                         self.perturbation_modulus,
                                         use_terminator=use_terminator,
                                         last_average=last_average, smearing=smearing)

    monkeypatch.setattr(DLg.Lanczos, "get_green_function_continued_fraction", cf)
    monkeypatch.chdir(tmp_path)
    fc = DLg.GetFreeEnergyCurvatureFromContinuedFraction(d["a_ns"], d["b_ns"], d["pols"],
                                                         d["masses"], mode_mixing=True,
                                                         use_terminator=True, last_average=3)
    np.testing.assert_allclose(fc, d["fc_mixing"], rtol=1e-10, atol=1e-10 * np.abs(fc).max())
    fc = DLg.GetFreeEnergyCurvatureFromContinuedFraction(d["a_ns"], d["b_ns"], d["pols"],
                                                         d["masses"], mode_mixing=False,
                                                         use_terminator=False, smearing=1e-3)
    np.testing.assert_allclose(fc, d["fc_diag_noterm"], rtol=1e-10,
                               atol=1e-10 * np.abs(fc).max())
    assert (tmp_path / "gf_mat.dat").exists() and (tmp_path / "fc_pols.dat").exists()
    # the corrected contraction: E F E^T with F = G^-1 from the saved fc_pols.dat
    fc_pols = np.loadtxt(tmp_path / "fc_pols.dat")
    e_m = d["pols"] * np.sqrt(d["masses"])[:, None]
    fix = DLg.GetFreeEnergyCurvatureFromContinuedFraction(
        d["a_ns"], d["b_ns"], d["pols"], d["masses"], mode_mixing=False, use_terminator=False,
        smearing=1e-3, reference_contraction=False)
    np.testing.assert_allclose(fix, e_m @ fc_pols @ e_m.T, rtol=1e-12, atol=1e-12 * np.abs(fix).max())
    assert DLg.is_julia_enabled() is False


def test_full_L_matrix_against_reference(golden, monkeypatch):
    """get_full_L_matrix against the reference's dense operators: dynamic (both
    directions, L applied by the oracle) and static (the batched static
    application replaced by the oracle's static operator)."""
    import types
    import tdscha_gb300.DynamicalLanczos as DLg
    d = golden("full_L_m4.npz")
    ens = dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"]))
    lanc = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), use_wigner=False)
    ol = oracle.OracleLanczos(ens, use_wigner=False)
    lanc._apply_dev = lambda psi, transpose, **kw: ol.apply_full_L(np.asarray(psi), transpose)
    np.testing.assert_allclose(DLg.get_full_L_matrix(lanc), d["L"], rtol=0,
                               atol=1e-12 * np.abs(d["L"]).max())
    np.testing.assert_allclose(DLg.get_full_L_matrix(lanc, transpose=True), d["LT"], rtol=0,
                               atol=1e-12 * np.abs(d["LT"]).max())
    ow = oracle.OracleLanczos(ens, use_wigner=True)
    # ARPACK on L (Wigner) from the same start vector as the reference's run_full_diag
    lw = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), use_wigner=True)
    lw._apply_dev = lambda psi, transpose, **kw: ow.apply_full_L(np.asarray(psi), transpose)
    lw.psi = d["diag_v0"].copy()
    ev, evec = lw.run_full_diag(3, discard_dyn=True, n_iter=20)
    np.testing.assert_allclose(ev, d["diag_eigvals"], rtol=1e-9)
    # eigenvectors up to sign
    sgn = np.sign(np.sum(evec * d["diag_eigvects"], axis=0))
    np.testing.assert_allclose(evec * sgn, d["diag_eigvects"], atol=1e-7)

    def unit_rows(self, i0, k, what):
        n = self._static_size()
        rows = []
        for i in range(i0, i0 + k):
            e = np.zeros(n)
            e[i] = 1.0
            out = np.zeros(n)
            if what & 1:
                out += oracle.static_L1(d["w"], float(d["T"]), e)
            if what & 2:
                out += oracle.static_anharmonic(ow, e)
            rows.append(out)
        return np.array(rows)

    lanc.use_wigner = True
    lanc._static_unit_rows = types.MethodType(unit_rows, lanc)
    for key, kw in (("L_static", {}), ("L_static_harm", {"compute_anharm": False})):
        got = DLg.get_full_L_matrix(lanc, static=True, chunk=5, **kw)
        np.testing.assert_allclose(got, d[key], rtol=0, atol=1e-11 * np.abs(d[key]).max())


def test_lehmann_representation_against_reference(golden):
    d = golden("lehmann_m3.npz")
    M = d["w"].size
    n = d["a"].size
    lanc = Lanczos.from_arrays(np.zeros((2, M)), np.zeros((2, M)), d["w"], np.ones(2),
                               float(d["T"]), pols=d["pols"], m=d["m"])
    lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs = list(d["a"]), list(d["b"]), []
    lanc.krilov_basis = [d["kb"][:, i] for i in range(n + 1)]
    lanc.arnoldi_matrix = [list(d["arnoldi"][i, :i + 1]) for i in range(n)]
    w, va, vb = d["wgrid"], d["v_a"], d["v_b"]
    tol = dict(rtol=1e-10)
    np.testing.assert_allclose(lanc.get_green_function_Lenmann(w, 1e-4, va, vb), d["gf"], **tol)
    np.testing.assert_allclose(lanc.get_green_function_Lenmann(w, 1e-4, va, vb, use_arnoldi=True),
                               d["gf_arnoldi"], **tol)
    np.testing.assert_allclose(lanc.get_spectral_function_from_Lenmann(w, 1e-4, use_arnoldi=False),
                               d["spectral"], rtol=1e-10, atol=1e-10 * np.abs(d["spectral"]).max())
    np.testing.assert_allclose(lanc.get_spectral_function_from_Lenmann(w, 1e-4),
                               d["spectral_arnoldi"], rtol=1e-10,
                               atol=1e-10 * np.abs(d["spectral_arnoldi"]).max())
    np.testing.assert_allclose(lanc.get_static_odd_fc(), d["fc"], **tol)
    lanc.krilov_basis = lanc.krilov_basis[:n]
    np.testing.assert_allclose(lanc.get_static_odd_fc(), d["fc_n"], **tol)
    lanc.c_coeffs = list(d["b"])
    with pytest.raises(AssertionError):
        lanc.get_green_function_Lenmann(w, 1e-4, va, vb)
