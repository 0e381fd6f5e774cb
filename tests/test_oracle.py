"""The oracle (oracle/) against fixtures produced by the reference itself."""
import numpy as np
import pytest

import oracle


def _syms(d, name, M):
    S = int(d[name + "/S"])
    n_deg = d[name + "/n_deg"]
    deg = d[name + "/deg_space"]
    sym = d[name + "/sym"]
    spaces, blocks, o, os_ = [], [], 0, 0
    for nd in n_deg:
        spaces.append(deg[o:o + nd])
        blocks.append(sym[os_:os_ + S * nd * nd].reshape(S, nd, nd))
        o += nd
        os_ += S * nd * nd
    return blocks, spaces, d[name + "/blocks_ids"]


CASES = ["m21_n200_s1", "m12_n30_s48", "m9_n7_s8", "m1_n5_s1"]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("d4", [0, 1])
def test_perturb_averages_bit_exact(golden, name, d4):
    d = golden("perturb_averages.npz")
    M = d[name + "/X"].shape[1]
    blocks, spaces, bid = _syms(d, name, M)
    f, d2v = oracle.perturb_averages(d[name + "/X"], d[name + "/Y"], d[name + "/w"],
                                     d[name + "/rho"], d[name + "/R1"], d[name + "/Y1"],
                                     float(d[name + "/T"]), d4, blocks, spaces, bid)
    key = "%s_d4%d" % (name, d4)
    # single-threaded restatement: same operation order as the reference
    np.testing.assert_array_equal(f, d[key + "/f"])
    np.testing.assert_array_equal(d2v, d[key + "/d2v"])


def test_perturb_averages_threads_split(golden):
    d = golden("perturb_averages.npz")
    name = "m21_n200_s1"
    M = d[name + "/X"].shape[1]
    blocks, spaces, bid = _syms(d, name, M)
    f, d2v = oracle.perturb_averages(d[name + "/X"], d[name + "/Y"], d[name + "/w"],
                                     d[name + "/rho"], d[name + "/R1"], d[name + "/Y1"],
                                     float(d[name + "/T"]), 1, blocks, spaces, bid, n_threads=5)
    np.testing.assert_allclose(f, d[name + "_d41/f"], rtol=1e-12, atol=1e-14 * np.abs(f).max())
    np.testing.assert_allclose(d2v, d[name + "_d41/d2v"], rtol=1e-12,
                               atol=1e-14 * np.abs(d2v).max())


def _ens(d):
    ens = dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"]))
    if "S" in d:
        blocks, spaces, bid = _syms({("x/" + k): v for k, v in d.items()}, "x", d["X"].shape[1])
        ens.update(symmetries=blocks, degenerate_space=spaces, sym_block_id=bid)
    return ens


RUNS = [("runft_m21_n1000.npz", "bilanczos", False, True),
        ("runft_m21_n1000.npz", "wigner", True, True),
        ("runft_m21_n1000.npz", "wigner_nod4", True, False),
        ("runft_m12_n120_s48.npz", "bilanczos", False, True),
        ("runft_m12_n120_s48.npz", "wigner", True, True)]


@pytest.mark.parametrize("fname,tag,wig,d4", RUNS)
def test_run_FT_matches_reference(golden, fname, tag, wig, d4):
    d = golden(fname)
    ol = oracle.OracleLanczos(_ens(d), use_wigner=wig, apply_d4=d4)
    # one application of L and L^T
    np.testing.assert_array_equal(ol.apply_full_L(d[tag + "/psi_r"]), d[tag + "/Lpsi"])
    np.testing.assert_array_equal(ol.apply_full_L(d[tag + "/psi_r"], transpose=True),
                                  d[tag + "/LTpsi"])
    ol.prepare_perturbation_R(d["R1"])
    ol.run_FT(int(d["n_steps"]))
    for k in "abc":
        np.testing.assert_array_equal(np.array(getattr(ol, k + "_coeffs")), d[tag + "/" + k])
    G = ol.get_green_function_continued_fraction(d["wgrid"], smearing=float(d["smearing"]))
    np.testing.assert_array_equal(G, d[tag + "/G"])


def test_snte_first_coefficient(golden):
    """a_0 of the reference's own saved run (tests/test_julia/LANCZOS_STEP5.npz).

    The start vector is a unit R-sector vector on mode 10, so a_0 only sees the
    harmonic R block and the (zero) Y1-driven force: it is reproducible without
    the 384 SnTe symmetry tables that the saved file does not contain."""
    d = golden("snte_lanczos_step5.npz")
    ens = dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"]))
    ol = oracle.OracleLanczos(ens, use_wigner=bool(d["use_wigner"]))
    ol.psi = d["q0"].copy()
    ol.run_FT(1)
    np.testing.assert_allclose(ol.a_coeffs[0], d["a"][0], rtol=1e-12)


def _cf(a, b, c, w, wig, **kw):
    return oracle.continued_fraction(a, b, c, np.asarray(w, float), wig, **kw)


def test_continued_fraction_known_answers():
    """The analytic cases of the reference's tests/test_continued_fraction.py."""
    a, b, c = [3.0, 10.0], [1.0, 1.0], [1.0, 1.0]
    w = np.array([0.0])
    g = _cf(a, b, c, w, False, use_terminator=True, last_average=1, smearing=0.0)
    disc = 10.0 ** 2 - 4
    gm = (10.0 - np.sqrt(disc + 0j)) / 2
    np.testing.assert_allclose(g[0], 1.0 / (3.0 - gm), rtol=1e-10)
    gw = _cf(a, b, c, w, True, use_terminator=True, last_average=1, smearing=0.0)
    ew = 1.0 / (3.0 - gm)
    np.testing.assert_allclose(gw[0], -ew.real + 1j * ew.imag, rtol=1e-10)
    a2, b2 = [1.0, 2.0, 3.0, 4.0, 5.0], [0.5, 0.6, 0.7, 0.8, 0.9]
    w2 = np.array([1.0])
    g0 = _cf(a2, b2, b2, w2, False, last_average=2, smooth_ramp=0)
    g3 = _cf(a2, b2, b2, w2, False, last_average=2, smooth_ramp=3)
    assert np.isfinite(g3[0]) and not np.allclose(g0, g3, rtol=1e-6)
    n1 = _cf(a2, b2, b2, w2, False, use_terminator=False, smearing=0.01, smooth_ramp=0)
    n2 = _cf(a2, b2, b2, w2, False, use_terminator=False, smearing=0.01, smooth_ramp=5)
    np.testing.assert_allclose(n1, n2, rtol=1e-14)


def _reference_module():
    """The reference's own C module, compiled from its sources into oracle/_ref by
    oracle/build_ref.sh (present only where the reference tree was available)."""
    import importlib
    import os
    import sys
    ref = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                       "_ref")
    if not os.path.isdir(ref):
        pytest.skip("oracle/_ref not built (no reference tree here)")
    if ref not in sys.path:
        sys.path.insert(0, ref)
    try:
        return importlib.import_module("sscha_HP_odd")
    except ImportError:
        pytest.skip("oracle/_ref holds no importable reference module")


@pytest.mark.parametrize("M,N,S", [(189, 6, 48), (573, 3, 1)])
def test_oracle_matches_reference_module_at_config_shapes(M, N, S):
    """The oracle against the reference's compiled module, run live, on slices of
    the benchmark shapes (189 modes with 48 images; 573 modes): bit-exact."""
    import contextlib
    import io
    from tdscha_gb300.synthetic import make_ensemble, random_R1, random_sym
    ref = _reference_module()
    ens = make_ensemble(M, N, seed=7 + M, n_syms=S, rho_sigma=0.1)
    if S > 1:
        syms, spaces, bid = ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]
    else:
        syms, spaces, bid = oracle.identity_symmetries(M)
    R1, Y1 = random_R1(M, 3), random_sym(M, 4, scale=1e-3)
    n_deg = np.array([len(b) for b in spaces], dtype=np.intc)
    for d4 in (0, 1):
        f_ref, d_ref = np.zeros(M), np.zeros((M, M))
        with contextlib.redirect_stdout(io.StringIO()):
            ref.GetPerturbAverageSym(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1, ens["T"],
                                     d4, int(syms[0].shape[0]), syms, n_deg, spaces,
                                     np.asarray(bid, dtype=np.intc), f_ref, d_ref)
        f, d2v = oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                         ens["T"], d4, syms, spaces, bid)
        np.testing.assert_array_equal(f, f_ref)
        np.testing.assert_array_equal(d2v, d_ref)


@pytest.mark.parametrize("M,N,S,wig", [(60, 300, 1, False), (60, 300, 1, True),
                                        (24, 60, 48, True)])
def test_oracle_run_FT_matches_reference_live(M, N, S, wig):
    """The oracle's Lanczos driver against the reference's own run_FT (its Python
    driver with stubbed physics modules and its compiled C module), run live in
    this test on shapes beyond the fixtures: coefficients bit-exact over 12 steps."""
    import os
    import sys
    _reference_module()
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    before = set(sys.modules)
    sys.path.insert(0, here)
    try:
        from ref_harness import load_reference, make_reference_lanczos
        try:
            load_reference()
        except ImportError as e:
            pytest.skip(str(e))
        _live_run_FT(make_reference_lanczos, M, N, S, wig)
    finally:
        sys.path.remove(here)
        # drop the reference modules and the physics stubs the harness installed
        for name in set(sys.modules) - before:
            if name.split(".")[0] in ("tdscha", "cellconstructor", "sscha", "spglib",
                                      "ref_harness"):
                del sys.modules[name]


def _live_run_FT(make_reference_lanczos, M, N, S, wig):
    import contextlib
    import io
    from tdscha_gb300.synthetic import make_ensemble, random_R1
    ens = make_ensemble(M, N, seed=3 + M, n_syms=S, rho_sigma=0.1)
    R1 = random_R1(M, 4)
    lanc = make_reference_lanczos(ens, use_wigner=wig)
    lanc.psi[:] = 0
    lanc.psi[:M] = R1
    lanc.perturbation_modulus = R1.dot(R1)
    with contextlib.redirect_stdout(io.StringIO()):
        lanc.run_FT(12, verbose=False)
    ol = oracle.OracleLanczos(ens, use_wigner=wig)
    ol.prepare_perturbation_R(R1)
    ol.run_FT(12)
    for k in "abc":
        np.testing.assert_array_equal(np.array(getattr(ol, k + "_coeffs")),
                                      np.array(getattr(lanc, k + "_coeffs")))
