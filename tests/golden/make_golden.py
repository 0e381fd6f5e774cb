"""Generate the golden fixtures in this folder from the reference itself.

Run where the reference tree is available ($TDSCHA_REFERENCE_ROOT, or a
directory "reference" beside this repository) after `oracle/build_ref.sh`:

    python tests/golden/make_golden.py

Every output below comes from the reference's own code: its C module
`sscha_HP_odd` compiled from CModules/*.c, and its Python driver
Modules/DynamicalLanczos.py (imported with stubbed physics deps by
ref_harness.py).  Inputs are seeded synthetic ensembles
(tdscha_gb300/synthetic.py) stored verbatim in the fixtures, so the tests
do not depend on the generator staying unchanged.
"""
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from ref_harness import load_reference, make_reference_lanczos, static_adapter  # noqa: E402
from tdscha_gb300.synthetic import (make_ensemble, random_R1, random_sym,  # noqa: E402
                                    RY_TO_CM)


def _ident(M):
    return ([np.ones((1, 1, 1))] * M, [np.array([i], dtype=np.intc) for i in range(M)],
            np.arange(M, dtype=np.intc))


def _pack_syms(syms, deg):
    n_deg = np.array([len(b) for b in deg], dtype=np.intc)
    return (n_deg, np.concatenate([np.asarray(b, dtype=np.intc) for b in deg]),
            np.concatenate([np.asarray(s).ravel() for s in syms]))


def perturb_cases():
    load_reference()
    import sscha_HP_odd
    out = {}
    cases = [("m21_n200_s1", 21, 200, 1, 0.0, 11), ("m12_n30_s48", 12, 30, 48, 0.1, 12),
             ("m9_n7_s8", 9, 7, 8, 0.1, 13), ("m1_n5_s1", 1, 5, 1, 0.0, 14)]
    for name, M, N, S, sig, seed in cases:
        if S > 1:
            ens = make_ensemble(M, N, seed=seed, n_syms=S, rho_sigma=sig)
            syms, deg, bid = ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]
        else:
            ens = make_ensemble(M, N, seed=seed, n_syms=1, rho_sigma=sig)
            syms, deg, bid = _ident(M)
        R1 = random_R1(M, seed + 100)
        Y1 = random_sym(M, seed + 200, scale=1e-3)
        n_deg, deg_flat, sym_flat = _pack_syms(syms, deg)
        for d4 in (0, 1):
            f = np.zeros(M)
            d2v = np.zeros((M, M))
            with contextlib.redirect_stdout(io.StringIO()):
                sscha_HP_odd.GetPerturbAverageSym(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                                  ens["T"], d4, syms[0].shape[0], syms, n_deg, deg,
                                                  bid, f, d2v)
            key = "%s_d4%d" % (name, d4)
            out[key + "/f"] = f
            out[key + "/d2v"] = d2v
        for k, v in dict(X=ens["X"], Y=ens["Y"], w=ens["w"], rho=ens["rho"], T=ens["T"], R1=R1,
                         Y1=Y1, n_deg=n_deg, deg_space=deg_flat, sym=sym_flat, blocks_ids=bid,
                         S=S).items():
            out["%s/%s" % (name, k)] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "perturb_averages.npz"), **out)


def run_case(fname, M, N, S, sig, seed, n_steps, variants):
    if S > 1:
        ens = make_ensemble(M, N, seed=seed, n_syms=S, rho_sigma=sig)
    else:
        ens = make_ensemble(M, N, seed=seed, n_syms=1, rho_sigma=sig)
    R1 = random_R1(M, seed + 1)
    wgrid = np.linspace(0.0, 600.0, 200) / RY_TO_CM
    smear = 5.0 / RY_TO_CM
    out = dict(X=ens["X"], Y=ens["Y"], w=ens["w"], rho=ens["rho"], T=ens["T"], R1=R1,
               wgrid=wgrid, smearing=smear, n_steps=n_steps)
    if S > 1:
        n_deg, deg_flat, sym_flat = _pack_syms(ens["symmetries"], ens["degenerate_space"])
        out.update(n_deg=n_deg, deg_space=deg_flat, sym=sym_flat, blocks_ids=ens["sym_block_id"],
                   S=S)
    for tag, wig, d4 in variants:
        lanc = make_reference_lanczos(ens, use_wigner=wig)
        lanc.ignore_v4 = not d4
        lanc.psi[:] = 0
        lanc.psi[:M] = R1
        lanc.perturbation_modulus = R1.dot(R1)
        with contextlib.redirect_stdout(io.StringIO()):
            lanc.run_FT(n_steps, verbose=False)
            g = lanc.get_green_function_continued_fraction(wgrid, smearing=smear)
            g_nt = lanc.get_green_function_continued_fraction(wgrid, use_terminator=False,
                                                              smearing=smear)
        out[tag + "/a"] = np.array(lanc.a_coeffs)
        out[tag + "/b"] = np.array(lanc.b_coeffs)
        out[tag + "/c"] = np.array(lanc.c_coeffs)
        out[tag + "/G"] = g
        out[tag + "/G_noterm"] = g_nt
        # one operator application on the start vector, both directions
        psi0 = np.zeros(M + M * (M + 1))
        psi0[:M] = R1
        rng = np.random.default_rng(seed + 7)
        psi_r = rng.standard_normal(len(psi0)) * 1e-2
        psi_r[:M] += R1
        with contextlib.redirect_stdout(io.StringIO()):
            out[tag + "/Lpsi"] = lanc.apply_full_L(psi_r.copy()).copy()
            out[tag + "/LTpsi"] = lanc.apply_full_L(psi_r.copy(), transpose=True).copy()
        out[tag + "/psi_r"] = psi_r
    np.savez_compressed(os.path.join(HERE, fname), **out)


def static_case(fname, M, N, seed, sh_steps):
    """The reference's static response (apply_L1_static, apply_anharmonic_static,
    run_hessian_calculation, StaticHessian.run) through static_adapter."""
    import importlib
    load_reference()
    SH = importlib.import_module("tdscha.StaticHessian")
    # frequencies of 0.36-1 Ry keep the static susceptibility O(1): the
    # reference asserts |G - G^T| < 1e-4 in absolute terms (:4319-4320), which
    # meV-scale modes (G ~ 1/w^2 ~ 1e5) cannot meet at its 1e-6 solver threshold
    ens = make_ensemble(M, N, seed=seed, n_syms=1, rho_sigma=0.1, w_min_cm=40000.0,
                        w_max_cm=110000.0)
    lanc = make_reference_lanczos(ens, use_wigner=True)
    Ps = M + M * (M + 1) // 2
    rng = np.random.default_rng(seed + 3)
    psi = rng.standard_normal(Ps)
    psi[:M] *= 10
    out = dict(X=ens["X"], Y=ens["Y"], w=ens["w"], rho=ens["rho"], T=ens["T"], psi_s=psi)
    with static_adapter(lanc), contextlib.redirect_stdout(io.StringIO()):
        out["L1"] = lanc.apply_L1_static(psi.copy())
        out["L1_inv_half"] = lanc.apply_L1_static(psi.copy(), inverse=True, power=0.5)
        lanc.psi = psi.copy()
        out["anh"] = lanc.apply_anharmonic_static().copy()
        lanc.ignore_v4 = True
        lanc.psi = psi.copy()
        out["anh_nod4"] = lanc.apply_anharmonic_static().copy()
        lanc.ignore_v4 = False
        out["hessian"] = lanc.run_hessian_calculation(verbose=False)
        out["hessian_noprec"] = lanc.run_hessian_calculation(verbose=False,
                                                             use_preconditioning=False)
        sh = SH.StaticHessian()
        sh.lanczos = lanc
        n_g = M * (M + 1) // 2
        n_w = M * (M * M + 3 * M + 2) // 6
        v0 = np.zeros(n_g + n_w)
        counter = 0
        for i in range(M):           # the preconditioned initial guess of StaticHessian.init
            v0[counter] = 1 / ens["w"][i]
            counter += M - i
        sh.vector = v0.copy()
        sh.run(sh_steps, threshold=1e-8, algorithm="cg-prec")
        out["sh_vector"] = sh.vector.copy()
        out["sh_hessian"] = sh.retrieve_hessian(noq=True)
        out["sh_steps"] = sh_steps
    np.savez_compressed(os.path.join(HERE, fname), **out)


def input_files_case(fname, M, N, S, seed):
    """Text of every file the reference's prepare_input_files writes."""
    import tempfile
    ens = make_ensemble(M, N, seed=seed, n_syms=S, rho_sigma=0.1)
    lanc = make_reference_lanczos(ens, use_wigner=False)
    lanc.psi[:M] = random_R1(M, seed + 1)
    lanc.perturbation_modulus = float(lanc.psi[:M].dot(lanc.psi[:M]))
    out = dict(X=ens["X"], Y=ens["Y"], w=ens["w"], rho=ens["rho"], T=ens["T"], psi=lanc.psi.copy())
    if S > 1:
        n_deg, deg_flat, sym_flat = _pack_syms(ens["symmetries"], ens["degenerate_space"])
        out.update(n_deg=n_deg, deg_space=deg_flat, sym=sym_flat, S=S)
    with tempfile.TemporaryDirectory() as d:
        lanc.prepare_input_files(root_name="case", n_steps=7, directory=d)
        for f in sorted(os.listdir(d)):
            with open(os.path.join(d, f)) as fp:
                out["file:" + f[len("case"):]] = np.array(fp.read())
    np.savez_compressed(os.path.join(HERE, fname), **out)


class _DynStub:
    """The three members of a cellconstructor Phonons object that the
    reference's IR / Raman perturbation builders read: effective charges,
    the supercell, and the Raman vector (here the plain contraction of a
    given Raman tensor with the two polarisations)."""

    def __init__(self, ec, raman, supercell):
        self.effective_charges = ec
        self.raman_tensor = raman
        self._sc = supercell

    def GetSupercell(self):
        return self._sc

    def GetRamanVector(self, p_in, p_out):
        return np.einsum("abc,a,b->c", self.raman_tensor, p_in, p_out)


def host_helpers_case(fname, seed):
    """Host-side Lanczos helpers: Wigner change of variables, the Lanczos
    matrix, the static frequency and the IR / Raman perturbation builders."""
    nat_uc, supercell = 2, (2, 1, 1)
    nat_sc = nat_uc * int(np.prod(supercell))
    M = 3 * nat_sc - 3
    ens = make_ensemble(M, 6, seed=seed, n_syms=1, rho_sigma=0.0)
    rng = np.random.default_rng(seed + 1)
    q, _ = np.linalg.qr(rng.standard_normal((3 * nat_sc, 3 * nat_sc)))
    pols = np.ascontiguousarray(q[:, :M])
    m = np.repeat(rng.uniform(1e3, 1e5, nat_sc), 3)
    ec = rng.standard_normal((nat_uc, 3, 3))
    raman = rng.standard_normal((3, 3, 3 * nat_uc))
    out = dict(w=ens["w"], T=ens["T"], X=ens["X"], Y=ens["Y"], rho=ens["rho"], pols=pols, m=m,
               ec=ec, raman=raman, supercell=np.array(supercell))
    lanc = make_reference_lanczos(ens, use_wigner=True)
    lanc.pols, lanc.m = pols, m
    lanc.dyn = _DynStub(ec, raman, supercell)
    psi = rng.standard_normal(M + M * (M + 1))
    out["psi"] = psi
    for tag, T in (("T", float(ens["T"])), ("T0", 0.0)):
        lanc.T = T
        lanc.psi = psi.copy()
        out["alpha1/" + tag] = lanc.get_alpha1_beta1_wigner(get_alpha=True)
        out["beta1/" + tag] = lanc.get_alpha1_beta1_wigner(get_alpha=False)
        out["a1/" + tag] = lanc.get_a1_b1_wigner(get_a1=True)
        out["b1/" + tag] = lanc.get_a1_b1_wigner(get_a1=False)
    lanc.T = float(ens["T"])

    def pert(key, fn, *a, **k):
        with contextlib.redirect_stdout(io.StringIO()):
            fn(*a, **k)
        out["psi/" + key] = lanc.psi[:M].copy()
        out["mod/" + key] = np.float64(lanc.perturbation_modulus)

    e = np.eye(3)
    pert("ir_x", lanc.prepare_ir, pol_vec=e[0])
    pert("ir_mix", lanc.prepare_ir, effective_charges=2 * ec, pol_vec=np.array([0.3, -0.5, 0.8]))
    pert("raman_xy", lanc.prepare_raman, pol_vec_in=e[0], pol_vec_out=e[1])
    pert("raman_mixed", lanc.prepare_raman, pol_vec_in=e[0], pol_vec_out=e[2], mixed=True,
         pol_in_2=e[1], pol_out_2=e[1])
    for k in range(7):
        pert("raman_unpol%d" % k, lanc.prepare_raman, unpolarized=k)
        pert("unpol%d" % k, lanc.prepare_unpolarized_raman, index=k)
        out["prefactor%d" % k] = np.float64(lanc.get_prefactors_unpolarized_raman(k))

    # the Lanczos matrix from given coefficients, both kinds, with and without reversal
    n = 6
    a, b, c = rng.standard_normal(n), rng.standard_normal(n - 1), rng.standard_normal(n - 1)
    out.update(coef_a=a, coef_b=b, coef_c=c)
    for tag, cc, rev, shift in (("bi", c, False, 0.0), ("sym", [], False, 0.0),
                                ("bi_rev", c, True, 0.7)):
        lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs = list(a), list(b), list(cc)
        lanc.reverse_L, lanc.shift_value = rev, shift
        out["matrix/" + tag] = lanc.build_lanczos_matrix_from_coeffs()
    lanc.reverse_L, lanc.shift_value = False, 0.0

    # static frequency from the coefficients of the 50-step reference runs
    run = np.load(os.path.join(HERE, "runft_m21_n1000.npz"))
    R1 = run["R1"]
    for tag, wig in (("bilanczos", False), ("wigner", True)):
        lanc.use_wigner = wig
        lanc.a_coeffs = list(run[tag + "/a"])
        lanc.b_coeffs = list(run[tag + "/b"])
        lanc.c_coeffs = list(run[tag + "/c"])
        lanc.perturbation_modulus = float(R1.dot(R1))
        for k, sm in enumerate((0.0, 1e-5)):
            with contextlib.redirect_stdout(io.StringIO()):
                out["wstatic/%s/%d" % (tag, k)] = np.asarray(lanc.get_static_frequency(sm))
    out["wstatic_smearing"] = np.array([0.0, 1e-5])
    out["wstatic_modulus"] = np.float64(R1.dot(R1))
    np.savez_compressed(os.path.join(HERE, fname), **out)


def fake_lanczos_run(lanc, A, B, C, calls):
    """A run_FT stand-in for the host logic of StaticHessian.run_no_mode_mixing:
    the coefficients of the prepared mode (psi[index] = 1) from the tables A, B, C
    (n_modes x steps); every call is recorded."""
    M = A.shape[0]

    def run_FT(n_iter, save_dir=None, verbose=True, prefix="LANCZOS", **kw):
        i = int(np.argmax(np.abs(np.asarray(lanc.psi[:M]))))
        calls.append((i, int(n_iter), prefix))
        lanc.a_coeffs = list(A[i, :n_iter])
        lanc.b_coeffs = list(B[i, :n_iter])
        lanc.c_coeffs = list(C[i, :n_iter])
    return run_FT


def no_mode_mixing_case(fname, M, seed, n_steps):
    """The reference's StaticHessian.run_no_mode_mixing with run_FT replaced by
    fake_lanczos_run (the host logic: modes, degeneracy skips, G(0) of the
    continued fraction without terminator, the Hessian from the diagonal G)."""
    import importlib
    load_reference()
    SH = importlib.import_module("tdscha.StaticHessian")
    ens = make_ensemble(M, 8, seed=seed, n_syms=1, rho_sigma=0.0)
    w = np.sort(ens["w"].copy())
    w[2] = w[1]                              # a degenerate pair: the second is skipped
    ens = dict(ens, w=w)
    lanc = make_reference_lanczos(ens, use_wigner=True)
    rng = np.random.default_rng(seed + 1)
    A = (w ** 2)[:, None] * rng.uniform(0.8, 1.2, (M, n_steps))
    B = (w ** 2)[:, None] * rng.uniform(0.05, 0.2, (M, n_steps))
    C = (w ** 2)[:, None] * rng.uniform(0.05, 0.2, (M, n_steps))
    calls = []
    # past the reference's attribute guard: an instance attribute shadows the method
    object.__setattr__(lanc, "run_FT", fake_lanczos_run(lanc, A, B, C, calls))
    sh = SH.StaticHessian()
    sh.lanczos = lanc
    sh.verbose = False
    with contextlib.redirect_stdout(io.StringIO()):
        try:
            sh.run_no_mode_mixing(n_steps)
        except AttributeError:
            pass    # the final retrieve_hessian() builds a cellconstructor Phonons object
    out = dict(w=w, X=ens["X"], Y=ens["Y"], rho=ens["rho"], T=ens["T"], A=A, B=B, C=C,
               n_steps=n_steps, vector=np.asarray(sh.vector),
               hessian=sh.retrieve_hessian(noq=True), calls=np.array([c[:2] for c in calls]))
    np.savez_compressed(os.path.join(HERE, fname), **out)


@contextlib.contextmanager
def _scipy_tol_adapter():
    """The reference's run_biconjugate_gradient passes tol= to scipy's bicg /
    bicgstab, a keyword recent scipy releases replaced by rtol; inside this
    context (fixture generation only) tol is forwarded as rtol."""
    import scipy.sparse.linalg as sla
    saved = {k: getattr(sla, k) for k in ("bicg", "bicgstab")}

    def wrap(fn):
        def call(*a, tol=None, **kw):
            if tol is not None:
                kw["rtol"] = tol
            return fn(*a, **kw)
        return call
    for k, fn in saved.items():
        setattr(sla, k, wrap(fn))
    try:
        yield
    finally:
        for k, fn in saved.items():
            setattr(sla, k, fn)


def l1_inverse_case(fname, M, N, seed):
    """apply_L1_inverse_FT (both directions, T > 0 and T = 0) and
    run_biconjugate_gradient (bicgstab with the L1-inverse preconditioner)."""
    import scipy.sparse.linalg
    P = M + M * (M + 1)
    rng = np.random.default_rng(seed + 1)
    psi_r = rng.standard_normal(P)
    # the harmonic inverse on thermally populated modes (50-500 cm^-1 at 300 K)
    # and at T = 0
    low = make_ensemble(M, N, seed=seed + 2, n_syms=1, rho_sigma=0.1)
    lanc = make_reference_lanczos(low, use_wigner=False)
    out = dict(w_low=low["w"], T_low=low["T"], psi_r=psi_r)
    for tag, T in (("T", float(low["T"])), ("T0", 0.0)):
        lanc.T = T
        out["inv/" + tag] = lanc.apply_L1_inverse_FT(psi_r.copy())
        out["invT/" + tag] = lanc.apply_L1_inverse_FT(psi_r.copy(), transpose=True)
    # 0.36-1 Ry frequencies for the solve, as in static_case: the reference's absolute
    # hermiticity assertion (|G - G^T| < 1e-4) needs G = O(1)
    ens = make_ensemble(M, N, seed=seed, n_syms=1, rho_sigma=0.1, w_min_cm=40000.0,
                        w_max_cm=110000.0)
    lanc = make_reference_lanczos(ens, use_wigner=False)
    out.update(X=ens["X"], Y=ens["Y"], w=ens["w"], rho=ens["rho"], T=ens["T"])
    lanc.M_linop = scipy.sparse.linalg.LinearOperator(
        shape=(P, P), matvec=lanc.apply_L1_inverse_FT,
        rmatvec=lambda v: lanc.apply_L1_inverse_FT(v, transpose=True), dtype=np.double)
    with _scipy_tol_adapter(), contextlib.redirect_stdout(io.StringIO()):
        out["G_inv/bicgstab"] = lanc.run_biconjugate_gradient(verbose=False, tol=1e-12,
                                                              maxiter=3000, algorithm="bicgstab")
        out["G_inv/cg-minimize"] = lanc.run_biconjugate_gradient(
            verbose=False, tol=1e-10, maxiter=3000, algorithm="cg-minimize")
    np.savez_compressed(os.path.join(HERE, fname), **out)


def curvature_case(fname, M, n_steps, seed):
    """GetFreeEnergyCurvatureFromContinuedFraction on given coefficient tables
    (diagonal and mixed-pair runs, some stopped early by a zero b_n)."""
    import tempfile
    DL = load_reference()
    rng = np.random.default_rng(seed)
    w2 = rng.uniform(1.0, 4.0, M)
    a = w2[:, None, None] * rng.uniform(0.8, 1.2, (M, M, n_steps))
    b = rng.uniform(0.1, 0.3, (M, M, n_steps - 1))
    b[0, 0, 5:] = 0.0           # a run that stopped after 6 steps
    b[1, 2, 3:] = 0.0
    nat_sc = 2
    pols, _ = np.linalg.qr(rng.standard_normal((3 * nat_sc, 3 * nat_sc)))
    pols = pols[:, :M]
    masses = np.repeat(rng.uniform(1e3, 1e5, nat_sc), 3)
    out = dict(a_ns=a, b_ns=b, pols=pols, masses=masses)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                out["fc_mixing"] = DL.GetFreeEnergyCurvatureFromContinuedFraction(
                    a, b, pols, masses, mode_mixing=True, use_terminator=True, last_average=3)
                out["fc_diag_noterm"] = DL.GetFreeEnergyCurvatureFromContinuedFraction(
                    a, b, pols, masses, mode_mixing=False, use_terminator=False, smearing=1e-3)
        finally:
            os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, fname), **out)


def full_L_case(fname, M, N, seed):
    """get_full_L_matrix: the dense dynamic L (normal representation, both
    directions) and the dense static operator (through static_adapter)."""
    ens = make_ensemble(M, N, seed=seed, n_syms=1, rho_sigma=0.1)
    out = dict(X=ens["X"], Y=ens["Y"], w=ens["w"], rho=ens["rho"], T=ens["T"])
    DL = load_reference()
    lanc = make_reference_lanczos(ens, use_wigner=False)
    with contextlib.redirect_stdout(io.StringIO()):
        out["L"] = DL.get_full_L_matrix(lanc)
        out["LT"] = DL.get_full_L_matrix(lanc, transpose=True)
    lanc = make_reference_lanczos(ens, use_wigner=True)
    rng = np.random.default_rng(seed + 1)
    v0 = rng.standard_normal(len(lanc.psi))
    lanc.psi = v0.copy()
    with contextlib.redirect_stdout(io.StringIO()):
        ev, evec = lanc.run_full_diag(3, discard_dyn=True, n_iter=20)
    out.update(diag_v0=v0, diag_eigvals=ev, diag_eigvects=evec)
    with static_adapter(lanc), contextlib.redirect_stdout(io.StringIO()):
        out["L_static"] = DL.get_full_L_matrix(lanc, static=True)
        out["L_static_harm"] = DL.get_full_L_matrix(lanc, static=True, compute_anharm=False)
    np.savez_compressed(os.path.join(HERE, fname), **out)


def lehmann_case(fname, M, n, seed):
    """get_green_function_Lenmann, get_spectral_function_from_Lenmann and
    get_static_odd_fc on a stored Krylov basis (the data a status saved by the
    reference's earlier symmetric Lanczos holds), tridiagonal and Arnoldi forms."""
    rng = np.random.default_rng(seed)
    ens = make_ensemble(M, 5, seed=seed, n_syms=1, rho_sigma=0.0)
    lanc = make_reference_lanczos(ens, use_wigner=True)
    P = M + M * (M + 1)
    nat = 2
    pols, _ = np.linalg.qr(rng.standard_normal((3 * nat, 3 * nat)))
    pols = pols[:, :M]
    m = np.repeat(rng.uniform(1e3, 1e5, nat), 3)
    kb, _ = np.linalg.qr(rng.standard_normal((P, n + 1)))
    a = rng.uniform(1e-6, 4e-6, n)
    b = rng.uniform(1e-7, 5e-7, n - 1)
    arn = [list(rng.uniform(-1e-7, 1e-7, i)) + [a[i]] for i in range(n)]
    lanc.pols, lanc.m, lanc.nat = pols, m, nat
    lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs = list(a), list(b), []
    lanc.krilov_basis = [kb[:, i].copy() for i in range(n + 1)]
    lanc.arnoldi_matrix = arn
    w = np.linspace(0, 3e-3, 40)
    v_a = rng.standard_normal(3 * nat)
    v_b = rng.standard_normal(3 * nat)
    out = dict(pols=pols, m=m, kb=kb, a=a, b=b, w=ens["w"], T=ens["T"], wgrid=w, v_a=v_a, v_b=v_b,
               arnoldi=np.array([np.pad(r, (0, n - len(r))) for r in arn]))
    with contextlib.redirect_stdout(io.StringIO()):
        out["gf"] = lanc.get_green_function_Lenmann(w, 1e-4, v_a, v_b)
        out["gf_arnoldi"] = lanc.get_green_function_Lenmann(w, 1e-4, v_a, v_b, use_arnoldi=True)
        out["spectral"] = lanc.get_spectral_function_from_Lenmann(w, 1e-4, use_arnoldi=False)
        out["spectral_arnoldi"] = lanc.get_spectral_function_from_Lenmann(w, 1e-4)
        out["fc"] = lanc.get_static_odd_fc()
        lanc.krilov_basis = lanc.krilov_basis[:n]        # a converged run: n vectors
        out["fc_n"] = lanc.get_static_odd_fc()
    np.savez_compressed(os.path.join(HERE, fname), **out)


def main():
    perturb_cases()
    run_case("runft_m21_n1000.npz", 21, 1000, 1, 0.0, 21, 50,
             [("bilanczos", False, True), ("wigner", True, True), ("wigner_nod4", True, False)])
    # 12 steps: this symmetric case nearly breaks down at step 14 (b_13 ~ 1e-8),
    # after which a rounding-order change alone (in the reference itself)
    # moves the coefficients by O(1).
    run_case("runft_m12_n120_s48.npz", 12, 120, 48, 0.1, 31, 12,
             [("bilanczos", False, True), ("wigner", True, True)])
    static_case("static_m12_n800.npz", 12, 800, 41, 25)
    input_files_case("input_files_m6_n5_s48.npz", 6, 5, 48, 51)
    host_helpers_case("host_helpers_m9.npz", 61)
    no_mode_mixing_case("no_mode_mixing_m5.npz", 5, 71, 12)
    l1_inverse_case("l1_inverse_m6.npz", 6, 40, 81)
    curvature_case("curvature_m4.npz", 4, 12, 91)
    full_L_case("full_L_m4.npz", 4, 30, 95)
    lehmann_case("lehmann_m3.npz", 3, 8, 97)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
