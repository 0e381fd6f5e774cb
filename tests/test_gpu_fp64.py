"""Float64 GPU path against the reference's own outputs (golden fixtures) and
against the oracle.  Tolerances: a perturbation-average call or one operator
application within 1e-11 of the largest entry; Lanczos coefficients and the
Green function within 1e-8 relative (the FP64 bar of the spec)."""
import ctypes

import numpy as np
import pytest

import oracle
from tdscha_gb300 import _native as nat
from tdscha_gb300 import sscha_HP_odd
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.synthetic import make_ensemble, random_R1, random_sym

pytestmark = pytest.mark.gpu

TOL_CALL = 1e-11
TOL_RUN = 1e-8


def close(got, ref, tol):
    got, ref = np.asarray(got), np.asarray(ref)
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(got - ref).max() / scale
    assert err <= tol, "max error %.3e relative to max |ref| (tol %.1e)" % (err, tol)


def _syms(d, name):
    S = int(d[name + "/S"])
    n_deg, deg, sym = d[name + "/n_deg"], d[name + "/deg_space"], d[name + "/sym"]
    spaces, blocks, o, os_ = [], [], 0, 0
    for nd in n_deg:
        spaces.append(deg[o:o + nd])
        blocks.append(sym[os_:os_ + S * nd * nd].reshape(S, nd, nd))
        o += nd
        os_ += S * nd * nd
    return blocks, spaces, d[name + "/blocks_ids"]


@pytest.mark.parametrize("name", ["m21_n200_s1", "m12_n30_s48", "m9_n7_s8", "m1_n5_s1"])
@pytest.mark.parametrize("d4", [0, 1])
def test_one_shot_matches_reference(gpu_lib, golden, name, d4):
    d = golden("perturb_averages.npz")
    blocks, spaces, bid = _syms(d, name)
    M = d[name + "/X"].shape[1]
    f = np.zeros(M)
    d2v = np.zeros((M, M))
    sscha_HP_odd.GetPerturbAverageSym(d[name + "/X"], d[name + "/Y"], d[name + "/w"],
                                      d[name + "/rho"], d[name + "/R1"], d[name + "/Y1"],
                                      float(d[name + "/T"]), d4, blocks[0].shape[0], blocks,
                                      np.array([len(s) for s in spaces], np.intc), spaces, bid,
                                      f, d2v)
    key = "%s_d4%d" % (name, d4)
    close(f, d[key + "/f"], TOL_CALL)
    close(d2v, d[key + "/d2v"], TOL_CALL)


@pytest.mark.parametrize("M,N,S", [(64, 3000, 1), (24, 400, 48), (131, 777, 1)])
def test_context_device_pointers_match_oracle(gpu_lib, M, N, S):
    import torch
    ens = make_ensemble(M, N, seed=M + N, n_syms=S, rho_sigma=0.1)
    if S == 1:
        syms, spaces, bid = oracle.identity_symmetries(M)
    else:
        syms, spaces, bid = ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]
    R1 = random_R1(M, 3)
    Y1 = random_sym(M, 4, scale=1e-3)
    f_ref, d_ref = oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                           ens["T"], 1, syms, spaces, bid, n_threads=8)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid)
    dev = torch.device("cuda")
    tR1, tY1 = torch.tensor(R1, device=dev), torch.tensor(Y1, device=dev)
    tf = torch.empty(M, dtype=torch.float64, device=dev)
    td = torch.empty((M, M), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    nat.check(gpu_lib.tdscha_perturb_averages(ctx.handle, tR1.data_ptr(), tY1.data_ptr(), 1,
                                              nat.PREC_FP64, tf.data_ptr(), td.data_ptr(), 1, st))
    torch.cuda.synchronize()
    close(tf.cpu().numpy(), f_ref, TOL_CALL)
    close(td.cpu().numpy(), d_ref, TOL_CALL)
    # deterministic: a second call gives the same bits
    tf2, td2 = torch.empty_like(tf), torch.empty_like(td)
    nat.check(gpu_lib.tdscha_perturb_averages(ctx.handle, tR1.data_ptr(), tY1.data_ptr(), 1,
                                              nat.PREC_FP64, tf2.data_ptr(), td2.data_ptr(), 1,
                                              st))
    torch.cuda.synchronize()
    assert torch.equal(tf, tf2) and torch.equal(td, td2)
    ctx.close()


def _ens(d):
    ens = dict(X=d["X"], Y=d["Y"], w=d["w"], rho=d["rho"], T=float(d["T"]))
    if "S" in d:
        blocks, spaces, bid = _syms({("x/" + k): v for k, v in d.items()}, "x")
        ens.update(symmetries=blocks, degenerate_space=spaces, sym_block_id=bid)
    return ens


def _lanczos(ens, wig, d4=True):
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"],
                               use_wigner=wig)
    if "symmetries" in ens:
        lanc.init(use_symmetries=True,
                  symmetries=(ens["symmetries"], ens["degenerate_space"]))
    else:
        lanc.init(use_symmetries=False)
    lanc.ignore_v4 = not d4
    lanc.verbose = False
    return lanc


RUNS = [("runft_m21_n1000.npz", "bilanczos", False, True),
        ("runft_m21_n1000.npz", "wigner", True, True),
        ("runft_m21_n1000.npz", "wigner_nod4", True, False),
        ("runft_m12_n120_s48.npz", "bilanczos", False, True),
        ("runft_m12_n120_s48.npz", "wigner", True, True)]


@pytest.mark.parametrize("fname,tag,wig,d4", RUNS)
def test_apply_full_L_matches_reference(gpu_lib, golden, fname, tag, wig, d4):
    d = golden(fname)
    lanc = _lanczos(_ens(d), wig, d4)
    close(lanc.apply_full_L(d[tag + "/psi_r"].copy()), d[tag + "/Lpsi"], TOL_CALL)
    close(lanc.apply_full_L(d[tag + "/psi_r"].copy(), transpose=True), d[tag + "/LTpsi"],
          TOL_CALL)


@pytest.mark.parametrize("fname,tag,wig,d4", RUNS)
def test_run_FT_matches_reference(gpu_lib, golden, fname, tag, wig, d4):
    d = golden(fname)
    lanc = _lanczos(_ens(d), wig, d4)
    lanc.prepare_perturbation(d["R1"], masses_exp=0)
    lanc.run_FT(int(d["n_steps"]), verbose=False)
    for k in "abc":
        got = np.array(getattr(lanc, k + "_coeffs"))
        ref = d[tag + "/" + k]
        assert got.shape == ref.shape
        rel = np.abs(got - ref) / np.abs(ref)
        assert rel.max() <= TOL_RUN, (k, rel.max())
    G = lanc.get_green_function_continued_fraction(d["wgrid"], smearing=float(d["smearing"]))
    close(G, d[tag + "/G"], TOL_RUN)
    close(G.imag, d[tag + "/G"].imag, TOL_RUN)
    Gn = lanc.get_green_function_continued_fraction(d["wgrid"], use_terminator=False,
                                                    smearing=float(d["smearing"]))
    close(Gn, d[tag + "/G_noterm"], TOL_RUN)


def test_restart_from_status_continues_the_run(gpu_lib, golden, tmp_path):
    d = golden("runft_m21_n1000.npz")
    ens = _ens(d)
    full = _lanczos(ens, True)
    full.prepare_perturbation(d["R1"], masses_exp=0)
    full.run_FT(30, verbose=False)
    part = _lanczos(ens, True)
    part.prepare_perturbation(d["R1"], masses_exp=0)
    part.run_FT(12, verbose=False, save_dir=str(tmp_path), save_each=6)
    resumed = Lanczos()
    resumed.load_status(str(tmp_path / "LANCZOS_STEP12"))
    resumed.prepare_symmetrization(no_sym=True)
    resumed.verbose = False
    resumed.run_FT(18, verbose=False)
    np.testing.assert_allclose(resumed.a_coeffs, full.a_coeffs, rtol=1e-12)
    np.testing.assert_allclose(resumed.c_coeffs, full.c_coeffs, rtol=1e-12)
    assert len(resumed.basis_Q) == len(full.basis_Q)


def test_basis_vectors_match_oracle(gpu_lib, golden):
    d = golden("runft_m21_n1000.npz")
    ens = _ens(d)
    lanc = _lanczos(ens, False)
    lanc.prepare_perturbation(d["R1"], masses_exp=0)
    lanc.run_FT(6, verbose=False)
    ol = oracle.OracleLanczos(ens, use_wigner=False)
    ol.prepare_perturbation_R(d["R1"])
    ol.run_FT(6)
    for q, qr in zip(lanc.basis_Q, ol.basis_Q):
        close(q, qr, 1e-10)
    for p, pr in zip(lanc.basis_P, ol.basis_P):
        close(p, pr, 1e-10)


def test_nan_start_vector_is_reported(gpu_lib):
    ens = make_ensemble(8, 50, seed=9)
    lanc = _lanczos(ens, True)
    lanc.psi[:] = 0
    lanc.psi[0] = np.inf
    with pytest.raises(nat.TdschaError) as e:
        lanc.run_FT(2, verbose=False)
    assert e.value.code == nat.ERR_NAN


def test_continued_fraction_gpu_matches_oracle(gpu_lib, golden):
    d = golden("runft_m21_n1000.npz")
    for tag, wig in (("bilanczos", False), ("wigner", True)):
        lanc = Lanczos()
        lanc.use_wigner = wig
        lanc.a_coeffs = list(d[tag + "/a"])
        lanc.b_coeffs = list(d[tag + "/b"])
        lanc.c_coeffs = list(d[tag + "/c"])
        for kw in (dict(smearing=float(d["smearing"])), dict(last_average=5, smooth_ramp=4),
                   dict(use_terminator=False, smearing=1e-5)):
            g = lanc.get_green_function_continued_fraction(d["wgrid"], **kw)
            ref = oracle.continued_fraction(lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs,
                                            d["wgrid"], wig, **kw)
            close(g, ref, 1e-12)


def test_ignore_v3_and_harmonic_switches(gpu_lib):
    ens = make_ensemble(10, 200, seed=4)
    ol = oracle.OracleLanczos(ens, use_wigner=False)
    rng = np.random.default_rng(0)
    psi = rng.standard_normal(10 + 110) * 1e-2
    for attr in ("ignore_v3", "ignore_harmonic"):
        lanc = _lanczos(ens, False)
        setattr(lanc, attr, True)
        setattr(ol, attr, True)
        close(lanc.apply_full_L(psi.copy()), ol.apply_full_L(psi.copy()), TOL_CALL)
        setattr(ol, attr, False)
    lanc = _lanczos(ens, False)
    lanc.reverse_L = True
    lanc.shift_value = 3e-6
    ol.reverse_L, ol.shift_value = True, 3e-6
    close(lanc.apply_full_L(psi.copy()), ol.apply_full_L(psi.copy()), TOL_CALL)


def test_full_reorth_keeps_biorthogonality(gpu_lib, golden):
    """With full re-biorthogonalisation the early coefficients equal the plain
    recurrence's (reference golden) and the stored bases stay biorthogonal."""
    d = golden("runft_m21_n1000.npz")
    ens = _ens(d)
    lanc = _lanczos(ens, False)
    lanc.full_reorth = True
    lanc.prepare_perturbation(d["R1"], masses_exp=0)
    lanc.run_FT(50, verbose=False)
    a = np.array(lanc.a_coeffs)
    ref = d["bilanczos/a"]
    rel = np.abs(a[:15] - ref[:15]) / np.abs(ref[:15])
    assert rel.max() <= TOL_RUN, rel.max()
    Q = np.array(lanc.basis_Q)
    Pm = np.array(lanc.basis_P)
    G = Pm @ Q.T
    dg = np.abs(np.diag(G))
    off = np.abs(G - np.diag(np.diag(G))) / np.sqrt(np.outer(dg, dg))
    assert off.max() < 1e-10, off.max()


@pytest.mark.parametrize("M", [21, 24])     # P = M (M + 2): 483 (odd) and 624 (even)
def test_reorth_row_stride_paths_agree(gpu_lib, M):
    """The re-biorthogonalisation reads element pairs when every basis row
    starts on 16 bytes (even row stride) and single elements otherwise; the
    row strides P, P + 1 and P padded to 32 doubles cover both forms for odd
    and even P.  The runs agree to rounding and the bases stay biorthogonal."""
    import torch
    ens = make_ensemble(M, 600, seed=31, n_syms=1, rho_sigma=0.1)
    ident = ([np.ones((1, 1, 1))] * M, [np.array([i], dtype=np.intc) for i in range(M)],
             np.arange(M, dtype=np.intc))
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], *ident)
    ctx.set_options(False, False, False, False, False, 0.0)
    P, n = ctx.P, 40
    cap = n + 2
    lib = nat.load()
    psi = np.zeros(P)
    psi[:M] = random_R1(M, 3)
    first = torch.from_numpy(psi / np.linalg.norm(psi)).cuda()
    runs = {}
    for ld in (P, P + 1, ctx.basis_ld()):
        ctx.set_basis_ld(ld)
        Qd = torch.zeros((cap, ld), dtype=torch.float64, device="cuda")
        Pd = torch.zeros((cap, ld), dtype=torch.float64, device="cuda")
        Qd[0, :P].copy_(first)
        Pd[0, :P].copy_(first)
        hist = np.zeros(4 * cap)
        hist[3] = 1.0
        done, conv = ctypes.c_int(0), ctypes.c_int(0)
        nat.check(lib.tdscha_lanczos_run(ctx.handle, Qd.data_ptr(), Pd.data_ptr(), cap, 0, n, 0,
                                         nat.PREC_FP64, 1, nat.dp(hist), ctypes.byref(done),
                                         ctypes.byref(conv), None))
        assert done.value == n and not conv.value
        Q = Qd[: n + 1, :P].cpu().numpy()
        Pm = Pd[: n + 1, :P].cpu().numpy()
        G = Pm @ Q.T
        dg = np.abs(np.diag(G))
        off = np.abs(G - np.diag(np.diag(G))) / np.sqrt(np.outer(dg, dg))
        assert off.max() < 1e-12, (ld, off.max())
        runs[ld] = hist[: 4 * n].reshape(n, 4)[:, :3]
    ref = runs[P]
    for ld, h in runs.items():
        np.testing.assert_allclose(h, ref, rtol=1e-9, atol=1e-14 * np.abs(ref).max())
    with pytest.raises(nat.TdschaError):
        ctx.set_basis_ld(P - 1)
    ctx.close()
