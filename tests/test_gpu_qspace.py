"""GPU q-space operator (csrc/qspace.cu) against the q-space oracle."""
import ctypes

import numpy as np
import pytest

import oracle.qspace as oq
from tdscha_gb300 import _native as nat
from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
from tdscha_gb300.synthetic import make_qspace_ensemble

pytestmark = pytest.mark.gpu

# float64 throughout; the operator sums O(N S) terms in a different order
TOL = 1e-11


def _translation_syms(e):
    """Lattice translations acting on Bloch vectors: diagonal phases
    exp(-2 pi i q.t) on every (q, band) entry."""
    q, cells, nb = e["q"], e["cells"], e["nb"]
    mats = []
    for t in cells:
        ph = np.exp(-2j * np.pi * (q @ t))
        mats.append(np.diag(np.repeat(ph, nb)))
    return mats


def _setup(dims, nb, N, pairing, iq_pert=0, syms=False, seed=5, T=250.0, mask_gamma=True):
    e = make_qspace_ensemble(dims, nb, N, seed=seed, T=T, dispersion=0.3, rho_sigma=0.2)
    lz = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"],
                                   q_points=e["q"], pairing=pairing)
    valid = np.ones((nb, e["n_q"]), dtype=bool)
    if mask_gamma:
        valid[0, 0] = False
    lz.valid_modes_q = valid
    symmetries = _translation_syms(e) if syms else None
    lz.prepare_symmetrization(symmetries=symmetries)
    lz.build_q_pair_map(iq_pert)
    o = oq.OracleQSpaceLanczos(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], lz.q_pair_map,
                               iq_pert, symmetries=symmetries, valid=valid)
    return e, lz, o


CASES = [((3, 1, 1), 3, 200, "sum", 0, False),
         ((4, 1, 1), 2, 300, "difference", 2, False),
         ((2, 2, 1), 3, 150, "sum", 3, True),
         ((3, 2, 1), 2, 120, "difference", 0, True)]


@pytest.mark.parametrize("dims,nb,N,pairing,iq,syms", CASES)
def test_perturb_averages_q(gpu_lib, dims, nb, N, pairing, iq, syms):
    e, lz, o = _setup(dims, nb, N, pairing, iq, syms)
    rng = np.random.default_rng(11)
    R1 = rng.standard_normal(nb) + 1j * rng.standard_normal(nb)
    blocks = [rng.standard_normal((nb, nb)) + 1j * rng.standard_normal((nb, nb))
              for _ in lz.unique_pairs]
    for d4 in (True, False):
        f, d2v = lz.get_perturb_averages_q(R1, blocks, d4)
        fo, do = oq.perturb_averages_qspace(e["X_q"], e["Y_q"], e["w_q"], e["rho"], R1, blocks,
                                            e["T"], d4, iq, o.pairs, o.symmetries, o.valid)
        scale = max(np.abs(fo).max(), 1e-300)
        assert np.abs(f - fo).max() / scale < TOL
        for a, b in zip(d2v, do):
            assert np.abs(a - b).max() / max(np.abs(b).max(), 1e-300) < TOL


@pytest.mark.parametrize("dims,nb,N,pairing,iq,syms", CASES)
def test_apply_full_L_q(gpu_lib, dims, nb, N, pairing, iq, syms):
    e, lz, o = _setup(dims, nb, N, pairing, iq, syms)
    rng = np.random.default_rng(12)
    psi = rng.standard_normal(o.P) + 1j * rng.standard_normal(o.P)
    # Hermitian blocks hold their upper triangle; their diagonal is real
    got = lz.apply_full_L(psi)
    ref = o.apply_full_L(psi)
    assert np.abs(got - ref).max() / np.abs(ref).max() < TOL
    # the host-assembled anharmonic part goes through tdscha_qperturb_averages
    lz.psi = psi.copy()
    o.psi = psi.copy()
    anh = lz.apply_anharmonic_FT()
    anh_o = o.apply_anharmonic_FT(psi)
    assert np.abs(anh - anh_o).max() / np.abs(anh_o).max() < TOL


@pytest.mark.parametrize("ignore", [(True, False, False), (False, True, False),
                                    (False, False, True), (False, True, True)])
def test_apply_full_L_q_switches(gpu_lib, ignore):
    e, lz, o = _setup((3, 1, 1), 2, 100, "sum")
    lz.ignore_harmonic, lz.ignore_v3, lz.ignore_v4 = ignore
    o.ignore_harmonic, o.ignore_v3, o.ignore_v4 = ignore
    rng = np.random.default_rng(13)
    psi = rng.standard_normal(o.P) + 1j * rng.standard_normal(o.P)
    got = lz.apply_full_L(psi)
    ref = o.apply_full_L(psi)
    assert np.abs(got - ref).max() <= TOL * max(np.abs(ref).max(), 1e-300)


def _well_conditioned(b, floor=1e-4):
    """Steps before the first near-breakdown (b_k / max|b| < floor): past it the
    Krylov space of these small blocks is exhausted and the coefficients carry
    amplified rounding, in the oracle and on the GPU alike."""
    b = np.abs(np.asarray(b))
    small = np.where(b / b.max() < floor)[0]
    return len(b) if len(small) == 0 else int(small[0]) + 1


LANCZOS_CASES = [((3, 1, 1), 3, 200, "sum", 0, False),
                 ((4, 1, 1), 3, 300, "difference", 2, False),
                 ((2, 2, 1), 3, 150, "sum", 3, True)]


@pytest.mark.parametrize("reorth", [True, False])
@pytest.mark.parametrize("dims,nb,N,pairing,iq,syms", LANCZOS_CASES)
def test_qspace_lanczos_matches_oracle(gpu_lib, dims, nb, N, pairing, iq, syms, reorth):
    e, lz, o = _setup(dims, nb, N, pairing, iq, syms)
    lz.prepare_mode_q(iq, 1)
    o.psi[1] = 1.0
    n = 20
    lz.run_FT(n, verbose=False, reorthogonalize=reorth)
    o.run_FT(n, reorthogonalize=reorth)
    assert len(lz.a_coeffs) == len(o.a_coeffs)
    k = _well_conditioned(o.b_coeffs)
    assert k >= 10
    np.testing.assert_allclose(lz.a_coeffs[:k], o.a_coeffs[:k], rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(lz.b_coeffs[:k], o.b_coeffs[:k], rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(lz.c_coeffs[:k], o.c_coeffs[:k], rtol=1e-8, atol=1e-14)
    if reorth:
        Q = np.array(lz.basis_Q)
        mask = lz.mask_dot_wigner()
        G = np.real(np.conj(Q) @ (Q * mask).T)
        assert np.abs(G - np.eye(len(Q))).max() < 1e-10
        np.testing.assert_array_equal(np.array(lz.basis_P), Q)


def test_qspace_lanczos_restart_and_green_function(gpu_lib, tmp_path):
    e, lz, o = _setup((4, 1, 1), 3, 150, "sum")
    lz.prepare_mode_q(0, 1)
    o.psi[1] = 1.0
    lz.run_FT(6, verbose=False)
    lz.save_status(str(tmp_path / "st"))
    lz2 = QSpaceLanczos()
    lz2.load_status(str(tmp_path / "st"))
    lz2.run_FT(6, verbose=False)
    o.run_FT(12)
    k = _well_conditioned(o.b_coeffs)
    assert k >= 8
    np.testing.assert_allclose(lz2.a_coeffs[:k], o.a_coeffs[:k], rtol=1e-8)
    w = np.linspace(0, 3e-3, 50)
    g = lz2.get_green_function_continued_fraction(w, use_terminator=False, smearing=1e-5)
    assert np.all(np.isfinite(g))


def test_qspace_errors(gpu_lib):
    lib = gpu_lib
    h = ctypes.c_void_p()
    X = np.zeros((1, 4, 40), dtype=np.complex128)
    rc = lib.tdscha_qctx_create(ctypes.byref(h), 1, 40, 4, nat.dp(X.view(np.float64)),
                                nat.dp(X.view(np.float64)), nat.dp(np.ones(40)), None,
                                nat.dp(np.ones(4)), 300.0, 0, None, None, None)
    assert rc == nat.ERR_ARG   # more than 32 bands
    # non-finite ensemble entries are found on the device after the upload
    Xn = np.zeros((2, 10, 3), dtype=np.complex128)
    Xn[1, 4, 2] = complex(0.0, np.nan)
    Yn = np.zeros_like(Xn)
    rc = lib.tdscha_qctx_create(ctypes.byref(h), 2, 3, 10, nat.dp(Xn.view(np.float64)),
                                nat.dp(Yn.view(np.float64)), nat.dp(np.ones(6)), None,
                                nat.dp(np.ones(10)), 300.0, 0, None, None, None)
    assert rc == nat.ERR_NAN and b"non-finite" in lib.tdscha_last_error()
    e, lz, o = _setup((3, 1, 1), 2, 50, "sum")
    ctx = lz._qcontext()
    with pytest.raises(nat.TdschaError):
        ctx.set_pert(0, np.array([1, 2, 0]))   # not an involution


# mixed precision: fp32 averages on the CUDA cores (24-bit operands), float64
# partial sums; the same per-call bar as the tensor-core real-space path
TOL_MIXED = 2e-5


@pytest.mark.parametrize("dims,nb,N,pairing,iq,syms", CASES + [((4, 4, 4), 6, 400, "sum", 5,
                                                                 False)])
def test_perturb_averages_q_mixed(gpu_lib, dims, nb, N, pairing, iq, syms):
    e, lz, o = _setup(dims, nb, N, pairing, iq, syms)
    lz.precision = "mixed"
    rng = np.random.default_rng(13)
    R1 = rng.standard_normal(nb) + 1j * rng.standard_normal(nb)
    blocks = [rng.standard_normal((nb, nb)) + 1j * rng.standard_normal((nb, nb))
              for _ in lz.unique_pairs]
    scale_d = None
    for d4 in (True, False):
        f, d2v = lz.get_perturb_averages_q(R1, blocks, d4)
        fo, do = oq.perturb_averages_qspace(e["X_q"], e["Y_q"], e["w_q"], e["rho"], R1, blocks,
                                            e["T"], d4, iq, o.pairs, o.symmetries, o.valid)
        scale_d = max(np.abs(b).max() for b in do)
        assert np.abs(f - fo).max() / max(np.abs(fo).max(), 1e-300) < TOL_MIXED
        assert max(np.abs(a - b).max() for a, b in zip(d2v, do)) / scale_d < TOL_MIXED
        f2, d22 = lz.get_perturb_averages_q(R1, blocks, d4)      # deterministic
        assert np.array_equal(f, f2) and all(np.array_equal(a, b) for a, b in zip(d2v, d22))


def test_qlanczos_mixed_spectral_error(gpu_lib):
    """Hermitian q-space Lanczos with Gram-Schmidt, 60 steps on a 4x4x4 grid:
    the fp32 averages against float64 within the spectral bar of the mixed
    path (1e-4 relative)."""
    from tdscha_gb300.synthetic import RY_TO_CM
    e = make_qspace_ensemble((4, 4, 4), 6, 2000, seed=9, T=250.0, dispersion=0.3, rho_sigma=0.2)
    w = np.linspace(0, 1200, 2000) / RY_TO_CM
    spec = {}
    for prec in ("fp64", "mixed"):
        lz = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"],
                                       q_points=e["q"], precision=prec)
        lz.init(use_symmetries=False)
        lz.prepare_mode_q(3, 2)
        lz.run_FT(60, verbose=False)
        spec[prec] = -lz.get_green_function_continued_fraction(w, smearing=5 / RY_TO_CM).imag
        lz._invalidate()
    err = np.abs(spec["mixed"] - spec["fp64"]).max() / np.abs(spec["fp64"]).max()
    print("q-space mixed spectral error %.2e" % err)
    assert err <= 1e-4
