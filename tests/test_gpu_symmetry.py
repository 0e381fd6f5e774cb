"""Symmetry images applied on the perturbation side (csrc/symmetry.cu).

When every symmetry matrix only mixes modes of equal frequency, the context
keeps the N configurations once and carries the perturbation to each image
(Y1 -> S_j^T Y1 S_j, R1 -> S_j^T R1) instead of storing the N*S image rows.
Checked here: the layout query, both precisions against the oracle (which
forms the image rows like the reference), the image-free path against the
stored-image path on the same inputs, tables that must keep the image rows,
and a mixed-precision Lanczos run at the 189-mode, 48-image shape against
float64.  (The reference's own S=48 runs in tests/golden pass through the
image-free path in tests/test_gpu_fp64.py.)

Tolerances as elsewhere: one float64 call 1e-11 of the largest entry, one
mixed call 2e-5, spectral function of a mixed run 1e-4 relative."""
import os

import numpy as np
import pytest

import oracle
from tdscha_gb300 import _native as nat
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.synthetic import RY_TO_CM, make_ensemble, random_R1, random_sym

pytestmark = pytest.mark.gpu

TOL64, TOL_CALL, TOL_SPECTRAL = 1e-11, 2e-5, 1e-4


def rel(got, ref):
    return np.abs(np.asarray(got) - ref).max() / max(np.abs(ref).max(), 1e-300)


def _context(ens, mixed, image_rows=False):
    old = os.environ.get("TDSCHA_SYMMETRY_IMAGES")
    if image_rows:
        os.environ["TDSCHA_SYMMETRY_IMAGES"] = "rows"
    try:
        return nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], ens["symmetries"],
                           ens["degenerate_space"], ens["sym_block_id"], with_mixed=mixed)
    finally:
        if image_rows:
            if old is None:
                del os.environ["TDSCHA_SYMMETRY_IMAGES"]
            else:
                os.environ["TDSCHA_SYMMETRY_IMAGES"] = old


def _call(ctx, R1, Y1, prec, d4=1):
    M = R1.size
    f, d2v = np.zeros(M), np.zeros((M, M))
    nat.check(nat.load().tdscha_perturb_averages(ctx.handle, R1.ctypes.data, Y1.ctypes.data, d4,
                                                 prec, f.ctypes.data, d2v.ctypes.data, 0, None))
    return f, d2v


def _oracle(ens, R1, Y1, d4=1):
    return oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1, ens["T"], d4,
                                   ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"],
                                   n_threads=16)


# N above 2048 rows: several W-build row chunks and force partials per image
@pytest.mark.parametrize("M,N,S", [(24, 400, 48), (48, 1500, 8), (189, 2000, 48), (189, 3500, 48),
                                   (48, 2100, 8)])
def test_image_free_averages_match_oracle(gpu_lib, M, N, S):
    ens = make_ensemble(M, N, seed=300 + M, n_syms=S, rho_sigma=0.1)
    R1, Y1 = random_R1(M, 4), random_sym(M, 5, scale=1e-3)
    ctx = _context(ens, mixed=True)
    assert ctx.layout() == (S, N)          # no image rows resident
    for d4 in (1, 0):
        f_ref, d_ref = _oracle(ens, R1, Y1, d4)
        f, d2v = _call(ctx, R1, Y1, nat.PREC_FP64, d4)
        assert rel(f, f_ref) <= TOL64 and rel(d2v, d_ref) <= TOL64, (rel(f, f_ref), rel(d2v, d_ref))
        fm, dm = _call(ctx, R1, Y1, nat.PREC_MIXED, d4)
        print("M=%d N=%d S=%d d4=%d: mixed f %.2e d2v %.2e" % (M, N, S, d4, rel(fm, f_ref),
                                                               rel(dm, d_ref)))
        assert rel(fm, f_ref) <= TOL_CALL and rel(dm, d_ref) <= TOL_CALL
        f2, d2 = _call(ctx, R1, Y1, nat.PREC_MIXED, d4)
        assert np.array_equal(fm, f2) and np.array_equal(dm, d2)     # deterministic
    ctx.close()


def test_image_free_equals_image_rows(gpu_lib):
    M, N, S = 48, 1200, 48
    ens = make_ensemble(M, N, seed=17, n_syms=S, rho_sigma=0.1)
    R1, Y1 = random_R1(M, 6), random_sym(M, 7, scale=1e-3)
    a = _context(ens, mixed=True)
    b = _context(ens, mixed=True, image_rows=True)
    assert a.layout() == (S, N) and b.layout() == (1, N * S)
    fa, da = _call(a, R1, Y1, nat.PREC_FP64)
    fb, db = _call(b, R1, Y1, nat.PREC_FP64)
    assert rel(fa, fb) <= 1e-12 and rel(da, db) <= 1e-12
    ma, mda = _call(a, R1, Y1, nat.PREC_MIXED)
    assert rel(ma, fb) <= TOL_CALL and rel(mda, db) <= TOL_CALL
    a.close()
    b.close()


def test_non_degenerate_tables_keep_image_rows(gpu_lib):
    """Symmetry tables that mix modes of different frequency cannot move to
    the perturbation side: the context stores the image rows and still
    matches the oracle."""
    M, N, S = 12, 300, 8
    ens = make_ensemble(M, N, seed=5, n_syms=S, rho_sigma=0.1)
    ens["w"] = ens["w"] * (1 + 1e-3 * np.arange(M))      # split the triplets
    R1, Y1 = random_R1(M, 2), random_sym(M, 3, scale=1e-3)
    ctx = _context(ens, mixed=False)
    assert ctx.layout() == (1, N * S)
    f_ref, d_ref = _oracle(ens, R1, Y1)
    f, d2v = _call(ctx, R1, Y1, nat.PREC_FP64)
    assert rel(f, f_ref) <= TOL64 and rel(d2v, d_ref) <= TOL64
    ctx.close()


def _run(ens, precision, steps, R1):
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"],
                               use_wigner=False, precision=precision)
    lanc.init(use_symmetries=True, symmetries=(ens["symmetries"], ens["degenerate_space"]))
    lanc.full_reorth = True
    lanc.prepare_perturbation(R1, masses_exp=0)
    lanc.run_FT(steps, verbose=False)
    w = np.linspace(0, 600, 2000) / RY_TO_CM
    return lanc, -lanc.get_green_function_continued_fraction(w, smearing=5 / RY_TO_CM).imag


def test_image_free_lanczos_spectral_error_189_modes_48_images(gpu_lib):
    """Bi-Lanczos at M=189, S=48 (N=2000), full re-biorthogonalisation: mixed
    against float64, and float64 with stored image rows against float64 with
    the images on the perturbation side, over the 50 steps in which two
    float64 runs of this symmetric operator reproduce each other.  (Its
    eigenvalues are exactly degenerate across the rows of each
    multi-dimensional irreducible representation; rounding noise in the
    partner rows later grows into extra copies of converged Ritz values at
    steps set by the noise, and two float64 runs that differ only in the
    summation order then part: 6e-5 at 100 steps, 8e-4 at 200, measured.)"""
    M, N, S, steps = 189, 2000, 48, 50
    ens = make_ensemble(M, N, seed=21, n_syms=S, rho_sigma=0.1)
    R1 = random_R1(M, 22)
    l64, A64 = _run(ens, "fp64", steps, R1)
    lmx, Amx = _run(ens, "mixed", steps, R1)
    os.environ["TDSCHA_SYMMETRY_IMAGES"] = "rows"
    try:
        lrows, Arows = _run(ens, "fp64", steps, R1)
    finally:
        del os.environ["TDSCHA_SYMMETRY_IMAGES"]
    err = np.abs(Amx - A64).max() / np.abs(A64).max()
    err64 = np.abs(Arows - A64).max() / np.abs(A64).max()
    print("spectral error mixed %.3e, float64 rows vs image-free %.3e over %d steps"
          % (err, err64, steps))
    assert len(l64.a_coeffs) == len(lmx.a_coeffs) == len(lrows.a_coeffs) == steps
    assert err <= TOL_SPECTRAL
    assert err64 <= 1e-10
