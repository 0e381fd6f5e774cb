"""Size-independent properties at the benchmark's size (M=573 modes, N=50 000
configurations, S=1), where the oracle would take minutes per call:

* the float64 averages are deterministic (two calls, identical bits) and
  linear in (R1, Y1) to rounding (1e-11 of the largest entry);
* the tensor-core averages agree with the float64 ones within the per-call
  tolerance of the mixed path (2e-5 of the largest entry) and are linear in
  (R1, Y1) within the same tolerance (their per-call operand scales make them
  only approximately linear);
* d2v is symmetric in both precisions;
* the one-shot host-buffer entry point (the GetPerturbAverageSym replacement)
  gives the context path's result."""
import numpy as np
import pytest

import oracle
from tdscha_gb300 import _native as nat
from tdscha_gb300 import sscha_HP_odd
from tdscha_gb300.synthetic import make_ensemble, random_R1, random_sym

pytestmark = pytest.mark.gpu

M, N = 573, 50000
TOL64 = 1e-11
TOL_MIXED = 2e-5


def rel(got, ref):
    return np.abs(np.asarray(got) - ref).max() / max(np.abs(ref).max(), 1e-300)


@pytest.fixture(scope="module")
def full():
    ens = make_ensemble(M, N, seed=2024, rho_sigma=0.1)
    syms, spaces, bid = oracle.identity_symmetries(M)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    yield ens, (syms, spaces, bid), ctx
    ctx.close()


def call(ctx, R1, Y1, prec, d4=1):
    f = np.zeros(M)
    d2v = np.zeros((M, M))
    nat.check(nat.load().tdscha_perturb_averages(ctx.handle, R1.ctypes.data, Y1.ctypes.data, d4,
                                                 prec, f.ctypes.data, d2v.ctypes.data, 0, None))
    return f, d2v


def test_fullsize_fp64_deterministic_symmetric_linear(gpu_lib, full):
    ens, _, ctx = full
    R1, Y1 = random_R1(M, 1), random_sym(M, 2, scale=1e-3)
    R2, Y2 = random_R1(M, 3), random_sym(M, 4, scale=1e-3)
    f1, d1 = call(ctx, R1, Y1, nat.PREC_FP64)
    f1b, d1b = call(ctx, R1, Y1, nat.PREC_FP64)
    np.testing.assert_array_equal(f1, f1b)
    np.testing.assert_array_equal(d1, d1b)
    assert np.abs(d1 - d1.T).max() <= 1e-14 * np.abs(d1).max()
    f2, d2 = call(ctx, R2, Y2, nat.PREC_FP64)
    a, b = 0.7, -1.3
    fl, dl = call(ctx, a * R1 + b * R2, a * Y1 + b * Y2, nat.PREC_FP64)
    assert rel(fl, a * f1 + b * f2) <= TOL64
    assert rel(dl, a * d1 + b * d2) <= TOL64


@pytest.mark.parametrize("d4", [1, 0])
def test_fullsize_mixed_matches_fp64(gpu_lib, full, d4):
    ens, _, ctx = full
    R1, Y1 = random_R1(M, 5), random_sym(M, 6, scale=1e-3)
    f64, d64 = call(ctx, R1, Y1, nat.PREC_FP64, d4)
    fm, dm = call(ctx, R1, Y1, nat.PREC_MIXED, d4)
    ef, ed = rel(fm, f64), rel(dm, d64)
    print("M=%d N=%d d4=%d: mixed vs float64 f %.2e d2v %.2e" % (M, N, d4, ef, ed))
    assert ef <= TOL_MIXED and ed <= TOL_MIXED
    assert np.abs(dm - dm.T).max() <= 1e-12 * np.abs(dm).max()


def test_fullsize_mixed_linear(gpu_lib, full):
    ens, _, ctx = full
    R1, Y1 = random_R1(M, 7), random_sym(M, 8, scale=1e-3)
    R2, Y2 = random_R1(M, 9), random_sym(M, 10, scale=1e-3)
    f1, d1 = call(ctx, R1, Y1, nat.PREC_MIXED)
    f2, d2 = call(ctx, R2, Y2, nat.PREC_MIXED)
    fl, dl = call(ctx, 0.5 * R1 + 2.0 * R2, 0.5 * Y1 + 2.0 * Y2, nat.PREC_MIXED)
    assert rel(fl, 0.5 * f1 + 2.0 * f2) <= TOL_MIXED
    assert rel(dl, 0.5 * d1 + 2.0 * d2) <= TOL_MIXED


def test_fullsize_one_shot_matches_context(gpu_lib, full):
    ens, (syms, spaces, bid), ctx = full
    R1, Y1 = random_R1(M, 11), random_sym(M, 12, scale=1e-3)
    f_ctx, d_ctx = call(ctx, R1, Y1, nat.PREC_FP64)
    f = np.zeros(M)
    d2v = np.zeros((M, M))
    sscha_HP_odd.GetPerturbAverageSym(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1, ens["T"], 1,
                                      1, syms, np.ones(M, dtype=np.intc), spaces, bid, f, d2v)
    assert rel(f, f_ctx) <= TOL64
    assert rel(d2v, d_ctx) <= TOL64
