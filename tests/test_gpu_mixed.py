"""Tensor-core (two-limb fp16 operands, fp32 accumulate) perturbation averages
and the mixed-precision Lanczos run, against the float64 oracle / float64 GPU
path.

Tolerances: one perturbation-average call within 2e-5 of the largest entry
(the operands carry about 22 significant bits); the spectral function of a
mixed-precision run within 1e-4 relative (max |dA| / max |A| over the
frequency grid) of the float64 run -- the accuracy bar of the mixed path --
with full re-biorthogonalisation in both runs, or over a short window
without it (the plain recurrence amplifies any rounding difference by about
20x per step once biorthogonality is lost, between two float64 runs too)."""
import os

import numpy as np
import pytest

import oracle
from tdscha_gb300 import _native as nat
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.synthetic import RY_TO_CM, make_ensemble, random_R1, random_sym

pytestmark = pytest.mark.gpu

TOL_CALL = 2e-5
TOL_SPECTRAL = 1e-4


def rel(got, ref):
    return np.abs(np.asarray(got) - ref).max() / max(np.abs(ref).max(), 1e-300)


def _mixed_call(ctx, R1, Y1, d4=1):
    M = R1.size
    f = np.zeros(M)
    d2v = np.zeros((M, M))
    nat.check(nat.load().tdscha_perturb_averages(ctx.handle, R1.ctypes.data, Y1.ctypes.data, d4,
                                                 nat.PREC_MIXED, f.ctypes.data, d2v.ctypes.data,
                                                 0, None))
    return f, d2v


@pytest.mark.parametrize("M,N,S", [(64, 3000, 1), (21, 1000, 1), (131, 2000, 1), (24, 300, 48),
                                   (573, 1500, 1)])
def test_mixed_perturb_matches_oracle(gpu_lib, M, N, S):
    ens = make_ensemble(M, N, seed=100 + M, n_syms=S, rho_sigma=0.1)
    if S == 1:
        syms, spaces, bid = oracle.identity_symmetries(M)
    else:
        syms, spaces, bid = ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]
    R1 = random_R1(M, 8)
    Y1 = random_sym(M, 9, scale=1e-3)
    f_ref, d_ref = oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                           ens["T"], 1, syms, spaces, bid, n_threads=8)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    f, d2v = _mixed_call(ctx, R1, Y1)
    ef, ed = rel(f, f_ref), rel(d2v, d_ref)
    print("M=%d N=%d S=%d: f err %.2e  d2v err %.2e" % (M, N, S, ef, ed))
    assert ef <= TOL_CALL and ed <= TOL_CALL
    f2, d2 = _mixed_call(ctx, R1, Y1)
    assert np.array_equal(f, f2) and np.array_equal(d2v, d2)      # deterministic
    ctx.close()


def _spectral_run(ens, precision, steps, R1, reorth=False):
    lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"],
                               use_wigner=False, precision=precision)
    lanc.init(use_symmetries=False)
    lanc.full_reorth = reorth
    lanc.prepare_perturbation(R1, masses_exp=0)
    lanc.run_FT(steps, verbose=False)
    w = np.linspace(0, 600, 2000) / RY_TO_CM
    G = lanc.get_green_function_continued_fraction(w, smearing=5 / RY_TO_CM)
    return lanc, -G.imag


@pytest.mark.parametrize("M,N,steps,reorth", [(48, 4000, 30, False), (96, 8000, 80, True),
                                              (189, 10000, 150, True)])
def test_mixed_lanczos_spectral_error(gpu_lib, M, N, steps, reorth):
    ens = make_ensemble(M, N, seed=7 + M, rho_sigma=0.1)
    R1 = random_R1(M, 3)
    l64, A64 = _spectral_run(ens, "fp64", steps, R1, reorth)
    lmx, Amx = _spectral_run(ens, "mixed", steps, R1, reorth)
    err = rel(Amx, A64)
    a64, amx = np.array(l64.a_coeffs), np.array(lmx.a_coeffs)
    print("M=%d N=%d: spectral err %.2e, a_0..9 max rel %.2e" % (
        M, N, err, np.max(np.abs(amx[:10] - a64[:10]) / np.abs(a64[:10]))))
    assert err <= TOL_SPECTRAL


def test_bounded_wait_reports_timeout_and_context_survives(gpu_lib, monkeypatch):
    M, N = 64, 512
    ens = make_ensemble(M, N, seed=5)
    syms, spaces, bid = oracle.identity_symmetries(M)
    R1, Y1 = random_R1(M, 1), random_sym(M, 2, scale=1e-3)
    monkeypatch.setenv("TDSCHA_WAIT_BUDGET_CYCLES", "0")
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    monkeypatch.delenv("TDSCHA_WAIT_BUDGET_CYCLES")
    with pytest.raises(nat.TdschaError) as e:
        _mixed_call(ctx, R1, Y1)
    assert e.value.code == nat.ERR_TIMEOUT
    ctx.close()
    # the CUDA context is still usable: a fresh context computes correctly
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    f, d2v = _mixed_call(ctx, R1, Y1)
    f_ref, d_ref = oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                           ens["T"], 1, syms, spaces, bid)
    assert rel(d2v, d_ref) <= TOL_CALL
    ctx.close()


def test_mixed_repeat_bitwise_identical(gpu_lib):
    """Thousands of back-to-back calls on the same inputs give the same bits.
    The stage A epilogue refills its d / g part buffers by TMA right after the
    warps' shared-memory reads; without a proxy fence before the refill about
    one call in 1500 read part of a refilled buffer (wrong q / s row dots in a
    few rows of one tile, errors near 4e-4). 4000 calls catch that rate with
    probability about 0.94."""
    M, N = 573, 20000
    ens = make_ensemble(M, N, seed=2024, rho_sigma=0.1)
    syms, spaces, bid = oracle.identity_symmetries(M)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    R1, Y1 = random_R1(M, 5), random_sym(M, 6, scale=1e-3)
    f0, d0 = _mixed_call(ctx, R1, Y1)
    bad = []
    for i in range(4000):
        f, d2v = _mixed_call(ctx, R1, Y1)
        if not (np.array_equal(f, f0) and np.array_equal(d2v, d0)):
            bad.append((i, rel(f, f0), rel(d2v, d0)))
    ctx.close()
    assert not bad, "calls with different results (index, rel f, rel d2v): %s" % bad[:5]


def test_release_cached_memory(gpu_lib):
    """Blocks of destroyed contexts stay cached for the next context of the same
    shape until tdscha_release_cached_memory hands them back."""
    import ctypes
    import torch
    M, N = 96, 4000
    ens = make_ensemble(M, N, seed=21)
    syms, spaces, bid = oracle.identity_symmetries(M)
    R1, Y1 = random_R1(M, 1), random_sym(M, 2, scale=1e-3)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    f0, d0 = _mixed_call(ctx, R1, Y1)
    ctx.close()
    # a second context of the same shape reuses the cached blocks and computes the same bits
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=True)
    f1, d1 = _mixed_call(ctx, R1, Y1)
    ctx.close()
    np.testing.assert_array_equal(f0, f1)
    np.testing.assert_array_equal(d0, d1)
    free_before = torch.cuda.mem_get_info()[0]
    got = ctypes.c_ulonglong(0)
    nat.check(gpu_lib.tdscha_release_cached_memory(ctypes.byref(got)))
    # at least the ensemble images D and F (2 x N x M doubles) were cached
    assert got.value >= 2 * N * M * 8
    assert torch.cuda.mem_get_info()[0] >= free_before + got.value // 2
    nat.check(gpu_lib.tdscha_release_cached_memory(ctypes.byref(got)))
    assert got.value == 0


def test_autotuner_choice_is_cached_and_accurate(gpu_lib):
    """The shape autotuner picks a stage A kernel and a split count, caches
    the choice for the shape (a second context of the same shape gives the
    same bits), and the tuned application stays within the per-call
    tolerance of the oracle."""
    M, N = 189, 6000
    ens = make_ensemble(M, N, seed=77, rho_sigma=0.1)
    syms, spaces, bid = oracle.identity_symmetries(M)
    R1, Y1 = random_R1(M, 78), random_sym(M, 79, scale=1e-3)
    a = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                    with_mixed=True)
    one_acc, splits, ms = a.tuning()
    assert one_acc in (0, 1) and splits >= 1 and ms > 0
    b = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                    with_mixed=True)
    assert b.tuning() == (one_acc, splits, ms)
    fa, da = _mixed_call(a, R1, Y1)
    fb, db = _mixed_call(b, R1, Y1)
    assert np.array_equal(fa, fb) and np.array_equal(da, db)
    f_ref, d_ref = oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1,
                                           ens["T"], 1, syms, spaces, bid, n_threads=8)
    assert rel(fa, f_ref) <= TOL_CALL and rel(da, d_ref) <= TOL_CALL
    a.close()
    b.close()


@pytest.mark.parametrize("M,N,S", [(96, 3000, 1), (97, 2000, 1), (24, 400, 48)])
def test_pair_application_bitwise(gpu_lib, monkeypatch, M, N, S):
    """A mixed bi-Lanczos step runs L q and L^T p as one two-perturbation call
    (each perturbation with its own W scales, images s*J .. s*J + J - 1 of the
    per-call buffers); it must give the bits of two one-perturbation calls
    (TDSCHA_PAIR_APPLY=0), with and without symmetry images."""
    ens = make_ensemble(M, N, seed=40 + M, n_syms=S, rho_sigma=0.1)
    R1 = random_R1(M, 9)
    runs = []
    for pair in ("1", "0"):
        monkeypatch.setenv("TDSCHA_PAIR_APPLY", pair)
        lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"],
                                   use_wigner=False, precision="mixed")
        if S > 1:
            lanc.init(use_symmetries=True, symmetries=(ens["symmetries"], ens["degenerate_space"]))
        else:
            lanc.init(use_symmetries=False)
        lanc.full_reorth = True
        lanc.prepare_perturbation(R1, masses_exp=0)
        lanc.run_FT(30, verbose=False)
        runs.append((np.array(lanc.a_coeffs), np.array(lanc.b_coeffs), np.array(lanc.c_coeffs),
                     np.array(lanc.basis_Q)))
        lanc._invalidate()
    for x, y in zip(*runs):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("M,N,S", [(96, 30000, 1), (24, 400, 48)])
def test_fp32_storage_context(gpu_lib, M, N, S):
    """with_mixed='fp32' keeps only the 4-byte operands: the float64 image rows
    (2 x rows x M doubles) go back to the device once the operands are built.
    Mixed calls and runs give the bits of a context that keeps both storages,
    and a float64 call is refused with TDSCHA_ERR_STATE."""
    import torch
    ens = make_ensemble(M, N, seed=60 + M, n_syms=S, rho_sigma=0.1)
    if S == 1:
        syms, spaces, bid = oracle.identity_symmetries(M)
    else:
        syms, spaces, bid = ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]
    R1, Y1 = random_R1(M, 3), random_sym(M, 4, scale=1e-3)
    lib = nat.load()
    outs, free = [], []
    for mode in (True, "fp32"):
        nat.check(lib.tdscha_release_cached_memory(None))
        torch.cuda.synchronize()
        ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                          with_mixed=mode)
        outs.append(_mixed_call(ctx, R1, Y1))
        rows = ctx.layout()[1]      # resident ensemble rows (N when images act on Y1)
        f = np.zeros(M)
        d2v = np.zeros((M, M))
        rc = lib.tdscha_perturb_averages(ctx.handle, R1.ctypes.data, Y1.ctypes.data, 1,
                                         nat.PREC_FP64, f.ctypes.data, d2v.ctypes.data, 0, None)
        assert (rc == nat.OK) == (mode is True)
        if mode == "fp32":
            assert rc == nat.ERR_STATE and not ctx.fp64_storage
        # after both calls: every kernel module the two contexts use is loaded
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        ctx.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    released = 2 * rows * M * 8     # float64 D and F rows
    if released >= 1 << 24:         # well above the device's allocation granularity
        assert free[1] - free[0] >= released // 2
    nat.check(lib.tdscha_release_cached_memory(None))
    # the Lanczos class: fp32_storage with precision 'mixed', same coefficients
    runs = []
    for only32 in (False, True):
        lanc = Lanczos.from_arrays(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"],
                                   use_wigner=False, precision="mixed")
        lanc.fp32_storage = only32
        if S > 1:
            lanc.init(use_symmetries=True, symmetries=(ens["symmetries"], ens["degenerate_space"]))
        else:
            lanc.init(use_symmetries=False)
        lanc.prepare_perturbation(random_R1(M, 9), masses_exp=0)
        lanc.run_FT(8, verbose=False)
        runs.append((np.array(lanc.a_coeffs), np.array(lanc.b_coeffs), np.array(lanc.c_coeffs)))
        assert lanc._ctx.fp64_storage == (not only32)
        lanc._invalidate()
    for x, y in zip(*runs):
        assert np.array_equal(x, y)
