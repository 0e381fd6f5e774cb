"""The allocation-free float64 entry point (tdscha_perturb_averages_noalloc).

It exists for callers that cannot let the library allocate device memory
(programs that own the whole GPU memory budget, or loops that cannot afford
cudaMalloc's synchronisation).  Checked through the C ABI against the
context entry point (tdscha_perturb_averages, float64) on two calls in a
row, which share the static scratch area; against the oracle at a small size
and at T = 0 with fewer configurations than one split; at M = 573 just under
the static area's limit; and for its on-device input check.  Collected last
on purpose."""
import numpy as np
import pytest

import oracle
from tdscha_gb300 import _native as nat
from tdscha_gb300.synthetic import make_ensemble, random_R1, random_sym

pytestmark = pytest.mark.gpu

TOL = 1e-11     # the float64 tolerance of the other GPU tests


def _close(got, ref):
    err = np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)
    assert err <= TOL, err


def test_noalloc_matches_context_entry_point_twice(gpu_lib):
    import torch
    dev = torch.device("cuda")
    st = torch.cuda.current_stream().cuda_stream
    M, N = 57, 3000
    ens = make_ensemble(M, N, seed=42, rho_sigma=0.1)
    syms, spaces, bid = oracle.identity_symmetries(M)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid)
    X = torch.tensor(ens["X"], device=dev)
    Y = torch.tensor(ens["Y"], device=dev)
    w = torch.tensor(ens["w"], device=dev)
    rho = torch.tensor(ens["rho"], device=dev)
    for call, (d4, seed) in enumerate([(1, 3), (0, 4)]):
        R1 = torch.tensor(random_R1(M, seed), device=dev)
        Y1 = torch.tensor(random_sym(M, seed + 10, scale=1e-3), device=dev)
        f = torch.full((M,), np.nan, dtype=torch.float64, device=dev)
        d2v = torch.full((M, M), np.nan, dtype=torch.float64, device=dev)
        nat.check(gpu_lib.tdscha_perturb_averages_noalloc(
            M, N, X.data_ptr(), Y.data_ptr(), w.data_ptr(), rho.data_ptr(), R1.data_ptr(),
            Y1.data_ptr(), float(ens["T"]), d4, f.data_ptr(), d2v.data_ptr(), st))
        fr = torch.empty_like(f)
        dr = torch.empty_like(d2v)
        nat.check(gpu_lib.tdscha_perturb_averages(ctx.handle, R1.data_ptr(), Y1.data_ptr(), d4,
                                                  nat.PREC_FP64, fr.data_ptr(), dr.data_ptr(),
                                                  1, st))
        torch.cuda.synchronize()
        _close(f.cpu().numpy(), fr.cpu().numpy())
        _close(d2v.cpu().numpy(), dr.cpu().numpy())
    ctx.close()


def test_noalloc_rejects_sizes_beyond_the_static_area(gpu_lib):
    one = np.zeros(1)
    rc = gpu_lib.tdscha_perturb_averages_noalloc(573, 1000000, one.ctypes.data, one.ctypes.data,
                                                 one.ctypes.data, one.ctypes.data,
                                                 one.ctypes.data, one.ctypes.data, 300.0, 1,
                                                 one.ctypes.data, one.ctypes.data, None)
    assert rc == nat.ERR_ARG
    assert b"static" in gpu_lib.tdscha_last_error()


def _noalloc(gpu_lib, ens, R1, Y1, d4, T=None):
    """One call on device copies of the inputs; returns (f, d2v) on the host."""
    import torch
    dev = torch.device("cuda")
    M, N = ens["X"].shape[1], ens["X"].shape[0]
    t = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    X, Y, w, rho, r1, y1 = (t(ens["X"]), t(ens["Y"]), t(ens["w"]), t(ens["rho"]), t(R1), t(Y1))
    f = torch.zeros(M, dtype=torch.float64, device=dev)
    d2v = torch.zeros((M, M), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    nat.check(gpu_lib.tdscha_perturb_averages_noalloc(
        M, N, X.data_ptr(), Y.data_ptr(), w.data_ptr(), rho.data_ptr(), r1.data_ptr(),
        y1.data_ptr(), float(ens["T"] if T is None else T), d4, f.data_ptr(), d2v.data_ptr(), st))
    torch.cuda.synchronize()
    return f.cpu().numpy(), d2v.cpu().numpy()


@pytest.mark.parametrize("M,N,T", [(21, 700, 300.0), (10, 40, 0.0)])
def test_noalloc_matches_oracle(gpu_lib, M, N, T):
    ens = make_ensemble(M, N, seed=5, rho_sigma=0.1)
    ens["T"] = T
    syms, spaces, bid = oracle.identity_symmetries(M)
    R1, Y1 = random_R1(M, 6), random_sym(M, 7, scale=1e-3)
    for d4 in (1, 0):
        f, d2v = _noalloc(gpu_lib, ens, R1, Y1, d4)
        fr, dr = oracle.perturb_averages(ens["X"], ens["Y"], ens["w"], ens["rho"], R1, Y1, T, d4,
                                         syms, spaces, bid)
        _close(f, fr)
        _close(d2v, dr)


def _words_needed(M, N):
    """The scratch size rule of noalloc.cu, in float64 words."""
    cd = lambda a, b: -(-a // b)
    nct = cd(M, 64)
    nsplit = min(max(1, cd(304, nct * nct)), max(1, N // 64))
    nfchunk = min(max(1, N // 256), 512)
    nset = max(1, min(2048, max(cd(M * M, 256), cd(M * N, 2048))))
    return 2 * M + M * M + 2 * nct * N + 4 * N + nsplit * M * M + nfchunk * M + 1 + nset


def test_noalloc_near_the_static_limit(gpu_lib):
    """M = 573 with N just under the largest size the 32 MiB area takes,
    against the float64 context path."""
    M, limit = 573, 4 << 20
    N = 1000
    while _words_needed(M, N + 1000) <= limit:
        N += 1000
    assert _words_needed(M, N) <= limit < _words_needed(M, N + 1000)
    ens = make_ensemble(M, N, seed=9, rho_sigma=0.1)
    syms, spaces, bid = oracle.identity_symmetries(M)
    R1, Y1 = random_R1(M, 1), random_sym(M, 2, scale=1e-3)
    f, d2v = _noalloc(gpu_lib, ens, R1, Y1, 1)
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid)
    fr, dr = np.zeros(M), np.zeros((M, M))
    nat.check(gpu_lib.tdscha_perturb_averages(ctx.handle, R1.ctypes.data, Y1.ctypes.data, 1,
                                              nat.PREC_FP64, fr.ctypes.data, dr.ctypes.data, 0,
                                              None))
    ctx.close()
    _close(f, fr)
    _close(d2v, dr)


def test_noalloc_invalid_input_gives_nan(gpu_lib):
    M, N = 12, 300
    ens = make_ensemble(M, N, seed=2, rho_sigma=0.1)
    R1, Y1 = random_R1(M, 3), random_sym(M, 4, scale=1e-3)
    f, d2v = _noalloc(gpu_lib, ens, R1, Y1, 1)
    assert np.all(np.isfinite(f)) and np.all(np.isfinite(d2v))
    bad = dict(ens)
    bad["X"] = ens["X"].copy()
    bad["X"][N - 1, M - 1] = np.inf
    f, d2v = _noalloc(gpu_lib, bad, R1, Y1, 1)
    assert np.all(np.isnan(f)) and np.all(np.isnan(d2v))
    bad = dict(ens, w=ens["w"].copy())
    bad["w"][0] = 0.0
    f, d2v = _noalloc(gpu_lib, bad, R1, Y1, 1)
    assert np.all(np.isnan(f)) and np.all(np.isnan(d2v))
    # the next valid call is unaffected
    f2, d2 = _noalloc(gpu_lib, ens, R1, Y1, 1)
    assert np.all(np.isfinite(f2)) and np.all(np.isfinite(d2))
