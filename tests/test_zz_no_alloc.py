"""The allocation-free float64 entry point (tdscha_perturb_averages_noalloc).

It exists for callers that cannot let the library allocate device memory
(programs that own the whole GPU memory budget, or loops that cannot afford
cudaMalloc's synchronisation).  Checked through the C ABI against the
context entry point (tdscha_perturb_averages, float64) on two calls in a
row, which share the static scratch area.  Collected last on purpose."""
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
