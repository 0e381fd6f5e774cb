"""q-space static Hessian: with one q-point and real data it is the real-space
static Hessian, which the reference's own run_hessian_calculation gives
(tests/golden/static_m12_n800.npz)."""
import numpy as np
import pytest

import oracle.qspace as oq
from tdscha_gb300.QSpaceHessian import QSpaceHessian
from tdscha_gb300.QSpaceLanczos import QSpaceLanczos


def _hessian(d, use_oracle):
    X, Y, w = d["X"], d["Y"], d["w"]
    ql = QSpaceLanczos.from_arrays(X[None].astype(complex), Y[None].astype(complex), w[:, None],
                                   d["rho"], float(d["T"]))
    ql.init(use_symmetries=False)
    if use_oracle:
        # the oracle stands in for the GPU averages (host-side logic test)
        def averages(R1, blocks, apply_v4=True):
            return oq.perturb_averages_qspace(ql.X_q, ql.Y_q, ql.w_q, ql.rho, R1, blocks, ql.T,
                                              apply_v4, ql.iq_pert, ql.unique_pairs)
        ql.get_perturb_averages_q = averages
    h = QSpaceHessian.from_qspace_lanczos(ql, verbose=False)
    return h.compute_hessian_at_q(0, tol=1e-10, use_mode_symmetry=False)


def test_single_q_static_hessian_matches_reference_host(golden):
    d = golden("static_m12_n800.npz")
    H = _hessian(d, use_oracle=True)
    ref = d["hessian"]
    assert np.abs(H.imag).max() < 1e-12 * np.abs(ref).max()
    np.testing.assert_allclose(H.real, ref, rtol=0, atol=2e-6 * np.abs(ref).max())


@pytest.mark.gpu
def test_single_q_static_hessian_matches_reference_gpu(gpu_lib, golden):
    d = golden("static_m12_n800.npz")
    H = _hessian(d, use_oracle=False)
    ref = d["hessian"]
    np.testing.assert_allclose(H.real, ref, rtol=0, atol=2e-6 * np.abs(ref).max())
