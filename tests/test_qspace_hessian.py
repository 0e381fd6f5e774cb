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


def test_static_propagator_limits():
    """Lambda is continuous across the degenerate limit and reduces to
    1 / (4 w1 w2 (w1 + w2)) at T = 0."""
    from tdscha_gb300.QSpaceHessian import static_propagator
    w = np.array([1e-3, 2e-3, 2e-3 + 1e-9, 3e-3])
    v = np.ones(4, bool)
    lam = static_propagator(w, v, w, v, 300.0)
    np.testing.assert_allclose(lam[1, 2], lam[1, 1], rtol=1e-5)
    # inside the 1e-8 Ry window the derivative is taken at the row mode
    np.testing.assert_allclose(lam, lam.T, rtol=1e-6)
    lam0 = static_propagator(w, v, w, v, 0.0)
    np.testing.assert_allclose(lam0, 1.0 / (4 * np.outer(w, w) * np.add.outer(w, w)), rtol=1e-14)
    v[0] = False
    assert np.all(static_propagator(w, v, w, v, 300.0)[0] == 0)


def test_degenerate_groups_and_schur_fill():
    from tdscha_gb300.QSpaceHessian import _fill_green, degenerate_groups
    w = np.array([0.0, 5.0, 2.0, 5.0, 2.0, 7.0, 5.0])
    valid = np.array([False, True, True, True, True, True, True])
    groups = degenerate_groups(w, valid)
    assert groups == [[1, 3, 6], [2, 4], [5]]
    nb = len(w)
    x = {k: np.arange(nb) + 10.0 * k for k in range(3)}
    G = _fill_green(np.zeros((nb, nb)), groups, [x[0], x[1], x[2]], nb)
    # triplet: c * I on its own block, nothing else of its size
    assert G[1, 1] == G[3, 3] == G[6, 6] == x[0][1] and G[3, 1] == 0
    assert G[2, 2] == G[4, 4] == x[1][2]
    assert G[5, 5] == x[2][5] and G[1, 5] == 0 and G[2, 5] == 0
