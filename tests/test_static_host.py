"""Host-side logic of the static response (no GPU)."""
import numpy as np
import pytest

from tdscha_gb300 import Tools
from tdscha_gb300.StaticHessian import StaticHessian


def test_get_G_W_round_trip_matches_loops():
    sh = StaticHessian()
    sh.lanczos.n_modes = 5
    M = 5
    n = M * (M + 1) // 2 + M * (M * M + 3 * M + 2) // 6
    v = np.random.default_rng(0).standard_normal(n)
    G, W = sh.get_G_W(v)
    # the reference's loops (StaticHessian.py:625-658), written out
    G2 = np.zeros((M, M))
    W2 = np.zeros((M, M, M))
    c = 0
    for i in range(M):
        for j in range(i, M):
            G2[i, j] = G2[j, i] = v[c]
            c += 1
    for i in range(M):
        for j in range(i, M):
            for k in range(j, M):
                for a, b, cc in ((i, j, k), (i, k, j), (j, i, k), (j, k, i), (k, i, j), (k, j, i)):
                    W2[a, b, cc] = v[c]
                c += 1
    np.testing.assert_array_equal(G, G2)
    np.testing.assert_array_equal(W, W2)
    np.testing.assert_array_equal(sh.get_vector(G, W), v)


def test_attribute_lock():
    sh = StaticHessian()
    sh.prefix = "x"
    with pytest.raises(AttributeError):
        sh.prefixx = "y"


def test_minimum_residual_solves_spd():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((30, 30))
    A = A @ A.T + 30 * np.eye(30)
    b = rng.standard_normal(30)

    class Op:
        def matvec(self, x):
            return A @ x

    x = Tools.minimum_residual_algorithm(Op(), b, b.copy(), verbose=False, max_iters=200,
                                         conv_thr=1e-12)
    np.testing.assert_allclose(A @ x, b, atol=1e-9)
    D = np.diag(1 / np.sqrt(np.diag(A)))

    class Pre:
        def matvec(self, x):
            return D @ x

    x2 = Tools.minimum_residual_algorithm_precond(Op(), b, Pre(), verbose=False, max_iters=200,
                                                  conv_thr=1e-12)
    np.testing.assert_allclose(A @ x2, b, atol=1e-9)


def test_batched_minimum_residual_equals_sequential():
    torch = pytest.importorskip("torch")
    import oracle
    rng = np.random.default_rng(2)
    A = rng.standard_normal((20, 20))
    A = A @ A.T + 20 * np.eye(20)
    B = rng.standard_normal((4, 20))
    At = torch.from_numpy(A)
    X, iters, conv = Tools.batched_minimum_residual(lambda Z: Z @ At.T, torch.from_numpy(B),
                                                    torch.from_numpy(B.copy()), 100, 1e-10)
    for r in range(4):
        x, it, c = oracle.minimum_residual(lambda v: A @ v, B[r], B[r].copy(), 100, 1e-10)
        np.testing.assert_allclose(X[r].numpy(), x, rtol=1e-10, atol=1e-12)
        assert iters[r] == it and conv[r] == c


def _fake_run(lanc, A, B, C, calls):
    """run_FT stand-in: the prepared mode's coefficients from the tables (the
    generator of tests/golden/no_mode_mixing_m5.npz uses the same rule)."""
    M = A.shape[0]

    def run_FT(n_iter, save_dir=None, verbose=True, prefix="LANCZOS", **kw):
        i = int(np.argmax(np.abs(np.asarray(lanc.psi[:M]))))
        calls.append((i, int(n_iter)))
        lanc.a_coeffs = list(A[i, :n_iter])
        lanc.b_coeffs = list(B[i, :n_iter])
        lanc.c_coeffs = list(C[i, :n_iter])
    return run_FT


def test_run_no_mode_mixing_matches_reference(golden, tmp_path):
    """StaticHessian.run_no_mode_mixing's host logic against the reference's, both
    driven by the same stand-in run: modes run and skipped (a degenerate pair),
    G(0) of the continued fraction without terminator, vector and Hessian."""
    import oracle
    from tdscha_gb300.DynamicalLanczos import Lanczos
    d = golden("no_mode_mixing_m5.npz")
    lanc = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), use_wigner=True)
    calls = []
    lanc.run_FT = _fake_run(lanc, d["A"], d["B"], d["C"], calls)

    def cf(w, use_terminator=True, smearing=0.0):
        return oracle.continued_fraction(lanc.a_coeffs, lanc.b_coeffs, lanc.c_coeffs, w,
                                         lanc.use_wigner, lanc.perturbation_modulus,
                                         use_terminator=use_terminator, smearing=smearing)

    lanc.get_green_function_continued_fraction = cf
    sh = StaticHessian()
    sh.lanczos = lanc
    hess = sh.run_no_mode_mixing(int(d["n_steps"]), noq=True)
    assert [c[0] for c in calls] == list(d["calls"][:, 0])
    np.testing.assert_allclose(sh.vector, d["vector"], rtol=1e-12)
    np.testing.assert_allclose(hess, d["hessian"], rtol=1e-11)
    assert sh.preconitioned is False
    # save_dir: each mode's final status; a second pass resumes from them and runs nothing
    calls.clear()
    sh.run_no_mode_mixing(int(d["n_steps"]), save_dir=str(tmp_path), noq=True)
    assert sorted(p.name for p in tmp_path.glob("*_conv.npz")) == \
        ["hessian_calculation_M%d_conv.npz" % (i + 1) for i in (0, 1, 3, 4)]
    calls.clear()
    sh.run_no_mode_mixing(int(d["n_steps"]), save_dir=str(tmp_path), restart_from_file=True,
                          noq=True)
    assert calls == []
    np.testing.assert_allclose(sh.vector, d["vector"], rtol=1e-12)
