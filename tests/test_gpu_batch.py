"""Batched runs (tdscha_lanczos_run_batch) give exactly what the runs give
one at a time."""
import numpy as np
import pytest

from tdscha_gb300 import _native as nat
from tdscha_gb300.batch import run_batch
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.QSpaceLanczos import QSpaceLanczos
from tdscha_gb300.synthetic import make_ensemble, make_qspace_ensemble, random_R1

pytestmark = pytest.mark.gpu


def _real(M, N, seed, wigner, precision, reorth):
    e = make_ensemble(M, N, seed=seed, rho_sigma=0.1)
    lz = Lanczos.from_arrays(e["X"], e["Y"], e["w"], e["rho"], e["T"], use_wigner=wigner,
                             precision=precision)
    lz.init(use_symmetries=False)
    lz.full_reorth = reorth
    lz.prepare_perturbation(random_R1(M, seed + 1), masses_exp=0)
    return lz


def _q(dims, nb, N, seed):
    e = make_qspace_ensemble(dims, nb, N, seed=seed, dispersion=0.2)
    ql = QSpaceLanczos.from_arrays(e["X_q"], e["Y_q"], e["w_q"], e["rho"], e["T"], q_points=e["q"])
    ql.init(use_symmetries=False)
    ql.prepare_mode_q(0, 1)
    return ql


def _make():
    return [_real(48, 3000, 1, False, "mixed", True), _real(96, 5000, 2, True, "fp64", False),
            _real(30, 800, 3, False, "fp64", True), _q((2, 2, 1), 3, 300, 4)]


def test_batch_equals_sequential(gpu_lib):
    n = 20
    seq = _make()
    for lz in seq:
        lz.run_FT(n, verbose=False)
    bat = _make()
    out = run_batch(bat, n)
    assert all(s == 0 for _, _, s in out)
    for a, b in zip(seq, bat):
        np.testing.assert_array_equal(a.a_coeffs, b.a_coeffs)
        np.testing.assert_array_equal(a.b_coeffs, b.b_coeffs)
        np.testing.assert_array_equal(a.c_coeffs, b.c_coeffs)
    # continuing a batch equals continuing each run
    for lz in seq:
        lz.run_FT(10, verbose=False)
    run_batch(bat, 10)
    for a, b in zip(seq, bat):
        np.testing.assert_array_equal(a.a_coeffs, b.a_coeffs)


def test_batch_rejects_shared_context(gpu_lib):
    lz = _real(30, 500, 5, False, "fp64", False)
    with pytest.raises(ValueError):
        run_batch([lz, lz], 3)
