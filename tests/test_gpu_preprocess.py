"""Ensemble preprocessing and gamma_only projection on the GPU vs the oracle."""
import numpy as np
import pytest

import oracle
from tdscha_gb300.DynamicalLanczos import Lanczos
from tdscha_gb300.preprocessing import BOHR, project_bloch, project_modes
from tdscha_gb300.synthetic import make_qspace_ensemble, translation_tables

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(b).max()


def test_project_modes(gpu_lib):
    rng = np.random.default_rng(0)
    N, n_cart, M = 700, 30, 27
    u = rng.standard_normal((N, n_cart)) * 0.1
    f = rng.standard_normal((N, n_cart)) * 0.01
    m = rng.uniform(1e4, 1e5, n_cart)
    pols = np.linalg.qr(rng.standard_normal((n_cart, n_cart)))[0][:, :M]
    fm = rng.standard_normal(n_cart) * 1e-3
    X, Y = project_modes(u, f, m, pols, fm)
    Xo, Yo = oracle.project_modes(u, f, m, pols, fm, 1 / BOHR, BOHR)
    assert _rel(X, Xo) < 1e-13 and _rel(Y, Yo) < 1e-13
    lz = Lanczos.from_cartesian(u, f + 1.0, np.ones_like(f), m, pols, np.linspace(1e-3, 4e-3, M),
                                np.ones(N), 300.0, f_mean=fm)
    assert _rel(lz.X, Xo) < 1e-13 and _rel(lz.Y, Yo) < 1e-12


def test_project_bloch(gpu_lib):
    rng = np.random.default_rng(1)
    n_q, N, n_cart, nb = 4, 300, 9, 9
    cplx = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)
    u_q, f_q, pols_q = cplx(n_q, N, n_cart), cplx(n_q, N, n_cart), cplx(n_q, n_cart, nb)
    m = rng.uniform(1e4, 1e5, n_cart)
    fm = cplx(n_cart)
    X, Y = project_bloch(u_q, f_q, m, pols_q, fm, u_scale=0.5, f_scale=2.0)
    sq = np.sqrt(m)
    for iq in range(n_q):
        Xo = (u_q[iq] * 0.5 * sq) @ np.conj(pols_q[iq])
        df = f_q[iq] - (fm if iq == 0 else 0)
        Yo = (df * (2.0 / sq)) @ np.conj(pols_q[iq])
        assert _rel(X[iq], Xo) < 1e-13 and _rel(Y[iq], Yo) < 1e-13


def test_gamma_only_projection(gpu_lib):
    """Operator with the translation projection (pols = identity, translations
    of a 3x2x1 supercell as permutations of band-major modes) vs the oracle."""
    e = make_qspace_ensemble((3, 2, 1), 2, 200, seed=6, dispersion=0.2)
    n_q, nb = e["n_q"], 2
    M = n_q * nb
    blocks, _, _ = translation_tables(n_q, nb, e["cells"], e["dims"])
    perms = []
    for t in range(n_q):
        p = np.zeros(M, dtype=int)
        for nu in range(nb):
            src = np.argmax(blocks[nu][t], axis=1)       # P_t[s, r] = 1: row s from r
            p[nu * n_q:(nu + 1) * n_q] = nu * n_q + src
        perms.append(p)
    lz = Lanczos.from_arrays(e["X_real"], e["Y_real"], e["w_real"], e["rho"], e["T"],
                             use_wigner=True)
    lz.init(use_symmetries=False)
    lz.set_translations(perms)
    ol = oracle.OracleLanczos(dict(X=e["X_real"], Y=e["Y_real"], w=e["w_real"], rho=e["rho"],
                                   T=e["T"]))
    ol.trans = (np.eye(M), perms)
    rng = np.random.default_rng(2)
    psi = rng.standard_normal(M + M * (M + 1)) * 1e-2
    got = lz.apply_full_L(psi.copy())
    ref = ol.apply_full_L(psi)
    assert _rel(got, ref) < 1e-11
    np.testing.assert_allclose(lz.trans_projector, oracle.translation_projector(np.eye(M), perms))
