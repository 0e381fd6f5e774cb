"""Ensemble preprocessing on the GPU: the mode projection of Lanczos.__init__
(Modules/DynamicalLanczos.py:392-452) and the Bloch projection of
QSpaceLanczos (Modules/QSpaceLanczos.py:221-296), through
tdscha_project_modes / tdscha_project_bloch."""
import numpy as np

from . import _native as nat

BOHR = 1.889725989      # Angstrom -> Bohr, sscha.Ensemble.Bohr


def project_modes(u, f, masses, pols, f_mean=None, u_scale=1.0 / BOHR, f_scale=BOHR):
    """X = (u u_scale sqrt(m)) . pols, Y = ((f - f_mean) f_scale / sqrt(m)) . pols.

    u: (N, n_cart) displacements, f: (N, n_cart) forces minus SSCHA forces,
    f_mean: (n_cart,) average force tiled on the supercell or None, masses
    (n_cart,), pols (n_cart, M).  Defaults convert Angstrom / Ry/Angstrom to
    Bohr / Ry/Bohr as the reference does."""
    u = nat.f64(u)
    f = nat.f64(f)
    masses = nat.f64(masses)
    pols = nat.f64(pols)
    N, n_cart = u.shape
    if f.shape != u.shape or masses.shape != (n_cart,) or pols.shape[0] != n_cart:
        raise ValueError("shapes: u, f (N, n_cart), masses (n_cart,), pols (n_cart, M)")
    M = pols.shape[1]
    X = np.empty((N, M))
    Y = np.empty((N, M))
    fm = nat.f64(f_mean) if f_mean is not None else None
    nat.check(nat.load().tdscha_project_modes(N, n_cart, M, nat.dp(u), nat.dp(f),
                                              nat.dp(fm) if fm is not None else None,
                                              nat.dp(masses), nat.dp(pols), float(u_scale),
                                              float(f_scale), nat.dp(X), nat.dp(Y)))
    return X, Y


def project_bloch(u_q, f_q, masses, pols_q, f_mean_gamma=None, u_scale=1.0, f_scale=1.0):
    """X_q = (u_q u_scale sqrt(m)) . conj(pols_q), Y_q = ((f_q - f_mean) f_scale /
    sqrt(m)) . conj(pols_q), f_mean subtracted at q index 0.

    u_q, f_q: (n_q, N, n_cart) complex; pols_q: (n_q, n_cart, n_bands) complex
    (the reference stores (n_cart, n_bands, n_q)); masses (n_cart,)."""
    u_q = np.ascontiguousarray(u_q, dtype=np.complex128)
    f_q = np.ascontiguousarray(f_q, dtype=np.complex128)
    pols_q = np.ascontiguousarray(pols_q, dtype=np.complex128)
    n_q, N, n_cart = u_q.shape
    nb = pols_q.shape[2]
    if f_q.shape != u_q.shape or pols_q.shape[:2] != (n_q, n_cart):
        raise ValueError("shapes: u_q, f_q (n_q, N, n_cart), pols_q (n_q, n_cart, n_bands)")
    X = np.empty((n_q, N, nb), dtype=np.complex128)
    Y = np.empty_like(X)
    fm = (np.ascontiguousarray(f_mean_gamma, dtype=np.complex128).view(np.float64)
          if f_mean_gamma is not None else None)
    nat.check(nat.load().tdscha_project_bloch(
        n_q, N, n_cart, nb, nat.dp(u_q.view(np.float64)), nat.dp(f_q.view(np.float64)),
        nat.dp(fm) if fm is not None else None, nat.dp(nat.f64(masses)),
        nat.dp(pols_q.view(np.float64)), float(u_scale), float(f_scale),
        nat.dp(X.view(np.float64)), nat.dp(Y.view(np.float64))))
    return X, Y
