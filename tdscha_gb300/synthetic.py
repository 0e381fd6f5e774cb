"""Seeded synthetic SCHA ensembles in the mode basis.

The reference builds X (mass-scaled displacements) and Y (mass-scaled forces
minus the SSCHA and mean forces) projected on the polarisation vectors,
C-order (N, M) float64 (Modules/DynamicalLanczos.py:392-452). Here the same
arrays are drawn directly in the mode basis:

* omega_mu ~ U[w_min, w_max] cm^-1 converted to Ry (per degenerate block);
* X_i ~ N(0, diag(f_psi(omega))), the SCHA Gaussian, f_psi = (1+2n)/(2 omega)
  (CModules/LanczosFunctions.c:24-30);
* Y = -1/2 Phi3:XX - 1/6 Phi4:XXX with Phi3, Phi4 fully symmetric random
  tensors held in symmetric CP form (sum_k c_k g_k^{x3}, sum_k d_k h_k^{x4}),
  so that they never need M^3 / M^4 storage; each is rescaled so its force
  has `anh_scale` times the RMS of the harmonic force -Phi2 X with
  Phi2 = diag(omega^2); the weighted mean force is then subtracted;
* rho = 1 or log-normal(0, sigma);
* symmetry images (optional): modes grouped in degenerate triplets, every
  group element acts on each triplet as a signed 3x3 permutation matrix
  (the 48 elements of O_h), stored as the reference's per-block tables
  (symmetries[b]: (S, deg, deg), degenerate_space[b], sym_block_id).
"""
import itertools

import numpy as np

RY_TO_K = 157887.32400374097
RY_TO_CM = 109691.40235


def f_psi(w, T):
    """(1 + 2 n) / (2 w), the covariance eigenvalue (LanczosFunctions.c:24)."""
    n = np.zeros_like(w) if T <= 0 else 1.0 / np.expm1(w * RY_TO_K / T)
    return (1 + 2 * n) / (2 * w)


def f_ups(w, T):
    """2 w / (1 + 2 n), the inverse covariance eigenvalue (LanczosFunctions.c:14)."""
    n = np.zeros_like(w) if T <= 0 else 1.0 / np.expm1(w * RY_TO_K / T)
    return 2 * w / (1 + 2 * n)


def oh_group():
    """The 48 signed 3x3 permutation matrices (the cubic point group O_h)."""
    mats = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1.0, -1.0), repeat=3):
            m = np.zeros((3, 3))
            for r, c in enumerate(perm):
                m[r, c] = signs[r]
            mats.append(m)
    return np.array(mats)


def _cp_force(Xs, order, rank, rng):
    """-(1/order!)*order * Phi:X^{order-1} for a symmetric CP tensor Phi.

    Phi = sum_k c_k g_k^{(x)order}; the derivative of (1/order!) Phi:X^order
    is (1/(order-1)!) sum_k c_k (g_k.X)^(order-1) g_k.
    """
    M = Xs.shape[1]
    G = rng.standard_normal((rank, M)) / np.sqrt(M)
    c = rng.standard_normal(rank)
    proj = Xs @ G.T                      # (N, rank)
    fact = 2.0 if order == 3 else 6.0
    return -((proj ** (order - 1)) * c) @ G / fact


def make_ensemble(M, N, seed=0, T=300.0, n_syms=1, rho_sigma=0.0,
                  w_min_cm=50.0, w_max_cm=500.0, anh_scale=0.05, rank=None,
                  dtype=np.float64):
    """Return a dict with X, Y, w, rho, T and (if n_syms > 1) the symmetry tables."""
    rng = np.random.default_rng(seed)
    if n_syms > 1:
        if M % 3:
            raise ValueError("symmetric ensembles need M divisible by 3")
        nb = M // 3
        wb = rng.uniform(w_min_cm, w_max_cm, nb)
        wb.sort()
        w = np.repeat(wb, 3) / RY_TO_CM
    else:
        w = np.sort(rng.uniform(w_min_cm, w_max_cm, M)) / RY_TO_CM
    sig = np.sqrt(f_psi(w, T))
    X = rng.standard_normal((N, M)) * sig
    R = rank if rank is not None else max(8, min(M, 64))
    h_force = X * (w ** 2)
    h_rms = np.sqrt(np.mean(h_force ** 2))
    f3 = _cp_force(X, 3, R, rng)
    f3 *= anh_scale * h_rms / max(np.sqrt(np.mean(f3 ** 2)), 1e-300)
    f4 = _cp_force(X, 4, R, rng)
    f4 *= anh_scale * h_rms / max(np.sqrt(np.mean(f4 ** 2)), 1e-300)
    Y = f3 + f4
    if rho_sigma > 0:
        rho = np.exp(rng.normal(0.0, rho_sigma, N))
    else:
        rho = np.ones(N)
    Y -= (rho[:, None] * Y).sum(0) / rho.sum()
    ens = dict(X=np.ascontiguousarray(X, dtype=dtype),
               Y=np.ascontiguousarray(Y, dtype=dtype),
               w=w.astype(np.float64), rho=rho.astype(np.float64), T=float(T))
    if n_syms > 1:
        G = oh_group()
        if n_syms > len(G):
            raise ValueError("at most 48 images")
        # identity first, then a seeded choice of the remaining elements
        order = [0] + list(rng.permutation(np.arange(1, len(G)))[: n_syms - 1])
        Gs = G[order]
        nb = M // 3
        syms, spaces = [], []
        for b in range(nb):
            # pseudo-vector representation on odd blocks: det(R) * R
            if b % 2:
                blk = np.array([np.linalg.det(g) * g for g in Gs])
            else:
                blk = Gs.copy()
            syms.append(np.ascontiguousarray(blk))
            spaces.append(np.arange(3 * b, 3 * b + 3, dtype=np.intc))
        ens["symmetries"] = syms
        ens["degenerate_space"] = spaces
        ens["sym_block_id"] = np.repeat(np.arange(nb), 3).astype(np.intc)
    return ens


def random_R1(M, seed=1):
    """Random unit R1 vector (the R sector of psi, as prepare_perturbation sets it)."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(M)
    return v / np.linalg.norm(v)


def random_sym(M, seed=2, scale=1.0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, M)) * scale
    return (A + A.T) / 2


# Workloads named by what they are (mode count, configurations, images, steps).
WORKLOADS = {
    "m21_n1k": dict(M=21, N=1000, n_syms=1, rho_sigma=0.0, steps=50),
    # check_steps: the mixed-vs-float64 spectral check runs over the window in
    # which two float64 runs of this symmetric operator reproduce each other
    "m189_n10k_s48": dict(M=189, N=10000, n_syms=48, rho_sigma=0.1, steps=200, check_steps=50),
    "m573_n50k": dict(M=573, N=50000, n_syms=1, rho_sigma=0.1, steps=300),
    # same modes, 20 000 configurations: the operands still exceed L2 but the
    # whole context stays under 1 GB (used for full profiler captures)
    "m573_n20k": dict(M=573, N=20000, n_syms=1, rho_sigma=0.1, steps=300),
}


def qgrid(dims):
    """Monkhorst-Pack-style Gamma-centred grid in crystal coordinates."""
    d = list(dims) + [1] * (3 - len(dims))
    return np.array([[i / d[0], j / d[1], k / d[2]] for i in range(d[0]) for j in range(d[1])
                     for k in range(d[2])])


def make_qspace_ensemble(dims, nb, N, seed=0, T=300.0, w_min_cm=50.0, w_max_cm=500.0,
                         dispersion=0.0, anh_scale=0.05, rho_sigma=0.0, rank=None):
    """Seeded supercell ensemble and its Bloch transform.

    Real-space cells R on the grid `dims` (n_q cells), nb bands per cell with
    frequencies w_q[nu, q] = w_nu * (1 + dispersion * (1 - cos 2 pi q.1)/2);
    displacements drawn in q space with X_{-q} = conj(X_q) (so the supercell
    data are real), transformed back to real space, forces from a fully
    symmetric CP cubic + quartic potential of the real-space coordinates,
    then Bloch transformed:
        X_q[iq, i, nu] = n_q^{-1/2} sum_R exp(-2 pi i q.R) u[i, R, nu].
    Returns the q-space arrays and the matching real-space ones (modes ordered
    band-major: index nu * n_q + R).
    """
    rng = np.random.default_rng(seed)
    q = qgrid(dims)
    n_q = len(q)
    R = q * np.array(list(dims) + [1] * (3 - len(dims)))[None, :]   # integer cell coords
    d = list(dims) + [1] * (3 - len(dims))
    cells = np.array([[i, j, k] for i in range(d[0]) for j in range(d[1]) for k in range(d[2])])
    wb = np.sort(rng.uniform(w_min_cm, w_max_cm, nb)) / RY_TO_CM
    w_q = np.zeros((nb, n_q))
    for iq in range(n_q):
        w_q[:, iq] = wb * (1 + dispersion * (1 - np.cos(2 * np.pi * q[iq].sum())) / 2)
    phase = np.exp(-2j * np.pi * (q @ cells.T))              # (n_q, n_cells)
    # displacements: real-space Gaussian with the per-q covariance, via q space
    X_q = np.zeros((n_q, N, nb), dtype=np.complex128)
    minus = np.array([np.argmin(np.abs(((q + q[i] + 0.5) % 1.0) - 0.5).sum(1)) for i in range(n_q)])
    for iq in range(n_q):
        jq = minus[iq]
        sig = np.sqrt(f_psi(w_q[:, iq], T))
        if jq == iq:
            X_q[iq] = rng.standard_normal((N, nb)) * sig
        elif iq < jq:
            z = (rng.standard_normal((N, nb)) + 1j * rng.standard_normal((N, nb))) / np.sqrt(2)
            X_q[iq] = z * sig
            X_q[jq] = np.conj(X_q[iq])
    u = np.real(np.einsum("qc,qin->icn", np.conj(phase), X_q, optimize=True)) / np.sqrt(n_q)   # (N, cells, nb)
    M = n_q * nb
    ureal = np.ascontiguousarray(np.transpose(u, (0, 2, 1)).reshape(N, M))     # band-major
    Rk = rank if rank is not None else max(8, min(M, 64))
    wreal = np.repeat(wb, n_q)
    h_rms = np.sqrt(np.mean((ureal * wreal ** 2) ** 2))
    f3 = _cp_force(ureal, 3, Rk, rng)
    f3 *= anh_scale * h_rms / max(np.sqrt(np.mean(f3 ** 2)), 1e-300)
    f4 = _cp_force(ureal, 4, Rk, rng)
    f4 *= anh_scale * h_rms / max(np.sqrt(np.mean(f4 ** 2)), 1e-300)
    freal = f3 + f4
    rho = np.exp(rng.normal(0.0, rho_sigma, N)) if rho_sigma > 0 else np.ones(N)
    freal -= (rho[:, None] * freal).sum(0) / rho.sum()
    fcell = np.transpose(freal.reshape(N, nb, n_q), (0, 2, 1))                  # (N, cells, nb)
    Y_q = np.einsum("qc,icn->qin", phase, fcell, optimize=True) / np.sqrt(n_q)
    return dict(X_q=X_q, Y_q=Y_q, w_q=w_q, rho=rho, T=float(T), q=q, dims=tuple(d),
                X_real=ureal, Y_real=freal, w_real=wreal, n_q=n_q, nb=nb, cells=cells)


def translation_tables(n_q, nb, cells, dims):
    """Real-space symmetry tables of all lattice translations (band-major modes):
    one block per band (its n_q cell copies), each translation a permutation."""
    d = np.array(dims)
    idx = {tuple(c): i for i, c in enumerate(cells)}
    blocks = []
    for nu in range(nb):
        mats = np.zeros((n_q, n_q, n_q))
        for t, tc in enumerate(cells):
            for r, rc in enumerate(cells):
                s = idx[tuple((rc + tc) % d)]
                mats[t, s, r] = 1.0
        blocks.append(mats)
    spaces = [np.arange(nu * n_q, (nu + 1) * n_q, dtype=np.intc) for nu in range(nb)]
    bid = np.repeat(np.arange(nb), n_q).astype(np.intc)
    return blocks, spaces, bid


# q-space workloads: Gamma-centred grid, bands per q-point, configurations
QWORKLOADS = {
    # a 4x4x4 supercell of a 4-atom cell (768 real-space modes), 10 000 configurations
    "q444_nb12_n10k": dict(dims=(4, 4, 4), nb=12, N=10000, steps=100),
    "q222_nb6_n2k": dict(dims=(2, 2, 2), nb=6, N=2000, steps=50),
}
