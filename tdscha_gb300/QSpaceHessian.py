"""Drop-in for tdscha.QSpaceHessian (Modules/QSpaceHessian.py) on the GPU.

The free-energy Hessian at a q-point is H_q = G_q^-1, with G_q[:, i] the R part
of the solution of L_static(q) x = e_i.  The static q-space operator acts on a
vector [R (n_bands) | W blocks of the unique q-pairs]:

    R -> w_q^2 R - f,     W_p -> W_p / Lambda_p + d2v_p,

where (f, d2v) are the q-space perturbation averages with R1 = R and
Y1_p = -2 (Y_w1 Y_w2^T) * W_p (Modules/QSpaceHessian.py:605-692).  The
averages, which carry all the cost, run on the GPU through the q-space context
(tdscha_qperturb_averages); everything here is host logic around them.

Design.  `_StaticQOperator` is built once per q-point and works on flat
vectors: the harmonic part is one elementwise product with a precomputed
diagonal, the W blocks are gathered from / scattered to the flat layout with
precomputed index arrays (a self-paired block is stored as its upper triangle
and expanded with its Hermitian conjugate).  The solves run in the metric-
symmetric variables x~ = sqrt(m) x (m the static inner-product weights), with
the inverse harmonic diagonal as preconditioner and as starting point; each
right-hand side goes through a chain of solvers (GMRES, then BiCGSTAB, then
-- only when allowed -- a least-squares solve of the assembled Hermitian
matrix), the first one that converges wins.
"""
import os
import time

import numpy as np
import scipy.sparse.linalg

from .QSpaceLanczos import QSpaceLanczos, RY_TO_K

__EPSILON__ = 1e-12
_DEGENERACY_TOL = 1e-8        # Ry, frequencies closer than this form one block


# ----------------------------------------------------------------- physics
def _occupations(w, valid, T):
    """Bose occupation of the valid modes (0 at T = 0 and on masked modes)."""
    n = np.zeros_like(w, dtype=np.float64)
    if T > __EPSILON__:
        n[valid] = 1.0 / np.expm1(w[valid] * (RY_TO_K / T))
    return n


def static_propagator(w1, valid1, w2, valid2, T):
    """Static two-phonon propagator Lambda[nu1, nu2] of a q-pair.

    Lambda = [(1 + n1 + n2) / (w1 + w2) - Dn] / (4 w1 w2), where Dn is the
    divided difference (n1 - n2) / (w1 - w2) of the Bose function and, for
    |w1 - w2| < 1e-8 Ry, its derivative dn/dw = -beta n (n + 1).  Zero where
    either mode is masked (Modules/QSpaceHessian.py:481-544 states the same
    propagator)."""
    n1 = _occupations(w1, valid1, T)[:, None]
    n2 = _occupations(w2, valid2, T)[None, :]
    a, b = np.asarray(w1, float)[:, None], np.asarray(w2, float)[None, :]
    ok = valid1[:, None] & valid2[None, :]
    gap = a - b
    close = np.abs(gap) < _DEGENERACY_TOL
    dn = np.zeros(ok.shape)
    if T > __EPSILON__:
        beta = RY_TO_K / T
        with np.errstate(divide="ignore", invalid="ignore"):
            dn = np.where(close, -beta * n1 * (n1 + 1.0), (n1 - n2) / np.where(close, 1.0, gap))
        dn = np.where(close & ~ok, 0.0, dn)
    with np.errstate(divide="ignore", invalid="ignore"):
        lam = ((1.0 + n1 + n2) / (a + b) - dn) / (4.0 * a * b)
    return np.where(ok, lam, 0.0)


def _f_upsilon(w, valid, T):
    """2 w / (2 n + 1) on valid modes, 0 elsewhere."""
    out = np.zeros_like(w, dtype=np.float64)
    n = _occupations(w, valid, T)
    out[valid] = 2.0 * w[valid] / (1.0 + 2.0 * n[valid])
    return out


def degenerate_groups(w, valid, tol=_DEGENERACY_TOL):
    """Valid bands grouped into runs of equal frequency (consecutive sorted
    frequencies closer than tol), each group sorted, groups ordered by their
    first band."""
    idx = np.flatnonzero(valid)
    if idx.size == 0:
        return []
    order = idx[np.argsort(w[idx], kind="stable")]
    cuts = np.flatnonzero(np.diff(w[order]) >= tol) + 1
    groups = [sorted(int(i) for i in g) for g in np.split(order, cuts)]
    return sorted(groups, key=lambda g: g[0])


# ---------------------------------------------------------------- operator
class _StaticQOperator:
    """The static operator of one perturbation q-point on flat vectors."""

    def __init__(self, qlanc, ignore_v3, ignore_v4):
        q = qlanc
        nb = q.n_bands
        self.q, self.nb = q, nb
        self.ignore_v3, self.ignore_v4 = ignore_v3, ignore_v4
        self.size = q.get_static_psi_size()
        self.n_pairs = len(q.unique_pairs)
        T = q.T
        vq = q.valid_modes_q
        wq = q.w_q
        diag = np.zeros(self.size)          # harmonic static operator
        weight = np.zeros(self.size)        # inner-product weights
        iq = q.iq_pert
        diag[:nb] = wq[:, iq] ** 2
        weight[:nb] = vq[:, iq]
        self._precond = np.zeros(self.size)
        self._precond[:nb] = np.where(vq[:, iq], 1.0 / np.where(vq[:, iq], wq[:, iq], 1.0) ** 2,
                                      0.0)
        iu_r, iu_c = np.triu_indices(nb)
        self._gather = []                   # per pair: (flat positions, rows, cols, self-paired)
        self._yw = np.zeros((self.n_pairs, nb, nb))
        for p, (q1, q2) in enumerate(q.unique_pairs):
            off = q.get_block_offset(p, "a")
            v1, v2 = vq[:, q1], vq[:, q2]
            lam = static_propagator(wq[:, q1], v1, wq[:, q2], v2, T)
            both = v1[:, None] & v2[None, :]
            if q1 < q2:
                rows, cols = np.divmod(np.arange(nb * nb), nb)
                w_el = np.where(both, 2.0, 0.0)[rows, cols]
            else:
                rows, cols = iu_r, iu_c
                w_el = np.where(both[rows, cols], np.where(rows == cols, 1.0, 2.0), 0.0)
            pos = off + np.arange(rows.size)
            el = lam[rows, cols]
            big = np.abs(el) > 1e-30
            diag[pos] = np.where(big, 1.0 / np.where(big, el, 1.0), 0.0)
            self._precond[pos] = el
            weight[pos] = w_el
            self._gather.append((pos, rows, cols, q1 == q2))
            self._yw[p] = -2.0 * np.outer(_f_upsilon(wq[:, q1], v1, T), _f_upsilon(wq[:, q2], v2, T))
        self.diag = diag
        self.weight = weight
        self.sqrt_w = np.sqrt(weight)
        self.inv_sqrt_w = np.where(weight > 0, 1.0 / np.where(weight > 0, self.sqrt_w, 1.0), 0.0)
        self.applications = 0

    # flat <-> blocks
    def blocks(self, x):
        out = np.zeros((self.n_pairs, self.nb, self.nb), dtype=np.complex128)
        for p, (pos, r, c, herm) in enumerate(self._gather):
            out[p, r, c] = x[pos]
            if herm:
                off = r != c
                out[p, c[off], r[off]] = np.conj(x[pos][off])
        return out

    def scatter(self, blocks, x):
        for p, (pos, r, c, _) in enumerate(self._gather):
            x[pos] = blocks[p][r, c]
        return x

    def anharmonic(self, x):
        """[-f | d2v] of the GPU averages (Modules/QSpaceHessian.py:640-692)."""
        out = np.zeros(self.size, dtype=np.complex128)
        if self.ignore_v3 and self.ignore_v4:
            return out
        R1 = np.zeros(self.nb, dtype=np.complex128) if self.ignore_v3 else \
            np.array(x[:self.nb], dtype=np.complex128)
        Y1 = self._yw * self.blocks(x)
        f, d2v = self.q.get_perturb_averages_q(R1, list(Y1), not self.ignore_v4)
        out[:self.nb] = -np.asarray(f)
        self.applications += 1
        return self.scatter(np.asarray(d2v), out)

    def apply(self, x):
        return self.diag * x + self.anharmonic(x)

    # metric-symmetric form
    def apply_tilde(self, xt):
        return self.apply(xt * self.inv_sqrt_w) * self.sqrt_w

    def precondition_tilde(self, xt):
        return self._precond * xt * (self.weight > 0)

    def dense_tilde(self):
        """The Hermitian part of the operator in x~ variables, column by column."""
        A = np.empty((self.size, self.size), dtype=np.complex128)
        e = np.zeros(self.size, dtype=np.complex128)
        for j in range(self.size):
            e[j] = 1.0
            A[:, j] = self.apply_tilde(e)
            e[j] = 0.0
        return 0.5 * (A + A.conj().T)


# ------------------------------------------------------------------ solvers
def _scipy_solver(fn):
    def run(A, b, x0, tol, maxiter, M, counter):
        kw = dict(x0=x0, maxiter=maxiter, M=M)
        if counter is not None:
            kw.update(callback=counter, callback_type="legacy")
        try:
            return fn(A, b, rtol=tol, **kw)
        except TypeError:                   # scipy releases before the rtol keyword
            return fn(A, b, tol=tol, **kw)
    return run


_gmres = _scipy_solver(scipy.sparse.linalg.gmres)
_bicgstab_raw = _scipy_solver(scipy.sparse.linalg.bicgstab)


def _bicgstab(A, b, x0, tol, maxiter, M, counter):
    return _bicgstab_raw(A, b, x0, tol, maxiter, M, None)


def _solve_chain(op, rhs, x0, tol, max_iters, M, dense_allowed, dense_cache, label):
    """Solve op x = rhs: GMRES (the operator may be indefinite), then BiCGSTAB
    from GMRES's last iterate, then a least-squares solve of the assembled
    matrix if dense_allowed.  Returns (x, iterations)."""
    iters = [0]

    def count(_):
        iters[0] += 1

    A = scipy.sparse.linalg.LinearOperator((op.size, op.size), matvec=op.apply_tilde,
                                           dtype=np.complex128)
    x, info = x0, 1
    for solver in (_gmres, _bicgstab):
        x, info = solver(A, rhs, x, tol, max_iters, M, count)
        if info == 0:
            return x, iters[0]
    if not dense_allowed:
        raise RuntimeError("Iterative solvers (GMRES, BiCGSTAB) did not converge for {} "
                           "(info={}). Set dense_fallback=True to use a dense solve "
                           "(warning: O(psi_size^2) memory).".format(label, info))
    if "A" not in dense_cache:
        dense_cache["A"] = op.dense_tilde()
    return np.linalg.lstsq(dense_cache["A"], rhs, rcond=1e-10)[0], iters[0]


def _fill_green(G, groups, solutions, nb):
    """Columns of G_q from one solve per group (Schur's lemma: between two
    copies of the same d-dimensional irrep G is a multiple of I_d, between
    different irreps zero).  solutions[k] is the R part of the solve for the
    first band of groups[k]; G[C_j, B_j] = x_B[C_0] for every pair of groups
    B, C of equal size, j = 0..d-1.  Without degeneracies every group is a
    single band and this is G[c, b] = x_b[c]."""
    by_size = {}
    for k, g in enumerate(groups):
        by_size.setdefault(len(g), []).append(k)
    for d, members in by_size.items():
        for kb in members:
            x = solutions[kb]
            for kc in members:
                C = groups[kc]
                for j in range(d):
                    G[C[j], groups[kb][j]] = x[C[0]]
    return G


# ------------------------------------------------------------------- driver
class QSpaceHessian:
    """Free-energy Hessian of every q-point from the static q-space operator
    (Modules/QSpaceHessian.py:57).  `H_q_dict[iq]` holds the mode-basis
    Hessian (n_bands x n_bands, complex) of each solved q-point."""

    def __init__(self, ensemble=None, verbose=True, ignore_v3=False, ignore_v4=False, **kwargs):
        qlanc = QSpaceLanczos(ensemble, **kwargs) if ensemble is not None else QSpaceLanczos()
        self._attach(qlanc, verbose)
        self.ensemble = ensemble
        self.ignore_v3 = ignore_v3
        self.ignore_v4 = ignore_v4

    def _attach(self, qlanc, verbose):
        object.__setattr__(self, "qlanc", qlanc)
        self.verbose = verbose
        for name in ("n_q", "n_bands", "q_points", "w_q", "pols_q"):
            setattr(self, name, getattr(qlanc, name))
        self.H_q_dict = {}
        self.irr_qpoints = None
        self.q_star_map = None
        self.last_operator = None

    def __setattr__(self, name, value):
        """The ignore flags are shared with the q-space engine."""
        super().__setattr__(name, value)
        if name in ("ignore_v3", "ignore_v4") and getattr(self, "qlanc", None) is not None:
            setattr(self.qlanc, name, value)

    @classmethod
    def from_qspace_lanczos(cls, qlanc, verbose=True, use_symmetries=True):
        """A Hessian driver on the data of an initialised QSpaceLanczos."""
        hess = cls.__new__(cls)
        hess._attach(qlanc, verbose)
        hess.ensemble = getattr(qlanc, "ensemble", None)
        hess.ignore_v3 = qlanc.ignore_v3
        hess.ignore_v4 = qlanc.ignore_v4
        hess._every_qpoint()
        return hess

    def _every_qpoint(self):
        """No irreducible-q reduction (it needs spglib and the crystal): every
        q-point is its own star."""
        self.irr_qpoints = list(range(self.n_q))
        self.q_star_map = {iq: [(iq, np.eye(3), np.zeros(3), False)] for iq in range(self.n_q)}

    def init(self, use_symmetries=True):
        """Initialise the q-space engine; all q-points are solved."""
        self.qlanc.init(use_symmetries=use_symmetries)
        self._every_qpoint()

    def static_operator(self, iq):
        """The static operator with the perturbation at q-point iq."""
        self.qlanc.build_q_pair_map(iq)
        return _StaticQOperator(self.qlanc, self.ignore_v3, self.ignore_v4)

    # ---------------------------------------------------------------- solve
    def compute_hessian_at_q(self, iq, tol=1e-6, max_iters=500, use_preconditioner=True,
                             dense_fallback=False, use_mode_symmetry=True):
        """H_q at one q-point: one static solve per degenerate group of bands
        (or per band without use_mode_symmetry), G_q filled by Schur's lemma,
        H_q the inverse of G_q's Hermitian part on the non-acoustic bands."""
        nb = self.n_bands
        op = self.static_operator(iq)
        self.last_operator = op
        valid = self.qlanc.valid_modes_q[:, iq]
        if use_mode_symmetry:
            groups = degenerate_groups(self.w_q[:, iq], valid)
        else:
            groups = [[int(b)] for b in np.flatnonzero(valid)]
        if self.verbose:
            print("  Solving at q={} ({} non-acoustic bands, {} solves)".format(
                iq, int(valid.sum()), len(groups)))
        M = None
        if use_preconditioner:
            M = scipy.sparse.linalg.LinearOperator((op.size, op.size),
                                                   matvec=op.precondition_tilde,
                                                   dtype=np.complex128)
        dense_cache = {}
        solutions, total = [], 0
        for g in groups:
            rhs = np.zeros(op.size, dtype=np.complex128)
            rhs[g[0]] = op.sqrt_w[g[0]]
            x0 = op.precondition_tilde(rhs) if use_preconditioner else None
            t0 = time.time()
            xt, n_it = _solve_chain(op, rhs, x0, tol, max_iters, M, dense_fallback, dense_cache,
                                    "band {} at iq={}".format(g[0], iq))
            total += n_it
            solutions.append((xt * op.inv_sqrt_w)[:nb])
            if self.verbose:
                print("    Band {}: {} iters, {:.2f}s".format(g[0], n_it, time.time() - t0))
        G = _fill_green(np.zeros((nb, nb), dtype=np.complex128), groups, solutions, nb)
        H = np.zeros((nb, nb), dtype=np.complex128)
        na = np.flatnonzero(valid)
        if na.size:
            Gs = G[np.ix_(na, na)]
            H[np.ix_(na, na)] = np.linalg.inv(0.5 * (Gs + Gs.conj().T))
        H = 0.5 * (H + H.conj().T)
        if self.verbose:
            print("  Total L applications: {}".format(total))
        self.H_q_dict[iq] = H
        return H

    def compute_full_hessian(self, tol=1e-6, max_iters=500, use_preconditioner=True,
                             dense_fallback=False, use_mode_symmetry=True, checkpoint=None):
        """H_q at every q-point, resumable from `checkpoint` (an npz written
        after each q-point).  Returns the dict of mode-basis matrices, or a
        CC.Phonons object when cellconstructor and the dynamical matrix exist."""
        if self.irr_qpoints is None:
            self._every_qpoint()
        done = set()
        if checkpoint is not None and os.path.exists(_npz_name(checkpoint)):
            done = self.load_status(checkpoint)
        for iq in (i for i in self.irr_qpoints if i not in done):
            self.compute_hessian_at_q(iq, tol=tol, max_iters=max_iters,
                                      use_preconditioner=use_preconditioner,
                                      dense_fallback=dense_fallback,
                                      use_mode_symmetry=use_mode_symmetry)
            if checkpoint is not None:
                self.save_status(checkpoint)
        if getattr(self.qlanc, "dyn", None) is None:
            return self.H_q_dict
        return self._as_phonons()

    def _as_phonons(self):
        """Cartesian force constants Phi_q = P H_q P^dagger, P the mass-scaled
        polarisation vectors, as a cellconstructor Phonons object."""
        import cellconstructor as CC
        import cellconstructor.Phonons  # noqa: F401
        dyn = self.qlanc.dyn
        out = CC.Phonons.Phonons(dyn.structure.copy(), nqirr=self.n_q)
        sqrt_m = np.sqrt(self.qlanc.m)[:, None]
        for iq in range(self.n_q):
            P = sqrt_m * self.pols_q[:, :, iq]
            out.dynmats[iq] = P.dot(self.H_q_dict[iq]).dot(P.conj().T)
            out.q_tot[iq] = np.array(dyn.q_tot)[iq]
        out.AdjustQStar()
        return out

    # ---------------------------------------------------------------- files
    def _metadata(self):
        return {"T": np.float64(self.qlanc.T), "n_q": np.int64(self.n_q),
                "n_bands": np.int64(self.n_bands), "ignore_v3": np.bool_(self.ignore_v3),
                "ignore_v4": np.bool_(self.ignore_v4)}

    def save_status(self, fname):
        """Checkpoint: the metadata, the solved q-points and their H_q, under
        the reference's npz keys."""
        keys = np.array(sorted(self.H_q_dict), dtype=np.int64)
        values = (np.stack([self.H_q_dict[int(k)] for k in keys]) if keys.size else
                  np.zeros((0, self.n_bands, self.n_bands), dtype=np.complex128))
        payload = dict(self._metadata(), completed_irr_qpoints=keys, H_q_keys=keys,
                       H_q_values=values)
        uci = getattr(self.qlanc, "uci_structure", None)
        if uci is not None:
            payload.update(unit_cell=uci.unit_cell, coords=uci.coords,
                           atom_types=uci.get_atomic_types())
        np.savez_compressed(_npz_name(fname), **payload)

    def load_status(self, fname):
        """Read a checkpoint into H_q_dict after checking that it belongs to
        this calculation; returns the set of completed q-points."""
        fname = _npz_name(fname)
        if not os.path.exists(fname):
            raise IOError("Checkpoint file not found: {}".format(fname))
        data = dict(np.load(fname, allow_pickle=True))
        mine = self._metadata()
        problems = []
        if not np.isclose(float(data["T"]), float(mine["T"]), atol=1e-10):
            problems.append("T: checkpoint={}, current={}".format(float(data["T"]),
                                                                 float(mine["T"])))
        for k in ("n_q", "n_bands"):
            if int(data[k]) != int(mine[k]):
                problems.append("{}: checkpoint={}, current={}".format(k, int(data[k]),
                                                                      int(mine[k])))
        for k in ("ignore_v3", "ignore_v4"):
            if bool(data[k]) != bool(mine[k]):
                problems.append("{} differs".format(k))
        if problems:
            raise ValueError("Checkpoint metadata mismatch:\n  " + "\n  ".join(problems))
        for k, H in zip(data["H_q_keys"].astype(int), data["H_q_values"]):
            self.H_q_dict[int(k)] = H
        return {int(k) for k in data["completed_irr_qpoints"]}


def _npz_name(fname):
    return fname if fname.lower().endswith(".npz") else fname + ".npz"
