"""Drop-in for tdscha.QSpaceHessian (Modules/QSpaceHessian.py) on the GPU.

The free-energy Hessian at each q-point from the static q-space operator:
L_static = [w^2 on R | 1/Lambda on the W blocks] + the anharmonic coupling,
solved for every non-acoustic band with GMRES (scipy) as the reference does.
The anharmonic coupling -- the ensemble average that dominates the cost --
runs on the GPU through the q-space context (tdscha_qperturb_averages): R1 from
the R sector, Y1 = -2 Upsilon_1 Upsilon_2 W per pair block (:640-692).
"""
import os
import time

import numpy as np
import scipy.sparse.linalg

from .QSpaceLanczos import QSpaceLanczos, RY_TO_K

__EPSILON__ = 1e-12


class QSpaceHessian:
    def __init__(self, ensemble=None, verbose=True, ignore_v3=False, ignore_v4=False, **kwargs):
        qlanc = QSpaceLanczos(ensemble, **kwargs) if ensemble is not None else QSpaceLanczos()
        self._setup(qlanc, verbose)
        self.ensemble = ensemble
        self.ignore_v3 = ignore_v3
        self.ignore_v4 = ignore_v4

    def _setup(self, qlanc, verbose):
        object.__setattr__(self, "qlanc", qlanc)
        self.verbose = verbose
        self.n_q = qlanc.n_q
        self.n_bands = qlanc.n_bands
        self.q_points = qlanc.q_points
        self.w_q = qlanc.w_q
        self.pols_q = qlanc.pols_q
        self.H_q_dict = {}
        self.irr_qpoints = None
        self.q_star_map = None
        self._cached_w_qp_sq = None
        self._cached_inv_w_qp_sq = None
        self._cached_inv_lambda = None
        self._cached_lambda = None
        self._cached_yw_outer = None
        self._has_symmetry_data = False

    def __setattr__(self, name, value):
        """ignore_v3 / ignore_v4 propagate to the q-space engine (:107-114)."""
        super().__setattr__(name, value)
        if name in ("ignore_v3", "ignore_v4") and getattr(self, "qlanc", None) is not None:
            setattr(self.qlanc, name, value)

    @classmethod
    def from_qspace_lanczos(cls, qlanc, verbose=True, use_symmetries=True):
        """Share the data of an initialised QSpaceLanczos (:1071-1129)."""
        hess = cls.__new__(cls)
        hess._setup(qlanc, verbose)
        hess.ensemble = getattr(qlanc, "ensemble", None)
        hess.ignore_v3 = qlanc.ignore_v3
        hess.ignore_v4 = qlanc.ignore_v4
        hess._all_qpoints()
        return hess

    def _all_qpoints(self):
        self.irr_qpoints = list(range(self.n_q))
        self.q_star_map = {iq: [(iq, np.eye(3), np.zeros(3), False)] for iq in range(self.n_q)}

    def init(self, use_symmetries=True):
        """Initialise the engine.  The irreducible-q reduction of the reference
        needs spglib and the crystal structure (:249-338); without them every
        q-point is solved, as the reference does when spglib is missing."""
        self.qlanc.init(use_symmetries=use_symmetries)
        self._all_qpoints()

    # --------------------------------------------------------------- layout
    def _get_static_psi_size(self):
        return self.qlanc.get_static_psi_size()

    def _get_W_block(self, psi, pair_idx):
        return self.qlanc.get_block(pair_idx, sector="a", source=psi)

    def _set_W_block(self, psi, pair_idx, matrix):
        self.qlanc.set_block_in_psi(pair_idx, matrix, "a", psi)

    def _static_mask(self):
        """Inner-product weights of the static psi (:434-479): R sector 1 (0 on
        masked modes), W blocks 2 (1 on self-paired diagonals, 0 if either mode
        is masked)."""
        psi_size = self._get_static_psi_size()
        mask = np.ones(psi_size, dtype=np.float64)
        nb = self.n_bands
        q = self.qlanc
        mask[:nb] = np.where(q.valid_modes_q[:, q.iq_pert], 1.0, 0.0)
        iu = np.triu_indices(nb)
        for p, (iq1, iq2) in enumerate(q.unique_pairs):
            off = q.get_block_offset(p, "a")
            v1, v2 = q.valid_modes_q[:, iq1], q.valid_modes_q[:, iq2]
            invalid = ~v1[:, None] | ~v2[None, :]
            full = np.where(invalid, 0.0, 2.0)
            if iq1 < iq2:
                mask[off:off + nb * nb] = full.ravel()
            else:
                np.fill_diagonal(full, np.where(v1 & v2, 1.0, 0.0))
                mask[off:off + q.get_block_size(p)] = full[iu]
        return mask

    # ----------------------------------------------------- static quantities
    def _bose(self, iq):
        w = self.w_q[:, iq]
        valid = self.qlanc.valid_modes_q[:, iq]
        n = np.zeros_like(w)
        if self.qlanc.T > __EPSILON__:
            n[valid] = 1.0 / (np.exp(w[valid] * (RY_TO_K / self.qlanc.T)) - 1.0)
        return n, valid

    def _compute_lambda_q(self, iq1, iq2):
        """Static two-phonon propagator of pair (iq1, iq2) (:481-544)."""
        T = self.qlanc.T
        w1, w2 = self.w_q[:, iq1][:, None], self.w_q[:, iq2][None, :]
        n1, v1 = self._bose(iq1)
        n2, v2 = self._bose(iq2)
        n1, n2 = n1[:, None], n2[None, :]
        valid = np.outer(v1, v2)
        diff_n = np.zeros(np.broadcast(w1, w2).shape)
        w_equal = np.abs(w1 - w2) < 1e-8
        if T > __EPSILON__:
            beta = RY_TO_K / T
            safe = np.where(w_equal, 1.0, w1 - w2)
            diff_n = np.where(w_equal, 0.0, (n1 - n2) / safe)
            w_eq = np.where(w_equal & valid, w1, 0.0)
            n_eq = np.where(w_equal & valid, n1, 0.0)
            deg = np.where(w_equal & valid, -beta * np.exp(w_eq * beta) * n_eq ** 2, 0.0)
            diff_n = np.where(w_equal, deg, diff_n)
        wsum = np.where(valid, w1 + w2, 1.0)
        wprod = np.where(valid, w1 * w2, 1.0)
        return np.where(valid, ((n1 + n2 + 1) / wsum - diff_n) / (4 * wprod), 0.0)

    def _compute_Y_w(self, iq):
        """2w / (2n + 1), 0 on masked modes (:546-562)."""
        w = self.w_q[:, iq]
        valid = self.qlanc.valid_modes_q[:, iq]
        n = np.zeros_like(w)
        if self.qlanc.T > __EPSILON__:
            n[valid] = 1.0 / (np.exp(w[valid] * RY_TO_K / self.qlanc.T) - 1.0)
        out = np.zeros_like(w)
        out[valid] = 2.0 * w[valid] / (2.0 * n[valid] + 1.0)
        return out

    def _precompute_static_quantities(self):
        """w^2, 1/w^2, Lambda, 1/Lambda, -2 Y_w1 Y_w2^T per pair (:564-600)."""
        q = self.qlanc
        w_qp = self.w_q[:, q.iq_pert]
        vp = q.valid_modes_q[:, q.iq_pert]
        self._cached_w_qp_sq = w_qp ** 2
        self._cached_inv_w_qp_sq = np.where(vp, 1.0 / np.where(vp, w_qp, 1.0) ** 2, 0.0)
        n_pairs = len(q.unique_pairs)
        self._cached_lambda = [None] * n_pairs
        self._cached_inv_lambda = [None] * n_pairs
        self._cached_yw_outer = [None] * n_pairs
        for p, (iq1, iq2) in enumerate(q.unique_pairs):
            lam = self._compute_lambda_q(iq1, iq2)
            self._cached_lambda[p] = lam
            ok = np.abs(lam) > 1e-30
            self._cached_inv_lambda[p] = np.where(ok, 1.0 / np.where(ok, lam, 1.0), 0.0)
            self._cached_yw_outer[p] = -2.0 * np.outer(self._compute_Y_w(iq1), self._compute_Y_w(iq2))

    # -------------------------------------------------------------- operator
    def _apply_L_static_q(self, psi):
        nb = self.n_bands
        out = np.zeros_like(psi)
        out[:nb] = self._cached_w_qp_sq * psi[:nb]
        for p in range(len(self.qlanc.unique_pairs)):
            self._set_W_block(out, p, self._cached_inv_lambda[p] * self._get_W_block(psi, p))
        return out + self._apply_anharmonic_static_q(psi)

    def _apply_anharmonic_static_q(self, psi):
        """R <- -f, W <- d2v from the GPU averages with R1 = psi_R and
        Y1 = -2 Y_w1 Y_w2 W (:640-692)."""
        nb = self.n_bands
        out = np.zeros_like(psi)
        if self.ignore_v3 and self.ignore_v4:
            return out
        R1 = np.array(psi[:nb], dtype=np.complex128)
        if self.ignore_v3:
            R1[:] = 0.0
        Y1 = [self._cached_yw_outer[p] * self._get_W_block(psi, p)
              for p in range(len(self.qlanc.unique_pairs))]
        f, d2v = self.qlanc.get_perturb_averages_q(R1, Y1, not self.ignore_v4)
        out[:nb] = -f
        for p in range(len(self.qlanc.unique_pairs)):
            self._set_W_block(out, p, d2v[p])
        return out

    def _apply_harmonic_preconditioner(self, psi_tilde, sqrt_mask, inv_sqrt_mask):
        nb = self.n_bands
        psi = psi_tilde * inv_sqrt_mask
        res = np.zeros_like(psi)
        res[:nb] = self._cached_inv_w_qp_sq * psi[:nb]
        for p in range(len(self.qlanc.unique_pairs)):
            self._set_W_block(res, p, self._cached_lambda[p] * self._get_W_block(psi, p))
        return res * sqrt_mask

    def _find_degenerate_blocks(self, iq, threshold=1e-8):
        """Non-acoustic bands at iq grouped by equal frequency (|dw| < threshold Ry)."""
        w = self.w_q[:, iq]
        valid = self.qlanc.valid_modes_q[:, iq]
        seen, blocks = set(), []
        for nu in range(self.n_bands):
            if nu in seen:
                continue
            if not valid[nu]:
                seen.add(nu)
                continue
            block = [b for b in range(self.n_bands)
                     if valid[b] and abs(w[b] - w[nu]) < threshold and b not in seen]
            seen.update(block)
            blocks.append(block)
        return blocks

    # ---------------------------------------------------------------- solver
    def compute_hessian_at_q(self, iq, tol=1e-6, max_iters=500, use_preconditioner=True,
                             dense_fallback=False, use_mode_symmetry=True):
        """H_q = inv(G_q), G_q[:, i] the R sector of L_static^-1 e_i (:720-956)."""
        nb = self.n_bands
        self.qlanc.build_q_pair_map(iq)
        psi_size = self._get_static_psi_size()
        self._precompute_static_quantities()
        mask = self._static_mask()
        sqrt_mask = np.sqrt(mask)
        inv_sqrt_mask = np.zeros_like(sqrt_mask)
        nz = mask > 0
        inv_sqrt_mask[nz] = 1.0 / sqrt_mask[nz]

        def apply_L_tilde(x_tilde):
            return self._apply_L_static_q(x_tilde * inv_sqrt_mask) * sqrt_mask

        L_op = scipy.sparse.linalg.LinearOperator((psi_size, psi_size), matvec=apply_L_tilde,
                                                  dtype=np.complex128)
        M_op = None
        if use_preconditioner:
            def apply_M_tilde(x_tilde):
                return self._apply_harmonic_preconditioner(x_tilde, sqrt_mask, inv_sqrt_mask)
            M_op = scipy.sparse.linalg.LinearOperator((psi_size, psi_size), matvec=apply_M_tilde,
                                                      dtype=np.complex128)
        non_acoustic = [nu for nu in range(nb) if self.qlanc.valid_modes_q[nu, iq]]
        if use_mode_symmetry:
            schedule = [(b[0], b) for b in self._find_degenerate_blocks(iq)]
        else:
            schedule = [(nu, [nu]) for nu in non_acoustic]
        if self.verbose:
            print("  Solving at q={} ({} non-acoustic bands, {} solves)".format(
                iq, len(non_acoustic), len(schedule)))
        G_q = np.zeros((nb, nb), dtype=np.complex128)
        total_iters = 0
        L_dense = None
        for band_i, block in schedule:
            rhs = np.zeros(psi_size, dtype=np.complex128)
            rhs[band_i] = 1.0
            rhs_tilde = rhs * sqrt_mask
            x0 = apply_M_tilde(rhs_tilde) if use_preconditioner else None
            n_it = [0]

            def _count(xk):
                n_it[0] += 1

            t1 = time.time()
            x_tilde, info = _gmres(L_op, rhs_tilde, x0, tol, max_iters, M_op, _count)
            if info != 0:
                x_tilde, info = _bicgstab(L_op, rhs_tilde, x_tilde, tol, max_iters, M_op)
                if info != 0:
                    if not dense_fallback:
                        raise RuntimeError(
                            "Iterative solvers (GMRES, BiCGSTAB) did not converge for band {} at "
                            "iq={} (info={}). Set dense_fallback=True to use a dense solve "
                            "(warning: O(psi_size^2) memory).".format(band_i, iq, info))
                    if L_dense is None:
                        L_dense = np.zeros((psi_size, psi_size), dtype=np.complex128)
                        for j in range(psi_size):
                            e_j = np.zeros(psi_size, dtype=np.complex128)
                            e_j[j] = 1.0
                            L_dense[:, j] = apply_L_tilde(e_j)
                        L_dense = (L_dense + L_dense.conj().T) / 2
                    x_tilde = np.linalg.lstsq(L_dense, rhs_tilde, rcond=1e-10)[0]
            total_iters += n_it[0]
            x = x_tilde * inv_sqrt_mask
            if len(block) == 1:
                G_q[:, band_i] = x[:nb]
                for _, other in schedule:
                    if len(other) >= 2:
                        for m in other:
                            G_q[m, band_i] = 0.0
            else:
                d = len(block)
                c_diag = x[band_i]
                for j in range(d):
                    col = block[j]
                    G_q[col, col] = c_diag
                    for _, other in schedule:
                        if other[0] == band_i:
                            continue
                        if len(other) == d:
                            G_q[other[j], col] = x[other[0]]
            if self.verbose:
                print("    Band {}: {} iters, {:.2f}s".format(band_i, n_it[0], time.time() - t1))
        G_q = (G_q + G_q.conj().T) / 2
        H_q = np.zeros((nb, nb), dtype=np.complex128)
        if non_acoustic:
            na = np.array(non_acoustic)
            H_q[np.ix_(na, na)] = np.linalg.inv(G_q[np.ix_(na, na)])
        H_q = (H_q + H_q.conj().T) / 2
        if self.verbose:
            print("  Total L applications: {}".format(total_iters))
        self.H_q_dict[iq] = H_q
        return H_q

    def compute_full_hessian(self, tol=1e-6, max_iters=500, use_preconditioner=True,
                             dense_fallback=False, use_mode_symmetry=True, checkpoint=None):
        """H_q at every (irreducible) q-point (:958-1049); returns the dict of
        mode-basis matrices, or a CC.Phonons object when cellconstructor and
        the crystal structure are available."""
        if self.irr_qpoints is None:
            self._all_qpoints()
        done = set()
        if checkpoint is not None:
            f = checkpoint if checkpoint.lower().endswith(".npz") else checkpoint + ".npz"
            if os.path.exists(f):
                done = self.load_status(checkpoint)
        for iq in self.irr_qpoints:
            if iq in done:
                continue
            self.compute_hessian_at_q(iq, tol=tol, max_iters=max_iters,
                                      use_preconditioner=use_preconditioner,
                                      dense_fallback=dense_fallback,
                                      use_mode_symmetry=use_mode_symmetry)
            if checkpoint is not None:
                self.save_status(checkpoint)
        if getattr(self.qlanc, "dyn", None) is None:
            return self.H_q_dict
        return self._build_phonons()

    def _build_phonons(self):
        import cellconstructor as CC
        import cellconstructor.Phonons
        q_points = np.array(self.qlanc.dyn.q_tot)
        hessian = CC.Phonons.Phonons(self.qlanc.dyn.structure.copy(), nqirr=self.n_q)
        for iq in range(self.n_q):
            pol_m = np.einsum("a, ab -> ab", np.sqrt(self.qlanc.m), self.pols_q[:, :, iq])
            hessian.dynmats[iq] = pol_m @ self.H_q_dict[iq] @ np.conj(pol_m).T
            hessian.q_tot[iq] = q_points[iq]
        hessian.AdjustQStar()
        return hessian

    # ------------------------------------------------------------------- I/O
    def save_status(self, fname):
        if not fname.lower().endswith(".npz"):
            fname += ".npz"
        d = dict(T=np.float64(self.qlanc.T), n_q=np.int64(self.n_q),
                 n_bands=np.int64(self.n_bands), ignore_v3=np.bool_(self.ignore_v3),
                 ignore_v4=np.bool_(self.ignore_v4))
        uci = getattr(self.qlanc, "uci_structure", None)
        if uci is not None:
            d.update(unit_cell=uci.unit_cell, coords=uci.coords, atom_types=uci.get_atomic_types())
        done = sorted(self.H_q_dict.keys())
        d["completed_irr_qpoints"] = np.array(done, dtype=np.int64)
        d["H_q_keys"] = np.array(done, dtype=np.int64)
        d["H_q_values"] = (np.stack([self.H_q_dict[iq] for iq in done]) if done else
                           np.zeros((0, self.n_bands, self.n_bands), dtype=np.complex128))
        np.savez_compressed(fname, **d)

    def load_status(self, fname):
        if not fname.lower().endswith(".npz"):
            fname += ".npz"
        if not os.path.exists(fname):
            raise IOError("Checkpoint file not found: {}".format(fname))
        data = dict(np.load(fname, allow_pickle=True))
        bad = []
        if not np.isclose(float(data["T"]), self.qlanc.T, atol=1e-10):
            bad.append("T: checkpoint={}, current={}".format(float(data["T"]), self.qlanc.T))
        if int(data["n_q"]) != self.n_q:
            bad.append("n_q: checkpoint={}, current={}".format(int(data["n_q"]), self.n_q))
        if int(data["n_bands"]) != self.n_bands:
            bad.append("n_bands: checkpoint={}, current={}".format(int(data["n_bands"]),
                                                                  self.n_bands))
        if bool(data["ignore_v3"]) != self.ignore_v3:
            bad.append("ignore_v3 differs")
        if bool(data["ignore_v4"]) != self.ignore_v4:
            bad.append("ignore_v4 differs")
        if bad:
            raise ValueError("Checkpoint metadata mismatch:\n  " + "\n  ".join(bad))
        for i, iq in enumerate(data["H_q_keys"].astype(int)):
            self.H_q_dict[int(iq)] = data["H_q_values"][i]
        return set(data["completed_irr_qpoints"].astype(int).tolist())


def _gmres(A, b, x0, tol, maxiter, M, cb):
    try:
        return scipy.sparse.linalg.gmres(A, b, x0=x0, rtol=tol, maxiter=maxiter, M=M, callback=cb,
                                         callback_type="legacy")
    except TypeError:       # scipy before the rtol keyword
        return scipy.sparse.linalg.gmres(A, b, x0=x0, tol=tol, maxiter=maxiter, M=M, callback=cb,
                                         callback_type="legacy")


def _bicgstab(A, b, x0, tol, maxiter, M):
    try:
        return scipy.sparse.linalg.bicgstab(A, b, x0=x0, rtol=tol, maxiter=maxiter, M=M)
    except TypeError:
        return scipy.sparse.linalg.bicgstab(A, b, x0=x0, tol=tol, maxiter=maxiter, M=M)
