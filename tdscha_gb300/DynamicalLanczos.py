"""GB300 drop-in for `tdscha.DynamicalLanczos.Lanczos` (Modules/DynamicalLanczos.py).

The public surface keeps the reference's names, argument meanings and error
behaviour: ensemble/perturbation setup, `init`, `prepare_perturbation`,
`prepare_mode`, `prepare_two_ph`, `prepare_ir`, `prepare_raman`,
`prepare_unpolarized_raman`, `apply_full_L`, `run_FT`,
`get_green_function_continued_fraction`, `get_static_frequency`,
`build_lanczos_matrix_from_coeffs`, `get_alpha1_beta1_wigner`,
`get_a1_b1_wigner`, `apply_L1_inverse_FT`, `L_linop` / `M_linop`,
`run_biconjugate_gradient`, `save_status` / `load_status`,
`save_abc` / `load_abc`, and the attributes `a_coeffs`, `b_coeffs`,
`c_coeffs`, `basis_Q`, `basis_P`, `s_norm`, `psi`, `use_wigner`,
`ignore_v3`, `ignore_v4`, `ignore_harmonic`, `reverse_L`, `shift_value`,
`perturbation_modulus`.

Every operator application and Lanczos step runs on the GPU through the
C ABI of libtdscha_gb300.so (no CPU path).  The Krylov basis lives in device
memory (torch tensors) and is copied to the host only when `basis_Q` /
`basis_P` are read or a status is saved.

Extra knobs: `precision` ("fp64" or "mixed": tensor-core perturbation
averages on two-limb fp16 operands with fp32 accumulation; the Lanczos
recurrence stays in float64) and `Lanczos.from_arrays` for ensembles already projected on the
mode basis.
"""
import os
import time

import numpy as np

from . import _native as nat

__EPSILON__ = 1e-12
__RyToK__ = 157887.32400374097
TYPE_DP = np.double

MODE_SLOW_SERIAL = 0
MODE_FAST_SERIAL = 1
MODE_FAST_MPI = 2
MODE_FAST_JULIA = 3
MODE_GB300 = 4


def f_ups(w, T):
    """2 w / (1 + 2 n) (Modules/DynamicalLanczos.py:141-153)."""
    n_w = bose_occupation(w, T)
    return 2 * w / (1 + 2 * n_w)


def bose_occupation(w, T):
    n_w = 0
    if T > 0:
        n_w = 1 / (np.exp(w * __RyToK__ / T) - 1)
    return n_w


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("tdscha_gb300 needs a CUDA GPU (no CPU fallback)")
    return torch


class Lanczos(object):
    def __init__(self, ensemble=None, mode=None, unwrap_symmetries=False, select_modes=None,
                 use_wigner=True, lo_to_split="random", precision="fp64"):
        self.mode = MODE_GB300 if mode is None else mode
        self.verbose = True
        self.T = 0
        self.nat = 0
        self.m = []
        self.w = []
        self.pols = []
        self.n_modes = 0
        self.ignore_harmonic = False
        self.ignore_v3 = False
        self.ignore_v4 = False
        self.N = 0
        self.rho = []
        self.N_eff = 0
        self.X = []
        self.Y = []
        self.psi = []
        self.eigvals = None
        self.eigvects = None
        self.a_coeffs = []
        self.b_coeffs = []
        self.c_coeffs = []
        self.krilov_basis = []
        self.s_norm = []
        self.arnoldi_matrix = []
        self.reverse_L = False
        self.shift_value = 0
        self.symmetrize = False
        self.symmetries = None
        self.degenerate_space = None
        self.N_degeneracy = None
        self.initialized = False
        self.perturbation_modulus = 1
        self.sym_block_id = None
        self.n_syms = 1
        self.sym_julia = None
        self.deg_julia = None
        self.gamma_only = False
        self.use_wigner = use_wigner
        self.ignore_small_w = False
        self.unwrapped = False
        self.precision = precision
        # mixed precision with the ensemble held in 4-byte storage only (the
        # float64 rows are released on the device once the operands are built)
        self.fp32_storage = False
        self.full_reorth = False
        self.trans_projector = None
        self.trans_cart_perms = None
        self.dyn = None             # cellconstructor Phonons of the ensemble, when built from one
        self._ctx = None
        self._ctx_key = None
        self._Qd = None
        self._Pd = None
        self._basis_host = None
        if ensemble is not None:
            self._init_from_ensemble(ensemble, unwrap_symmetries, select_modes, lo_to_split)

    # ------------------------------------------------------------------ setup
    @classmethod
    def from_arrays(cls, X, Y, w, rho, T, pols=None, m=None, use_wigner=True, precision="fp64"):
        """Ensemble already in the mass-scaled mode basis: X, Y (N, M), w (M) in Ry."""
        self = cls(use_wigner=use_wigner, precision=precision)
        self.set_ensemble(X, Y, w, rho, T, pols, m)
        return self

    @classmethod
    def from_cartesian(cls, u_disps, forces, sscha_forces, masses, pols, w, rho, T, f_mean=None,
                       use_wigner=True, precision="fp64"):
        """Ensemble in Cartesian coordinates (Angstrom, Ry/Angstrom) as python-sscha
        stores it: the mode projection of Lanczos.__init__ (:392-452) on the GPU.
        masses per Cartesian coordinate (3 nat), pols (3 nat, n_modes), f_mean the
        symmetrised average force tiled on the supercell (3 nat) or None."""
        from .preprocessing import project_modes
        f = np.asarray(forces, dtype=np.float64) - np.asarray(sscha_forces, dtype=np.float64)
        X, Y = project_modes(u_disps, f, masses, pols, f_mean)
        self = cls(use_wigner=use_wigner, precision=precision)
        self.set_ensemble(X, Y, w, rho, T, pols, masses)
        return self

    def set_translations(self, trans_cart_perms):
        """gamma_only: project the averages on translation-invariant quantities
        (:746-786, :3173-3191) given the supercell's lattice translations as
        Cartesian index permutations (the reference's trans_cart_perms)."""
        perms = [np.asarray(p, dtype=np.intp) for p in trans_cart_perms]
        self.trans_cart_perms = perms
        self.trans_projector = np.mean([self.pols.T @ self.pols[p, :] for p in perms], axis=0)
        self.gamma_only = True
        self._invalidate()

    def set_ensemble(self, X, Y, w, rho, T, pols=None, m=None):
        X = np.ascontiguousarray(X, dtype=TYPE_DP)
        Y = np.ascontiguousarray(Y, dtype=TYPE_DP)
        if X.ndim != 2 or X.shape != Y.shape:
            raise ValueError("X and Y must have the same (N, n_modes) shape")
        self.X, self.Y = X, Y
        self.N, self.n_modes = X.shape
        self.w = np.asarray(w, dtype=TYPE_DP).copy()
        self.rho = np.asarray(rho, dtype=TYPE_DP).copy()
        self.N_eff = np.sum(self.rho)
        self.T = float(T)
        M = self.n_modes
        self.pols = np.eye(M) if pols is None else np.asarray(pols, dtype=TYPE_DP)
        self.m = np.ones(self.pols.shape[0]) if m is None else np.asarray(m, dtype=TYPE_DP)
        self.nat = self.pols.shape[0] // 3
        self.psi = np.zeros(M + M * (M + 1), dtype=TYPE_DP)
        self._invalidate()

    def _init_from_ensemble(self, ensemble, unwrap_symmetries, select_modes, lo_to_split):
        """Project a python-sscha ensemble on the modes (DynamicalLanczos.py:300-452)."""
        import cellconstructor as CC  # noqa: F401  (physics deps of the reference)
        import cellconstructor.Methods
        import sscha.Ensemble as Ensemble
        dyn = ensemble.current_dyn.Copy()
        super_structure = dyn.structure.generate_supercell(dyn.GetSupercell())
        ws, pols = dyn.DiagonalizeSupercell(lo_to_split=lo_to_split)
        nat_sc = super_structure.N_atoms
        m = super_structure.get_masses_array()
        mm = np.tile(m, (3, 1)).T.ravel()
        trans_mask = CC.Methods.get_translations(pols, m)
        good = ~trans_mask
        if select_modes is not None:
            good = good & np.asarray(select_modes, dtype=bool)
        w = ws[good]
        pols = pols[:, good]
        N = ensemble.N
        rho = ensemble.rho.copy()
        u = ensemble.u_disps / Ensemble.Bohr
        f = ensemble.forces.reshape(N, 3 * nat_sc).copy()
        f -= ensemble.sscha_forces.reshape(N, 3 * nat_sc)
        f_mean = ensemble.get_average_forces(get_error=False)
        qe_sym = CC.symmetries.QE_Symmetry(dyn.structure)
        qe_sym.SetupQPoint()
        qe_sym.SymmetrizeVector(f_mean)
        f_mean = np.tile(f_mean, (np.prod(ensemble.current_dyn.GetSupercell()), 1)).ravel()
        f_mean *= Ensemble.Bohr
        f *= Ensemble.Bohr
        if unwrap_symmetries:
            u, f, rho = ensemble.get_unwrapped_ensemble()
            N = len(rho)
            self.unwrapped = True
            u /= Ensemble.Bohr
            f *= Ensemble.Bohr
        f[:, :] -= np.tile(f_mean, (N, 1))
        from .preprocessing import project_modes
        X, Y = project_modes(u, f, mm, pols, u_scale=1.0, f_scale=1.0)
        self.dyn = dyn
        self.set_ensemble(X, Y, w, rho, ensemble.current_T, pols, mm)
        self.nat = nat_sc

    def _invalidate(self):
        if self._ctx is not None:
            self._ctx.close()
        self._ctx = None
        self._ctx_key = None

    def reset(self):
        """Reset the Lanczos state keeping ensemble and options (:527-557)."""
        M = self.n_modes
        self.psi = np.zeros(M + M * (M + 1), dtype=TYPE_DP)
        self.eigvals = None
        self.eigvects = None
        self.a_coeffs = []
        self.b_coeffs = []
        self.c_coeffs = []
        self.basis_P = []
        self.basis_Q = []
        self.s_norm = []
        self.krilov_basis = []
        self.arnoldi_matrix = []

    def init(self, use_symmetries=True, symmetries=None):
        """Allocate psi and prepare the symmetry tables (:564-582)."""
        M = self.n_modes
        self.psi = np.zeros(M + M * (M + 1), dtype=TYPE_DP)
        self.prepare_symmetrization(no_sym=not use_symmetries, symmetries=symmetries)
        self.initialized = True

    def prepare_symmetrization(self, no_sym=False, verbose=True, symmetries=None):
        """Mode-space symmetry blocks (:694-871).

        `symmetries` may be a (symmetries, degenerate_space) pair of per-block
        lists already in the mode basis (what CC.symmetries.GetSymmetriesOnModesDeg
        returns).  Without it, and without no_sym, the reference asks spglib
        for the supercell symmetries; that needs cellconstructor and spglib.
        """
        self.initialized = True
        M = self.n_modes
        if no_sym or self.unwrapped:
            # one-mode blocks with the identity as their only image: the tables
            # set_symmetries would build, without a Python step per mode
            ident = np.ones((1, 1, 1), dtype=np.double)
            self.symmetries = [ident] * M
            self.degenerate_space = list(np.arange(M, dtype=np.intc).reshape(M, 1))
            self.N_degeneracy = np.ones(M, dtype=np.intc)
            self.sym_block_id = np.arange(M, dtype=np.intc)
            self.n_syms = 1
            self.initialized = True
            self._invalidate()
            return
        if symmetries is None:
            import spglib
            import cellconstructor as CC
            import cellconstructor.symmetries
            super_structure = self.dyn.structure.generate_supercell(self.dyn.GetSupercell())
            super_symmetries = CC.symmetries.GetSymmetriesFromSPGLIB(
                spglib.get_symmetry(super_structure.get_spglib_cell()), False)
            pol_syms, basis = CC.symmetries.GetSymmetriesOnModesDeg(super_symmetries,
                                                                    super_structure, self.pols,
                                                                    self.w)
            self.set_symmetries(pol_syms, basis)
            return
        syms, basis = symmetries
        self.set_symmetries(syms, basis)

    def set_symmetries(self, symmetries, degenerate_space, sym_block_id=None):
        M = self.n_modes
        self.symmetries = [np.ascontiguousarray(s, dtype=np.double) for s in symmetries]
        self.degenerate_space = [np.array(x, dtype=np.intc) for x in degenerate_space]
        self.N_degeneracy = np.array([len(x) for x in self.degenerate_space], dtype=np.intc)
        if sym_block_id is None:
            sym_block_id = -np.ones(M, dtype=np.intc)
            for j, block in enumerate(self.degenerate_space):
                sym_block_id[block] = j
            if np.any(sym_block_id < 0):
                raise ValueError("Error, something went wrong during the symmetrization")
        self.sym_block_id = np.asarray(sym_block_id, dtype=np.intc)
        self.n_syms = self.symmetries[0].shape[0]
        self.initialized = True
        self._invalidate()

    # -------------------------------------------------------- perturbations
    def prepare_perturbation(self, vector, masses_exp=1, add=False):
        """psi[:M] (+)= sum_a v_a e_mu^a sqrt(m_a)^masses_exp (:2023-2075)."""
        if not add:
            self.reset()
            self.psi = np.zeros(self.psi.shape, dtype=TYPE_DP)
        m_on = np.sqrt(self.m) ** masses_exp
        new_v = np.einsum("a, a, ab->b", m_on, vector, self.pols)
        self.psi[: self.n_modes] += new_v
        self.perturbation_modulus = new_v.dot(new_v)

    def prepare_mode(self, index):
        """Unit perturbation on one mode (:2077-2091)."""
        self.reset()
        self.psi[:] = 0
        self.psi[index] = 1
        self.perturbation_modulus = 1

    def prepare_two_ph(self, a, b):
        """Two-phonon perturbation, Wigner only (:2095-2145)."""
        if not self.use_wigner:
            raise NotImplementedError("The two phonon response is available only in Wigner")
        if a > self.n_modes or b > self.n_modes:
            raise ValueError("The a-b indices must be smaller than {}".format(self.n_modes))
        self.reset()
        self.psi[:] = 0
        chi_plus = self.get_chi_plus()
        chi_minus = self.get_chi_minus()
        mat = np.zeros((self.n_modes, self.n_modes))
        mat[a, b] = 0.5
        mat[b, a] += 0.5
        pert_a = -np.sqrt(-0.5 * chi_minus) * mat
        pert_b = +np.sqrt(+0.5 * chi_plus) * mat
        iu = np.triu_indices(self.n_modes)
        h = len(iu[0])
        M = self.n_modes
        self.psi[M:M + h] = pert_a[iu]
        self.psi[M + h:] = pert_b[iu]
        self.perturbation_modulus = self.psi.dot(self.psi * self.mask_dot_wigner())

    # ------------------------------------------ IR / Raman perturbations
    def _supercell_size(self, n_uc_coords, n_supercell):
        if self.dyn is not None:
            return int(np.prod(self.dyn.GetSupercell()))
        if n_supercell is not None:
            return int(n_supercell)
        n_coords = np.shape(self.pols)[0]
        if n_uc_coords <= 0 or n_coords % n_uc_coords:
            raise ValueError("cannot infer the supercell: %d Cartesian coordinates, %d per unit cell"
                             % (n_coords, n_uc_coords))
        return n_coords // n_uc_coords

    def prepare_ir(self, effective_charges=None, pol_vec=np.array([1, 0, 0]), n_supercell=None):
        """IR perturbation (:1705-1751): the effective charges (n_atoms_uc, 3, 3; atom,
        field component, coordinate) contracted with the light polarisation, tiled over
        the supercell, as a Cartesian vector with masses_exp = -1.  Without a dynamical
        matrix (self.dyn) the charges must be given; the supercell size is then
        n_supercell or (Cartesian coordinates of pols) / (3 n_atoms_uc)."""
        ec = effective_charges
        if ec is None and self.dyn is not None:
            ec = self.dyn.effective_charges
        if ec is None:
            raise AssertionError("Error, no effective charge found. Cannot initialize IR responce")
        ec = np.asarray(ec, dtype=np.double)
        if ec.ndim != 3:
            raise AssertionError("Error, effective charges of the wrong shape: {}".format(ec.shape))
        n_sc = self._supercell_size(3 * ec.shape[0], n_supercell)
        msg = ("Error, effective charges of the wrong shape: {}\nNumber of modes : {}\n"
               "Dimension of the supercell : {}".format(ec.shape, self.n_modes, n_sc))
        if not self.ignore_small_w and ec.shape[0] * ec.shape[2] * n_sc != self.n_modes + 3:
            raise AssertionError(msg)
        if not ec.shape[1] == ec.shape[2] == 3:
            raise AssertionError(msg)
        z_eff = np.einsum("abc, b", ec, pol_vec)
        self.prepare_perturbation(np.tile(z_eff.ravel(), n_sc), masses_exp=-1)

    def _raman_vector_fn(self, raman_tensor):
        """Raman vector for two polarisations: the dynamical matrix's GetRamanVector, or
        sum_ab p_in[a] p_out[b] R[a, b, :] of a given tensor R (3, 3, 3 n_atoms_uc) that
        already obeys the acoustic sum rule."""
        if raman_tensor is not None:
            R = np.asarray(raman_tensor, dtype=np.double)
            if R.ndim != 3 or R.shape[:2] != (3, 3):
                raise ValueError("raman_tensor must have shape (3, 3, 3 n_atoms), got %s"
                                 % (R.shape,))
            return (lambda p_in, p_out: np.einsum("abc,a,b->c", R, np.asarray(p_in, np.double),
                                                  np.asarray(p_out, np.double))), R.shape[2]
        if self.dyn is None or getattr(self.dyn, "raman_tensor", None) is None:
            raise AssertionError("Error, no Raman tensor found. Cannot initialize the Raman responce")
        return self.dyn.GetRamanVector, np.shape(self.dyn.raman_tensor)[-1]

    # unpolarised components: (pol_in, pol_out) pairs with their factors, for
    # alpha^2 = (xx+yy+zz)^2/9, beta_1..3 = (xx-yy)^2/2, (xx-zz)^2/2, (yy-zz)^2/2,
    # beta_4..6 = 3 xy^2, 3 yz^2, 3 xz^2 (:1115-1175)
    _THIRD = staticmethod(lambda v: v / 3)
    _HALF = staticmethod(lambda v: v / np.sqrt(2))
    _MHALF = staticmethod(lambda v: -v / np.sqrt(2))
    _SQRT3 = staticmethod(lambda v: v * np.sqrt(3))
    _UNPOL = {0: ((0, 0, _THIRD), (1, 1, _THIRD), (2, 2, _THIRD)),
              1: ((0, 0, _HALF), (1, 1, _MHALF)),
              2: ((0, 0, _HALF), (2, 2, _MHALF)),
              3: ((1, 1, _HALF), (2, 2, _MHALF)),
              4: ((0, 1, _SQRT3),),
              5: ((1, 2, _SQRT3),),
              6: ((0, 2, _SQRT3),)}

    def prepare_raman(self, pol_vec_in=np.array([1, 0, 0]), pol_vec_out=np.array([1, 0, 0]),
                      mixed=False, pol_in_2=None, pol_out_2=None, unpolarized=None,
                      raman_tensor=None, n_supercell=None, sum_components=False):
        """Raman perturbation (:1061-1182) from the Raman vector of the two polarisations
        (or of one unpolarised component, 0..6), tiled over the supercell, masses_exp = -1.

        The reference ends with a plain prepare_perturbation of the last vector it built,
        so `mixed` has no effect and the unpolarised components 0-3 keep only their last
        term; that result is reproduced by default.  sum_components=True keeps every term
        (the mixed polarisation pair added, the unpolarised terms summed)."""
        vec_fn, n_uc_coords = self._raman_vector_fn(raman_tensor)
        n_sc = self._supercell_size(n_uc_coords, n_supercell)
        e = np.eye(3)
        if unpolarized is None:
            terms = [(pol_vec_in, pol_vec_out, None)]
            if mixed and sum_components:
                terms.append((pol_in_2, pol_out_2, None))
        elif unpolarized in self._UNPOL:
            terms = [(e[i], e[j], f) for i, j, f in self._UNPOL[unpolarized]]
        else:
            raise ValueError("Error, unpolarized must be between [0, ... ,6] got invalid {}."
                             .format(unpolarized))
        vecs = []
        for p_in, p_out, scale in terms:
            v = np.tile(np.asarray(vec_fn(p_in, p_out)).ravel(), n_sc)
            vecs.append(v if scale is None else scale(v))
        if not sum_components:
            self.prepare_perturbation(vecs[-1], masses_exp=-1)
            return
        self.prepare_perturbation(vecs[0], masses_exp=-1)
        for v in vecs[1:]:
            self.prepare_perturbation(v, masses_exp=-1, add=True)
        self.perturbation_modulus = self.psi[:self.n_modes].dot(self.psi[:self.n_modes])

    def get_prefactors_unpolarized_raman(self, index):
        """Weight of unpolarised component `index` in 45/9 (xx+yy+zz)^2 +
        7/2 [(xx-yy)^2 + (xx-zz)^2 + (yy-zz)^2] + 21 [xy^2 + xz^2 + yz^2] (:1184-1208)."""
        labels = list(range(7))
        if index not in labels:
            raise ValueError('{} should be in {}'.format(index, labels))
        return (45 / 9, 7 / 2, 7 / 2, 7 / 2, 7 * 3, 7 * 3, 7 * 3)[index]

    # components of prepare_unpolarized_raman: xx+yy+zz, xx-yy, xx-zz, yy-zz, xy, xz, yz
    _UNPOL_SUM = {0: ((0, 0, 1), (1, 1, 1), (2, 2, 1)), 1: ((0, 0, 1), (1, 1, -1)),
                  2: ((0, 0, 1), (2, 2, -1)), 3: ((1, 1, 1), (2, 2, -1)),
                  4: ((0, 1, 1),), 5: ((0, 2, 1),), 6: ((1, 2, 1),)}

    def prepare_unpolarized_raman(self, index=0, debug=False, raman_tensor=None,
                                  n_supercell=None):
        """Perturbation of unpolarised Raman component `index` (:1210-1278): the summed
        (or differenced) Raman vectors of the component, tiled over the supercell,
        masses_exp = -1.  debug saves the unit-cell vector as raman_v_<index>.npy."""
        vec_fn, n_uc_coords = self._raman_vector_fn(raman_tensor)
        labels = list(range(7))
        if index not in labels:
            raise ValueError('{} should be in {}'.format(index, labels))
        e = np.eye(3)
        raman_v = None
        for i, j, sgn in self._UNPOL_SUM[index]:
            v = np.asarray(vec_fn(e[i], e[j]), dtype=np.double)
            raman_v = v.copy() if raman_v is None else (raman_v + v if sgn > 0 else raman_v - v)
        if debug:
            np.save('raman_v_{}'.format(index), raman_v)
        n_sc = self._supercell_size(n_uc_coords, n_supercell)
        self.prepare_perturbation(np.tile(raman_v.ravel(), n_sc), masses_exp=-1)

    def set_max_frequency(self, freq):
        """Reverse-and-shift setup (:2227-2253)."""
        self.shift_value = 4 * freq * freq
        self.reverse_L = True

    # ------------------------------------------------------ host helpers
    def _bose_matrix(self):
        M = self.n_modes
        w = np.tile(self.w, (M, 1))
        n = np.zeros((M, M), dtype=np.double)
        if self.T > __EPSILON__:
            n = 1.0 / (np.exp(w * 157887.32400374097 / self.T) - 1.0)
        return w, n

    def get_chi_minus(self):
        w, n = self._bose_matrix()
        return (w - w.T) * (n - n.T) / (2. * w * w.T)

    def get_chi_plus(self):
        w, n = self._bose_matrix()
        return (w + w.T) * (1 + n + n.T) / (2. * w * w.T)

    def mask_dot_wigner(self, debug=False):
        M = self.n_modes
        mask = np.ones(M + M * (M + 1))
        r, c = np.triu_indices(M)
        h = len(r)
        mask[M:M + h][r < c] = 2
        mask[M + h:][r < c] = 2
        return mask

    def _sym_from_sector(self, start, half_off_diagonal):
        M = self.n_modes
        h = M * (M + 1) // 2
        A = np.zeros((M, M))
        iu = np.triu_indices(M)
        A[iu] = self.psi[start:start + h]
        A.T[iu] = self.psi[start:start + h]
        if half_off_diagonal:
            nm = np.ones((M, M)) / 2
            np.fill_diagonal(nm, 1)
            A *= nm
        return A

    def get_Y1(self, half_off_diagonal=False):
        return self._sym_from_sector(self.n_modes, half_off_diagonal)

    def get_ReA1(self, half_off_diagonal=False):
        return self._sym_from_sector(self.n_modes + self.n_modes * (self.n_modes + 1) // 2,
                                     half_off_diagonal)

    def _wigner_pair_factors(self):
        """Per mode pair (i <= j, row-major like the psi sectors): X = (1+2n_i)(1+2n_j)/8,
        w_i w_j, chi^- and chi^+ (:2816-2836, :2732-2752)."""
        iu = np.triu_indices(self.n_modes)
        w_i, w_j = self.w[iu[0]], self.w[iu[1]]
        n_i = n_j = 0
        if self.T > 0:
            kT = np.double(self.T / __RyToK__)
            n_i = 1 / (np.exp(w_i / kT) - 1)
            n_j = 1 / (np.exp(w_j / kT) - 1)
        X = (1 + 2 * n_i) * (1 + 2 * n_j) / 8
        ww = w_i * w_j
        chi_m = (w_j - w_i) * (n_j - n_i) / (2 * ww)
        chi_p = (w_j + w_i) * (1 + n_j + n_i) / (2 * ww)
        return iu, X, ww, chi_m, chi_p

    def get_alpha1_beta1_wigner(self, get_alpha=True):
        """Upsilon^(1) = alpha^(1) (get_alpha) or beta^(1) as (n_modes, n_modes) matrices
        from the Wigner sectors a'^(1), b'^(1) of psi (:2773-2882):
        alpha = w_i w_j / X (sqrt(-chi^-/2) a' - sqrt(chi^+/2) b'),
        beta = (sqrt(-chi^-/2) a' + sqrt(chi^+/2) b') / X."""
        M = self.n_modes
        h = M * (M + 1) // 2
        iu, X, ww, chi_m, chi_p = self._wigner_pair_factors()
        a_sec = np.asarray(self.psi[M:M + h])
        b_sec = np.asarray(self.psi[M + h:])
        if get_alpha:
            packed = (ww / X) * np.sqrt(-0.5 * chi_m) * a_sec - (ww / X) * np.sqrt(0.5 * chi_p) * b_sec
        else:
            packed = (np.sqrt(-0.5 * chi_m) / X) * a_sec + (np.sqrt(0.5 * chi_p) / X) * b_sec
        out = np.zeros((M, M), dtype=np.double)
        out[iu] = packed
        out.T[iu] = packed
        return out

    def get_a1_b1_wigner(self, get_a1=True):
        """The inverse change of variables (:2690-2771): sqrt(-chi^-/2) a' (get_a1) or b'
        as upper-triangle vectors of length n_modes (n_modes + 1) / 2, from the
        alpha^(1) and beta^(1) of get_alpha1_beta1_wigner."""
        iu, X, ww, chi_m, chi_p = self._wigner_pair_factors()
        alpha1 = self.get_alpha1_beta1_wigner(get_alpha=True)[iu]
        beta1 = self.get_alpha1_beta1_wigner(get_alpha=False)[iu]
        if get_a1:
            return 0.5 * X * (alpha1 / ww + beta1)
        return -0.5 * X * (alpha1 / ww - beta1) / np.sqrt(0.5 * chi_p)

    # ------------------------------------------------------------ device side
    def _context(self):
        if not self.initialized:
            raise ValueError("Error, this class must be initialized before lunching the "
                             "computation:\n Use the .init()")
        want_mixed = self.precision == "mixed"
        only32 = want_mixed and bool(self.fp32_storage)
        key = (id(self.X), id(self.Y), id(self.rho), self.T, id(self.symmetries),
               bool(self.gamma_only), id(self.trans_cart_perms))
        if self._ctx is not None and (self._ctx_key != key or
                                      (want_mixed and not self._ctx.with_mixed) or
                                      (not want_mixed and not self._ctx.fp64_storage) or
                                      (only32 and self._ctx.fp64_storage)):
            self._invalidate()
        if self._ctx is None:
            _torch()
            self._ctx = nat.Context(self.X, self.Y, self.w, self.rho, self.T, self.symmetries,
                                    self.degenerate_space, self.sym_block_id,
                                    with_mixed="fp32" if only32 else want_mixed)
            self._ctx_key = key
            if self.gamma_only and self.trans_cart_perms is not None:
                perms = np.ascontiguousarray(np.array(self.trans_cart_perms), dtype=np.intc)
                pols = nat.f64(self.pols)
                nat.check(nat.load().tdscha_ctx_set_translations(
                    self._ctx.handle, pols.shape[0], nat.dp(pols), perms.shape[0], nat.ip(perms)))
        self._ctx.set_options(self.use_wigner, self.ignore_harmonic, self.ignore_v3,
                              self.ignore_v4, self.reverse_L, self.shift_value)
        return self._ctx

    def _prec(self):
        if self.precision == "fp64":
            return nat.PREC_FP64
        if self.precision == "mixed":
            return nat.PREC_MIXED
        raise ValueError("precision must be 'fp64' or 'mixed', got %r" % (self.precision,))

    def _apply_dev(self, psi, transpose, ignore_harmonic=None, ignore_v3=None, plain=False):
        torch = _torch()
        ctx = self._context()
        if ignore_harmonic is not None or ignore_v3 is not None or plain:
            ctx.set_options(self.use_wigner,
                            self.ignore_harmonic if ignore_harmonic is None else ignore_harmonic,
                            self.ignore_v3 if ignore_v3 is None else ignore_v3, self.ignore_v4,
                            False if plain else self.reverse_L, 0 if plain else self.shift_value)
        x = torch.as_tensor(np.ascontiguousarray(psi, dtype=np.float64)).cuda()
        y = torch.empty_like(x)
        st = torch.cuda.current_stream().cuda_stream
        nat.check(nat.load().tdscha_apply_full_L(ctx.handle, x.data_ptr(), y.data_ptr(),
                                                 1 if transpose else 0, self._prec(), st))
        out = y.cpu().numpy()
        return out

    # ------------------------------------------- harmonic inverse and solvers
    def _free_pair_propagator(self):
        """Per mode pair (upper triangle rows, w_a the column mode, w_b the row mode):
        the 2 x 2 block (X, Y; X1, Y1) of the non-interacting two-phonon propagator
        and the occupations used for it (:2478-2513).  Occupations are zeroed
        where 0.01 w_a > k_B T, for both modes of the pair, as the reference does."""
        iu = np.triu_indices(self.n_modes)
        w_a, w_b = self.w[iu[1]], self.w[iu[0]]
        n_a = np.zeros(np.shape(w_a), dtype=TYPE_DP)
        n_b = np.zeros(np.shape(w_a), dtype=TYPE_DP)
        cold = 0.01 * w_a * __RyToK__ > self.T
        if self.T > 0:
            kT = np.double(self.T / __RyToK__)
            n_a = 1 / (np.exp(w_a / kT) - 1)
            n_b = 1 / (np.exp(w_b / kT) - 1)
            n_a[cold] = 0
            n_b[cold] = 0
        occ = (2 * n_a + 1) * (2 * n_b + 1)
        cross = 2 * w_a * w_b
        s = 2 * n_a * n_b + n_a + n_b
        X = -w_a ** 2 - w_b ** 2 - cross / occ
        Y = -(8 * w_a * w_b) / occ
        X1 = -s * (s + 1) * cross / occ
        Y1 = -w_a ** 2 - w_b ** 2 + cross / occ
        return w_a, w_b, n_a, X, Y, X1, Y1

    def apply_L1_inverse_FT(self, psi, transpose=False):
        """Inverse of the harmonic operator (:2451-2560), the preconditioner of
        run_biconjugate_gradient: 1/w^2 on the R sector and the inverse of each
        pair's 2 x 2 block on the (Y, ReA) sectors.  A block with determinant below
        1e-12 keeps only -1/X on its Y entry; at T > 0 a diagonal pair of populated
        modes also inverts its ReA entry alone."""
        out = np.zeros(np.shape(self.psi), dtype=TYPE_DP)
        if self.ignore_harmonic:
            return out
        M = self.n_modes
        psi = np.asarray(psi)
        out[:M] = (psi[:M] / self.w) / self.w
        w_a, w_b, n_a, X, Y, X1, Y1 = self._free_pair_propagator()
        h = len(w_a)
        if len(psi) != M + 2 * h:
            raise AssertionError("\nERROR,\nThe initial vector for the Lanczos algorithm has a "
                                 "wrong dimension. \nThis may be caused by the Lanczos "
                                 "initialized at the wrong temperature.\n")
        det = X * Y1 - X1 * Y
        singular = det < __EPSILON__
        det[singular] = np.inf
        iX, iY, iX1, iY1 = -Y1 / det, Y / det, X1 / det, -X / det
        iX[singular] = -1 / X[singular]
        if self.T > __EPSILON__:
            lone = (w_a == w_b) & (n_a > __EPSILON__)
            iY1[lone] = -1 / Y1[lone]
        pY, pA = psi[M:M + h], psi[M + h:]
        oY, oA = out[M:M + h], out[M + h:]
        oY[:] = iX * pY
        if transpose:
            oA += iY * pY
            oY += iX1 * pA
        else:
            oY += iY * pA
            oA += iX1 * pY
        oA += iY1 * pA
        return out

    @property
    def L_linop(self):
        """scipy LinearOperator of the full L on the GPU; like the reference's
        (:478-483), matvec is apply_full_L (which overwrites self.psi) and rmatvec
        its transpose."""
        import scipy.sparse.linalg
        n = len(self.psi)
        return scipy.sparse.linalg.LinearOperator(
            shape=(n, n), matvec=self.apply_full_L,
            rmatvec=lambda v: self.apply_full_L(v, transpose=True), dtype=TYPE_DP)

    @property
    def M_linop(self):
        """scipy LinearOperator of apply_L1_inverse_FT (:485-489)."""
        import scipy.sparse.linalg
        n = len(self.psi)
        return scipy.sparse.linalg.LinearOperator(
            shape=(n, n), matvec=self.apply_L1_inverse_FT,
            rmatvec=lambda v: self.apply_L1_inverse_FT(v, transpose=True), dtype=TYPE_DP)

    def run_biconjugate_gradient(self, verbose=True, tol=5e-4, maxiter=1000, save_g=None,
                                 save_each=1, use_preconditioning=True, algorithm="bicgstab"):
        """Static response by solving L x_i = e_i for every mode (:3842-4052) with
        scipy's bicgstab / bicg (tol as their relative tolerance) or a BFGS
        minimisation of (Lx - b) H^-1 (Lx - b) / 2 ('cg-minimize'), every
        application of L on the GPU.  Returns the inverse of the symmetrised
        one-phonon block of G (the mass-rescaled free-energy Hessian)."""
        import inspect
        import scipy.optimize
        import scipy.sparse.linalg as sla
        algo = algorithm.lower()
        if algo not in ("bicgstab", "bicg", "cg-minimize"):
            raise ValueError("\nError, algorithm type '{}' in subroutine run_biconjugate_gradient "
                             "not implemented.\n       the only supported algorithms are "
                             "['bicgstab', 'bicg']\n".format(algorithm))
        if not self.initialized:
            self.prepare_symmetrization()
        M = self.n_modes
        G = np.zeros((M, M), dtype=np.double)
        L, Minv = self.L_linop, self.M_linop
        for i in range(M):
            self.psi = np.zeros(self.psi.shape, dtype=TYPE_DP)
            self.psi[i] = 1
            b = self.psi
            x0 = Minv.matvec(b)
            last = [b.copy(), 0]

            def callback(xk):
                if np.isnan(np.sum(xk)):
                    raise ValueError("Error, NaN value found during the Biconjugate Gradient.")
                if verbose:
                    print("BCG STEP {} | solution changed by {} (tol = {})".format(
                        last[1], np.sum((xk - last[0]) ** 2), tol))
                last[0], last[1] = xk.copy(), last[1] + 1

            t1 = time.time()
            if algo == "cg-minimize":
                def func(x, rhs):
                    r = L.matvec(x) - rhs
                    h_r = Minv.matvec(Minv.rmatvec(r)) if use_preconditioning else r
                    return 0.5 * np.sum(r * h_r), L.rmatvec(h_r)
                res = scipy.optimize.minimize(func, x0, args=(b.copy(),), method="bfgs", jac=True,
                                              options={"gtol": tol, "maxiter": maxiter,
                                                       "disp": verbose, "norm": 2})
                info, x = (0 if res.success else 1), res.x.copy()
            else:
                solver = sla.bicgstab if algo == "bicgstab" else sla.bicg
                key = "rtol" if "rtol" in inspect.signature(solver).parameters else "tol"
                x, info = solver(L, b, x0=x0, maxiter=maxiter, callback=callback,
                                 M=Minv if use_preconditioning else None, **{key: tol})
            if info < 0:
                raise AssertionError("Error on input or breakdown of biconjugate gradient "
                                     "algorithm (info = {})".format(info))
            if verbose:
                print("Time to solve the linear system: {} s".format(time.time() - t1))
                if info > 0:
                    print("The biconjugate gradient (step {}) algorithm did not converge after {} "
                          "iterations.".format(i + 1, maxiter))
            G[i, :] = x[:M]
            if save_g is not None and i % save_each == 0:
                np.save(save_g, G)
        if save_g is not None:
            np.save(save_g, G)
        if np.max(np.abs(G - G.T)) >= 1e-4:
            raise AssertionError("Error, the resulting one-phonon Green function is not Hermitian.")
        return np.linalg.inv(0.5 * (G + G.T))

    def apply_L1_FT(self, transpose=False):
        """Harmonic part only, on self.psi (:2287-2445)."""
        return self._apply_dev(self.psi, transpose, ignore_v3=True, plain=True)

    def apply_anharmonic_FT(self, transpose=False, test_weights=False, use_old_version=False):
        """Anharmonic part only, on self.psi (:2951-3363)."""
        return self._apply_dev(self.psi, transpose, ignore_harmonic=True, ignore_v3=False,
                               plain=True)

    def apply_full_L(self, target=None, force_t_0=False, force_FT=True, transpose=False,
                     fast_lanczos=True):
        """psi <- L psi on the GPU (:3549-3651); overwrites and returns self.psi."""
        if force_t_0 and force_FT:
            raise ValueError("Error, only one between force_t_0 and force_FT can be True")
        if target is not None:
            self.psi = target
        out = self._apply_dev(self.psi, transpose)
        self.psi = out
        return self.psi

    # ------------------------------------------------------- static response
    def _static_size(self):
        return self.n_modes + (self.n_modes * (self.n_modes + 1)) // 2

    def _static_dev(self, X, what, power=1.0):
        """Batched static operator on a (k, M + M(M+1)/2) float64 device tensor."""
        torch = _torch()
        ctx = self._context()
        X = X.contiguous()
        Y = torch.empty_like(X)
        st = torch.cuda.current_stream().cuda_stream
        nat.check(nat.load().tdscha_static_L(ctx.handle, X.shape[0], X.data_ptr(), Y.data_ptr(),
                                             what, float(power), self._prec(), st))
        return Y

    def _static_host(self, psi, what, power=1.0):
        torch = _torch()
        expected_dim = self._static_size()
        psi = np.asarray(psi, dtype=np.float64)
        if psi.ndim != 1 or len(psi) != expected_dim:
            raise AssertionError("\nError, for the static calculation the vector must be of "
                                 "dimension {}, got {}\n".format(expected_dim, len(psi)))
        X = torch.from_numpy(np.ascontiguousarray(psi)).cuda()[None, :]
        Y = self._static_dev(X, what, power)
        nat.check(nat.load().tdscha_ctx_sync(self._ctx.handle,
                                             torch.cuda.current_stream().cuda_stream))
        return Y[0].cpu().numpy()

    def _static_unit_rows(self, i0, k, what):
        """The static operator (what: 1 harmonic, 2 anharmonic, 3 both) on the unit
        vectors e_i0 .. e_{i0+k-1}, one batched GPU call; rows of a (k, n) array."""
        torch = _torch()
        n = self._static_size()
        dev = torch.device("cuda")
        E = torch.zeros((k, n), dtype=torch.float64, device=dev)
        E[torch.arange(k, device=dev), torch.arange(i0, i0 + k, device=dev)] = 1.0
        Y = self._static_dev(E, what)
        nat.check(nat.load().tdscha_ctx_sync(self._ctx.handle,
                                             torch.cuda.current_stream().cuda_stream))
        return Y.cpu().numpy()

    def apply_L1_static(self, psi, inverse=False, power=1):
        """Harmonic part of the static operator (:2562-2624): psi_R w^(2p) and
        psi_W / Lambda^p, p = -power when inverse."""
        if inverse:
            power = -power
        return self._static_host(psi, 1, power)

    def apply_anharmonic_static(self):
        """Anharmonic part of the static operator on self.psi (:3369-3430):
        R1 = psi_R, Y1 = -2 Upsilon psi_W Upsilon, output [-f | d2v upper rows]."""
        return self._static_host(self.psi, 2)

    def run_hessian_calculation(self, verbose=True, eigen_shift=1, tol=5e-4, max_iters=1000,
                                save_g=None, save_each=1, use_preconditioning=True,
                                algorithm="cg"):
        """Free-energy Hessian from the static response (:4054-4330).

        One minimal-residual solve per mode as in the reference (threshold 1e-6
        of Tools.minimum_residual_algorithm; `tol` is unused there too), all
        n_modes solves advanced together on the GPU (each system keeps its own
        scalars and stops at its own convergence).  Returns the mass-rescaled
        Hessian inv((G + G^T)/2)."""
        from . import Tools
        torch = _torch()
        if not self.initialized:
            self.prepare_symmetrization()
        M = self.n_modes
        Ps = self._static_size()
        self.psi = np.zeros(Ps, dtype=TYPE_DP)
        dev = torch.device("cuda")
        if algorithm.lower() != "cg":
            if algorithm.lower() not in ("minimize", "minimize-quad"):
                raise ValueError("\nError, algorithm type '{}' in subroutine run_biconjugate_gradient "
                                 "not implemented.\n       the only supported algorithms are "
                                 "['bicgstab', 'bicg']\n".format(algorithm))
            return self._run_hessian_minimize(eigen_shift, tol, max_iters, save_g, algorithm,
                                              verbose)

        def L(X):
            Xs = X.clone()
            Xs[:, M:] *= eigen_shift
            Y = self._static_dev(Xs, 3)
            Y[:, M:] *= eigen_shift
            return Y

        def Ph(X):
            return self._static_dev(X, 1, -0.5)

        B = torch.zeros((M, Ps), dtype=torch.float64, device=dev)
        B[torch.arange(M), torch.arange(M)] = 1.0
        t1 = time.time()
        if use_preconditioning:
            Bt = Ph(B)
            Xt, iters, conv = Tools.batched_minimum_residual(lambda Z: Ph(L(Ph(Z))), Bt,
                                                             Bt.clone(), max_iters, 1e-6,
                                                             verbose=verbose)
            res = Ph(Xt)
        else:
            res, iters, conv = Tools.batched_minimum_residual(L, B, B.clone(), max_iters, 1e-6,
                                                              verbose=verbose)
        nat.check(nat.load().tdscha_ctx_sync(self._ctx.handle,
                                             torch.cuda.current_stream().cuda_stream))
        G_one_phonon = res[:, :M].cpu().numpy()
        if verbose:
            print("Static response: %d systems, %d-%d iterations, %.3f s"
                  % (M, iters.min(), iters.max(), time.time() - t1))
        for i in np.where(~conv)[0]:
            print("WARNING: cg did not converge after {} iterations.".format(max_iters))
        if save_g is not None:
            np.save(save_g, G_one_phonon)
        disp = np.max(np.abs(G_one_phonon - G_one_phonon.T))
        assert disp < 1e-4, "Error, the resulting one-phonon Green function is not Hermitian."
        G = 0.5 * (G_one_phonon + G_one_phonon.T)
        return np.linalg.inv(G)

    def _run_hessian_minimize(self, eigen_shift, tol, max_iters, save_g, algorithm, verbose):
        """The scipy BFGS variants of run_hessian_calculation (:4191-4265), with
        the static operator on the GPU."""
        import scipy.optimize
        M = self.n_modes
        Ps = self._static_size()

        def L(x):
            p = np.array(x, dtype=np.float64)
            p[M:] *= eigen_shift
            ret = self._static_host(p, 3)
            ret[M:] *= eigen_shift
            return ret

        def func_quad(x, b):
            r = L(x) - b
            return 0.5 * np.sum(r ** 2), L(r)

        def func_standard(x, b):
            Lx = L(x)
            return 0.5 * x.dot(Lx) - b.dot(x), Lx - b

        G = np.zeros((M, M))
        options = {"gtol": tol, "maxiter": max_iters, "disp": verbose, "norm": 2}
        fun = func_quad if algorithm.lower() == "minimize-quad" else func_standard
        for i in range(M):
            b = np.zeros(Ps)
            b[i] = 1
            res = scipy.optimize.minimize(fun, b.copy(), args=(b,), method="bfgs", jac=True,
                                          options=options)
            G[i, :] = res.x[:M]
            if save_g is not None:
                np.save(save_g, G)
        disp = np.max(np.abs(G - G.T))
        assert disp < 1e-4, "Error, the resulting one-phonon Green function is not Hermitian."
        return np.linalg.inv(0.5 * (G + G.T))

    def get_perturb_averages(self, R1, Y1, apply_d4=True):
        """(f_pert_av, d2v_pert_av) of the resident ensemble (GetPerturbAverageSym)."""
        ctx = self._context()
        R1 = nat.f64(R1)
        Y1 = nat.f64(Y1)
        f = np.zeros(self.n_modes)
        d2v = np.zeros((self.n_modes, self.n_modes))
        nat.check(nat.load().tdscha_perturb_averages(ctx.handle, R1.ctypes.data, Y1.ctypes.data,
                                                     1 if apply_d4 else 0, self._prec(),
                                                     f.ctypes.data, d2v.ctypes.data, 0, None))
        return f, d2v

    # ------------------------------------------------------------- Krylov
    @property
    def basis_Q(self):
        self._sync_basis()
        return self._basis_host[0]

    @basis_Q.setter
    def basis_Q(self, v):
        self._sync_basis(drop_device=True)
        self._basis_host = (list(v), self._basis_host[1] if self._basis_host else [])

    @property
    def basis_P(self):
        self._sync_basis()
        return self._basis_host[1]

    @basis_P.setter
    def basis_P(self, v):
        self._sync_basis(drop_device=True)
        self._basis_host = (self._basis_host[0] if self._basis_host else [], list(v))

    def _sync_basis(self, drop_device=False):
        if getattr(self, "_Qd", None) is not None:
            n, P = self._nbasis, self._Plen
            Q = self._Qd[:n, :P].cpu().numpy()
            Pm = self._Pd[:n, :P].cpu().numpy()
            self._basis_host = ([q for q in Q], [p for p in Pm])
            if drop_device:
                self._Qd = self._Pd = None
        elif getattr(self, "_basis_host", None) is None:
            self._basis_host = ([], [])

    def run_FT(self, n_iter, save_dir=None, save_each=5, verbose=True, n_rep_orth=0, n_ortho=10,
               flush_output=True, debug=False, prefix="LANCZOS", run_simm=None, optimized=False):
        """Lanczos iterations on the GPU (:5958-6497).

        n_rep_orth > 0 enables one pass of full re-biorthogonalisation of each
        new pair against the whole stored basis (the reference's own
        Gram-Schmidt loop is not reproduced); the default 0 matches the
        reference's default run.
        """
        self.verbose = verbose
        if not self.initialized:
            self.prepare_symmetrization()
        if self.psi is None:
            raise ValueError("Error, you must initialize a perturbation to start the Lanczos.")
        psi_norm = np.sum(np.asarray(self.psi) ** 2)
        if np.isnan(psi_norm) or psi_norm == 0:
            raise ValueError("Error, you must initialize a perturbation to start the Lanczos.\n"
                             "Use prepare_raman/ir or prepare_perturbation before calling the run method.")
        if save_dir is not None and not os.path.exists(save_dir):
            os.makedirs(save_dir)
        if run_simm is None:
            run_simm = self.use_wigner
        if run_simm and not self.use_wigner:
            raise NotImplementedError("The symmetric Lanczos works only with Wigner. Set "
                                      "use_wigner to True")
        setup = self._ft_setup(n_iter, run_simm, 1 if (n_rep_orth > 0 or self.full_reorth) else 0)
        torch = _torch()
        steps_done = nat.ctypes.c_int(0)
        conv = nat.ctypes.c_int(0)
        st = torch.cuda.current_stream().cuda_stream
        chunk = save_each if save_dir is not None else n_iter
        done = 0
        converged = False
        i_step = setup["start"]
        while done < n_iter and not converged:
            todo = min(chunk, n_iter - done)
            start = i_step + done
            t0 = time.time()
            nat.check(nat.load().tdscha_lanczos_run(
                setup["ctx"], self._Qd.data_ptr(), self._Pd.data_ptr(), setup["cap"], start, todo,
                setup["run_simm"], setup["precision"], setup["reorth"], nat.dp(setup["hist"]),
                nat.ctypes.byref(steps_done), nat.ctypes.byref(conv), st))
            n = steps_done.value
            self._ft_collect(setup["hist"], start, n, bool(conv.value))
            converged = bool(conv.value)
            done += n
            if verbose:
                print("Lanczos steps %d-%d in %.3f s" % (start + 1, start + n, time.time() - t0))
            if save_dir is not None and not converged and (start + n) % save_each == 0:
                self.save_status("%s/%s_STEP%d" % (save_dir, prefix, start + n))
        if converged and verbose:
            print("   last a coeff = {}".format(self.a_coeffs[-1]))

    def _ft_setup(self, n_iter, run_simm, reorth):
        """Device basis with room for n_iter more steps and the coefficient
        history in the C-ABI layout (rows of a, b, c, s_norm)."""
        torch = _torch()
        ctx = self._context()
        P = ctx.P
        i_step = len(self.a_coeffs)
        mask = self.mask_dot_wigner() if run_simm else None
        dev = torch.device("cuda")
        if i_step == 0:
            psi = np.asarray(self.psi, dtype=np.float64)
            if not run_simm:
                first = psi / np.sqrt(psi.dot(psi))
            else:
                first = psi / np.sqrt(psi.dot(psi * mask))
            self.s_norm = [1]
        else:
            if len(self.b_coeffs) != len(self.c_coeffs):
                raise AssertionError("Something wrong when restoring the Lanczos. len b = {} len c = {}"
                                     .format(len(self.b_coeffs), len(self.c_coeffs)))
        cap = i_step + n_iter + 2
        # rows padded to 32 doubles; the context is told the stride
        ld = ctx.basis_ld()
        ctx.set_basis_ld(ld)
        if i_step == 0 or self._Qd is None or self._Qd.shape[0] < cap:
            Qd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
            Pd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
            if i_step == 0:
                Qd[0, :P].copy_(torch.from_numpy(first))
                Pd[0, :P].copy_(torch.from_numpy(first))
            elif self._Qd is not None:
                Qd[: self._nbasis].copy_(self._Qd[: self._nbasis])
                Pd[: self._nbasis].copy_(self._Pd[: self._nbasis])
            else:
                Qh = np.asarray(self._basis_host[0], dtype=np.float64)
                Ph = np.asarray(self._basis_host[1], dtype=np.float64)
                Qd[: len(Qh), :P].copy_(torch.from_numpy(Qh))
                Pd[: len(Ph), :P].copy_(torch.from_numpy(Ph))
            self._Qd, self._Pd, self._Plen = Qd, Pd, P
        self._nbasis = i_step + 1
        self._basis_host = None
        hist = np.zeros(4 * cap, dtype=np.float64)
        hist[0:4 * len(self.a_coeffs):4] = self.a_coeffs
        hist[1:4 * len(self.b_coeffs):4] = self.b_coeffs
        hist[2:4 * len(self.c_coeffs):4] = self.c_coeffs
        s_prev = list(self.s_norm)[: i_step + 1]
        hist[3:4 * len(s_prev):4] = s_prev
        return {"ctx": ctx.handle, "cap": cap, "start": i_step, "hist": hist, "kind": 0,
                "run_simm": 1 if run_simm else 0, "precision": self._prec(), "reorth": reorth}

    def _ft_collect(self, hist, start, n, converged):
        """Append the coefficients of steps start .. start+n-1 from the history."""
        for k in range(start, start + n):
            self.a_coeffs.append(float(hist[4 * k]))
            if converged and k == start + n - 1:
                break
            self.b_coeffs.append(float(hist[4 * k + 1]))
            self.c_coeffs.append(float(hist[4 * k + 2]))
            self.s_norm.append(float(hist[4 * (k + 1) + 3]))
            self._nbasis = k + 2

    def get_green_function_continued_fraction(self, w_array, use_terminator=True, last_average=1,
                                              smearing=0, smooth_ramp=0):
        """G(w) by the continued fraction, evaluated on the GPU (:5032-5162)."""
        w_array = np.ascontiguousarray(w_array, dtype=np.float64)
        a = np.ascontiguousarray(self.a_coeffs, dtype=np.float64)
        b = np.ascontiguousarray(self.b_coeffs, dtype=np.float64)
        c = np.ascontiguousarray(self.c_coeffs, dtype=np.float64)
        if len(a) == 0:
            raise ValueError("no Lanczos coefficients")
        out = np.zeros(2 * w_array.size, dtype=np.float64)
        nat.check(nat.load().tdscha_continued_fraction(
            nat.dp(a), len(a), nat.dp(b), len(b), nat.dp(c), len(c),
            nat.dp(w_array.ravel()), w_array.size, 1 if self.use_wigner else 0,
            float(self.perturbation_modulus), 1 if self.reverse_L else 0,
            float(self.shift_value), 1 if use_terminator else 0, int(last_average),
            float(smearing), int(smooth_ramp), nat.dp(out)))
        return (out[0::2] + 1j * out[1::2]).reshape(w_array.shape)

    def get_static_frequency(self, smearing=0):
        """sign(w2) sqrt(|w2|) with w2 = 1 / Re G(w = 0 + i smearing), G the continued
        fraction without terminator (:5424-5461): the free-energy curvature along the
        perturbation, negative when it is unstable.  Returned in the reference's form
        (a one-element float64 array)."""
        gf = self.get_green_function_continued_fraction(np.array([0]), False, smearing=smearing)
        w2 = 1 / np.real(gf)
        return np.float64(np.sqrt(np.abs(w2)) * np.sign(w2))

    def build_lanczos_matrix_from_coeffs(self, use_arnoldi=False):
        """The tridiagonal Lanczos matrix (a on the diagonal, b below, c above, b above
        when no c were produced), or the symmetric matrix of the stored Arnoldi rows;
        reversed and shifted as the operator was (:4652-4693)."""
        n = len(self.a_coeffs)
        if use_arnoldi:
            if not len(self.b_coeffs) > len(self.c_coeffs):
                raise AssertionError("Error, cannot Arnoldi with non-symmetric Lanczos not implemented")
            matrix = np.zeros((n, n), dtype=TYPE_DP)
            for i in range(n):
                matrix[:i + 1, i] = self.arnoldi_matrix[i]
                matrix[i, :i + 1] = self.arnoldi_matrix[i]
        else:
            a = np.asarray(self.a_coeffs, dtype=TYPE_DP)
            b = np.asarray(self.b_coeffs, dtype=TYPE_DP)[:max(n - 1, 0)]
            up = b if len(self.c_coeffs) != len(self.b_coeffs) else \
                np.asarray(self.c_coeffs, dtype=TYPE_DP)[:max(n - 1, 0)]
            matrix = np.diag(a) + np.diag(b, -1) + np.diag(up, 1)
        sign = -1 if self.reverse_L else 1
        return sign * matrix - sign * np.eye(n) * self.shift_value

    # ------------------------- Lehmann representation on a stored Krylov basis
    def _krylov_eigenpairs(self, use_arnoldi, drop_last):
        """Eigenpairs of the Lanczos (or Arnoldi) matrix with the eigenvectors taken
        back to psi space through the stored Krylov basis (krilov_basis, the vectors a
        status saved by the reference's earlier symmetric Lanczos holds).  drop_last:
        "always" drops the basis' last vector, "extra" only when it has one vector
        more than the matrix (a run that did not converge)."""
        matrix = self.build_lanczos_matrix_from_coeffs(use_arnoldi)
        vals, vecs = np.linalg.eigh(matrix)
        kb = np.array(self.krilov_basis)
        if drop_last == "always" or (drop_last == "extra" and kb.shape[0] > len(vals)):
            kb = kb[:-1, :]
        return vals, kb.T @ vecs

    def _to_modes(self, v):
        return (np.asarray(v) / np.sqrt(self.m)) @ self.pols

    def get_green_function_Lenmann(self, w_array, smearing, v_a, v_b, use_arnoldi=False):
        """G_ab(w) = sum_j <v_a|j><j|v_b> / (lambda_j - w^2 + 2 i w smearing) over the
        eigenpairs of the symmetric Lanczos matrix (:4696-4750); v_a, v_b Cartesian
        (3 nat), mass-scaled into the mode basis."""
        if not len(self.c_coeffs) < len(self.b_coeffs):
            raise AssertionError("Lenmann cannot be used with non-symmetric Lanczos")
        va, vb = self._to_modes(v_a), self._to_modes(v_b)
        vals, vecs = self._krylov_eigenpairs(use_arnoldi, "always")
        R = vecs[:self.n_modes, :]
        weights = (va @ R) * (vb @ R)
        w = np.asarray(w_array)
        den = vals[None, :] - (w ** 2)[:, None] + 2j * (w * smearing)[:, None]
        return np.sum(weights[None, :] / den, axis=1)

    def get_spectral_function_from_Lenmann(self, w_array, smearing, use_arnoldi=True):
        """-Im sum_j |<R|j>|^2 / (lambda_j - w^2 + 2 i w smearing), the R-sector weight
        of every eigenvector (:4984-5030)."""
        vals, vecs = self._krylov_eigenpairs(use_arnoldi, "extra")
        R = vecs[:self.n_modes, :]
        weights = np.sum(np.conj(R) * R, axis=0)
        w = np.asarray(w_array)
        den = vals[None, :] - (w ** 2)[:, None] + 2j * (w * smearing)[:, None]
        return -np.imag(np.sum(weights[None, :] / den, axis=1))

    def get_static_odd_fc(self, use_arnoldi=False):
        """Static force constants from the Lanczos eigenpairs (:4752-4822):
        D = sum_i lambda_i R_i R_i^T in the mode basis, taken to Cartesian coordinates
        and scaled by sqrt(m_a m_b)."""
        vals, vecs = self._krylov_eigenpairs(use_arnoldi, "extra")
        R = vecs[:self.n_modes, :]
        D = (R * vals[None, :]) @ R.T
        fc = self.pols @ D @ self.pols.T
        return fc * np.sqrt(np.outer(self.m, self.m))

    def run_full_diag(self, number, discard_dyn=True, n_iter=100):
        """The `number` largest eigenpairs of L by ARPACK (scipy eigsh on L_linop, every
        application on the GPU) from the current psi (:6500-6543); eigvects keep only
        the R sector when discard_dyn.  Like the reference, eigsh treats L as symmetric."""
        import scipy.sparse.linalg
        eigvals, eigvects = scipy.sparse.linalg.eigsh(self.L_linop, k=number, v0=self.psi,
                                                      ncv=n_iter)
        self.eigvals = eigvals
        self.eigvects = eigvects
        if discard_dyn:
            eigvects = eigvects[:self.n_modes, :]
        return eigvals, eigvects

    def run(self, n_iter, save_dir=".", verbose=True):
        """Deprecated in the reference (:4497-4517): use run_FT."""
        raise ValueError("Error, this run funciton has been deprecated, use run_FT instead.")

    # ------------------------------------------- input files of the executable
    def prepare_input_files(self, root_name="tdscha", n_steps=100, start_from_scratch=True,
                            directory=".", run_symm=False):
        """Write the input of the input-file Lanczos program (:873-975): the same
        files and formats as the reference, read by tdscha-lanczos-gb300 (and by
        the reference's tdscha-lanczos.x)."""
        import json
        if not self.initialized:
            self.prepare_symmetrization()
        Nsyms = int(np.shape(self.symmetries[0])[0])
        json_data = {"T": self.T, "n_steps": n_steps, "ignore_v2": self.ignore_harmonic,
                     "ignore_v3": self.ignore_v3, "ignore_v4": self.ignore_v4,
                     "use_wigner": self.use_wigner, "run_sym": run_symm,
                     "data": {"n_configs": int(self.N), "n_modes": int(self.n_modes),
                              "n_syms": Nsyms, "n_blocks": len(self.symmetries),
                              "perturbation_modulus": self.perturbation_modulus,
                              "reverse": self.reverse_L, "shift": self.shift_value}}
        if not start_from_scratch:
            raise NotImplementedError("Error, restarting from a previous calculation is not yet "
                                      "implemented.")
        root = os.path.join(directory, root_name)
        if not os.path.exists(directory):
            os.makedirs(directory)
        with open(root + ".json", "w") as fp:
            json.dump(json_data, fp)
        np.savetxt(root + ".ndegs", self.N_degeneracy, fmt="%d")
        np.savetxt(root + ".blockid", self.sym_block_id, fmt="%d")
        np.savetxt(root + ".masses", self.m)
        np.savetxt(root + ".freqs", self.w)
        np.savetxt(root + ".rho", self.rho)
        np.savetxt(root + ".X.dat", self.X)
        np.savetxt(root + ".Y.dat", self.Y)
        np.savetxt(root + ".psi", self.psi)
        for i, sym in enumerate(self.symmetries):
            np.savetxt(root + ".block{:d}".format(i), self.degenerate_space[i], fmt="%d")
            ns, b1, b2 = sym.shape
            with open(root + ".symsb{:d}".format(i), "w") as fp:
                for isym in range(ns):
                    for k1 in range(b1):
                        fp.write("".join(" {:22.16f}".format(sym[isym, k1, k2])
                                         for k2 in range(b2)))
                        fp.write("\n")
                    fp.write("\n")

    def load_from_input_files(self, root_name="tdscha", directory="."):
        """Read the output of the input-file Lanczos program (:978-1057)."""
        import json
        import warnings
        if not os.path.exists(directory):
            raise IOError("Error, the specified directory '{}' does not exist".format(directory))
        abc_file = os.path.join(directory, "{}.abc".format(root_name))
        if not os.path.exists(abc_file):
            errmsg = ("\nError, the file '{}' does not exist. \n       please, check if you "
                      "correctly run the tdscha-lanczos.x executable.\n".format(abc_file))
            print(errmsg)
            raise IOError(errmsg)
        with open(abc_file) as fp:
            rows = [l.split() for l in fp if l.strip()]
        full = [r for r in rows if len(r) == 3]
        self.a_coeffs = [float(r[0]) for r in rows]
        self.b_coeffs = [float(r[1]) for r in full]
        self.c_coeffs = [float(r[2]) for r in full]
        q_file = os.path.join(directory, "{}.qbasis.out".format(root_name))
        p_file = os.path.join(directory, "{}.pbasis.out".format(root_name))
        s_file = os.path.join(directory, "{}.snorm.out".format(root_name))
        Qb = Pb = None
        if os.path.exists(q_file):
            Qb = np.atleast_2d(np.loadtxt(q_file, dtype=np.double))
        else:
            warnings.warn("\nFile {} not found. basis_Q not loaded.\n".format(q_file))
        if os.path.exists(p_file):
            Pb = np.atleast_2d(np.loadtxt(p_file, dtype=np.double))
        else:
            warnings.warn("\nFile {} not found. basis_P not loaded.\n".format(p_file))
        if Qb is not None or Pb is not None:
            self._Qd = self._Pd = None
            self._basis_host = (list(Qb) if Qb is not None else [],
                                list(Pb) if Pb is not None else [])
        if os.path.exists(s_file):
            self.s_norm = list(np.loadtxt(s_file, dtype=np.double).ravel())
        else:
            warnings.warn("\nFile {} not found. S norm not loaded.\n".format(s_file))
        with open(os.path.join(directory, root_name + ".json"), "r") as fp:
            js = json.load(fp)
        self.perturbation_modulus = js["data"]["perturbation_modulus"]
        self.T = js["T"]
        self.ignore_harmonic = js["ignore_v2"]
        self.ignore_v3 = js["ignore_v3"]
        self.ignore_v4 = js["ignore_v4"]
        self.N = js["data"]["n_configs"]
        self.n_modes = js["data"]["n_modes"]
        self.reverse_L = js["data"]["reverse"]
        self.shift_value = js["data"]["shift"]

    # ------------------------------------------------------------ I/O
    def save_abc(self, file):
        total = len(self.a_coeffs)
        abc = np.zeros((total, 3), dtype=np.double)
        abc[:, 0] = self.a_coeffs
        abc[: len(self.b_coeffs), 1] = self.b_coeffs
        abc[: len(self.c_coeffs), 2] = self.c_coeffs
        np.savetxt(file, abc, header="a; b; c")

    def load_abc(self, file):
        abc = np.loadtxt(file)
        self.a_coeffs = abc[:, 0]
        self.b_coeffs = abc[:, 1]
        self.c_coeffs = abc[:, 2]

    def save_status(self, file):
        """npz with the reference's key set (:3678-3727)."""
        if ".npz" not in file.lower():
            file += ".npz"
        np.savez_compressed(file, T=self.T, nat=self.nat, m=self.m, w=self.w, pols=self.pols,
                            n_modes=self.n_modes, ignore_v3=self.ignore_v3,
                            ignore_v4=self.ignore_v4, N=self.N, rho=self.rho, X=self.X, Y=self.Y,
                            psi=self.psi, a_coeffs=self.a_coeffs, b_coeffs=self.b_coeffs,
                            c_coeffs=self.c_coeffs, basis_Q=np.asarray(self.basis_Q),
                            basis_P=np.asarray(self.basis_P), s_norm=self.s_norm,
                            krilov_basis=self.krilov_basis, arnoldi_matrix=self.arnoldi_matrix,
                            reverse=self.reverse_L, shift=self.shift_value,
                            perturbation_modulus=self.perturbation_modulus,
                            use_wigner=self.use_wigner, ignore_small_w=self.ignore_small_w,
                            sym_julia=self.sym_julia, deg_julia=self.deg_julia,
                            n_syms=self.n_syms)

    def load_status(self, file, is_file_instance=False):
        """Restore a status written by save_status (this class's or the reference's)."""
        if not is_file_instance:
            if ".npz" not in file.lower():
                file += ".npz"
            if not os.path.exists(file):
                raise IOError("Error while loading %s" % file)
        data = dict(np.load(file, allow_pickle=True))
        self.T = np.double(data["T"])
        self.nat = int(data["nat"])
        self.m = data["m"]
        self.w = data["w"]
        self.pols = data["pols"]
        self.n_modes = int(data["n_modes"])
        self.ignore_v3 = bool(data["ignore_v3"])
        self.ignore_v4 = bool(data["ignore_v4"])
        self.N = int(data["N"])
        self.rho = data["rho"]
        self.N_eff = np.sum(self.rho)
        self.X = np.ascontiguousarray(data["X"])
        self.Y = np.ascontiguousarray(data["Y"])
        self.psi = data["psi"]
        self.a_coeffs = list(data["a_coeffs"])
        self.b_coeffs = list(data["b_coeffs"])
        self.c_coeffs = list(data["c_coeffs"]) if "c_coeffs" in data else []
        self.krilov_basis = data["krilov_basis"]
        self.arnoldi_matrix = data["arnoldi_matrix"]
        self.n_syms = int(data["n_syms"]) if "n_syms" in data else 1
        self._Qd = self._Pd = None
        self._basis_host = (list(data["basis_Q"]), list(data["basis_P"]))
        self.s_norm = list(data["s_norm"])
        self.use_wigner = bool(data["use_wigner"])
        self.ignore_small_w = bool(data.get("ignore_small_w", False))
        if "reverse" in data:
            self.reverse_L = bool(data["reverse"])
            self.shift_value = float(data["shift"])
        if "perturbation_modulus" in data:
            self.perturbation_modulus = float(data["perturbation_modulus"])
        self._invalidate()


def is_julia_enabled():
    """The reference's switch for its Julia kernels (:171-180); this build has none."""
    return False


def _run_length(b_row, n_steps):
    """Steps of a run whose b_n table is zero-padded after it stopped: up to and
    including the step before the first zero b_n."""
    zeros = np.flatnonzero(np.asarray(b_row)[:n_steps - 1] == 0)
    return n_steps if zeros.size == 0 else int(zeros[0]) + 1


def GetFreeEnergyCurvatureFromContinuedFraction(a_ns, b_ns, pols_sc, masses, mode_mixing=True,
                                                use_terminator=True, last_average=5, smearing=0,
                                                reference_contraction=True):
    """Free-energy curvature in the supercell from one symmetric Lanczos run per
    mode (a_ns[i, i]) and, with mode_mixing, per pair of modes (a_ns[i, j], the run
    started from e_i + e_j) (:7084-7192).  G_ij(0) comes from each run's continued
    fraction (on the GPU); the pair runs give the off-diagonal terms as
    (G_{i+j} - G_ii - G_jj) / 2; the curvature is G^-1 = F taken back to Cartesian
    coordinates with E = sqrt(m) e.  Like the reference, writes gf_mat.dat and
    fc_pols.dat in the working directory.

    The reference's final contraction, einsum("ab, ca, da -> cd"), sums F over its
    second index before the change of basis: sum_a (sum_b F_ab) E_ca E_da rather
    than E F E^T.  That result is returned by default (parity);
    reference_contraction=False returns E F E^T."""
    a_ns, b_ns = np.asarray(a_ns), np.asarray(b_ns)
    n_modes = np.shape(pols_sc)[1]
    n_steps = np.shape(a_ns)[2]
    if n_steps - 1 != np.shape(b_ns)[2]:
        raise AssertionError("Error, an and bn has an incompatible size:\n a_n = {}, b_n = {}"
                             .format(np.shape(a_ns), np.shape(b_ns)))

    def g0(i, j, modulus):
        n = _run_length(b_ns[i, j], n_steps)
        lanc = Lanczos(None)
        lanc.a_coeffs = a_ns[i, j, :n]
        lanc.b_coeffs = b_ns[i, j, :n - 1]
        lanc.perturbation_modulus = modulus
        print("Computing ({},{}) ... n_steps = {}".format(i, j, n))
        return np.real(lanc.get_green_function_continued_fraction(
            np.array([0]), use_terminator=use_terminator, smearing=smearing,
            last_average=last_average)[0])

    G = np.zeros((n_modes, n_modes), dtype=np.double)
    for i in range(n_modes):
        G[i, i] = g0(i, i, 1)
    if mode_mixing:
        for i in range(n_modes):
            for j in range(i + 1, n_modes):
                G[i, j] = G[j, i] = (g0(i, j, 2) - G[i, i] - G[j, j]) / 2
    np.savetxt("gf_mat.dat", G)
    fc_pols = np.linalg.inv(G)
    np.savetxt("fc_pols.dat", fc_pols)
    e_m = np.asarray(pols_sc) * np.sqrt(np.asarray(masses))[:, None]
    if reference_contraction:
        return np.einsum("a, ca, da -> cd", fc_pols.sum(axis=1), e_m, e_m)
    return e_m @ fc_pols @ e_m.T


def get_full_L_matrix(lanczos, transpose=False, static=False, compute_anharm=True,
                      compute_harm=True, chunk=1024):
    """The dense operator, column by column, for checks on small systems (:7365-7418).
    Dynamic: L e_i (or L^T e_i) through lanczos.L_linop, one GPU application per
    column (which, like the reference's, leaves the last column in lanczos.psi).
    static=True: the static operator on the M + M(M+1)/2 sector, harmonic and/or
    anharmonic part, applied to `chunk` unit vectors per batched GPU call (the static
    operator is symmetric, so transpose does not change it)."""
    print()
    print('Getting the full L matrix')
    print('Are we using the Wigner representation = {}'.format(lanczos.use_wigner))
    print()
    if not static:
        L_op = lanczos.L_linop
        n = len(lanczos.psi)
        L = np.zeros((n, n), dtype=np.double)
        v = np.zeros(n, dtype=np.double)
        for i in range(n):
            print("Step {} out of {}".format(i + 1, n))
            v[:] = 0.0
            v[i] = 1.0
            L[:, i] = L_op.rmatvec(v) if transpose else L_op.matvec(v)
        return L
    what = (1 if compute_harm else 0) | (2 if compute_anharm else 0)
    n = lanczos._static_size()
    L = np.zeros((n, n), dtype=np.double)
    lanczos.psi = np.zeros(n, dtype=TYPE_DP)
    if what == 0:
        return L
    for i0 in range(0, n, chunk):
        k = min(chunk, n - i0)
        L[:, i0:i0 + k] = lanczos._static_unit_rows(i0, k, what).T
    return L
