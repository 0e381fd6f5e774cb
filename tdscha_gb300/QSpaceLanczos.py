"""Drop-in for tdscha.QSpaceLanczos (Modules/QSpaceLanczos.py) on the GPU.

The q-space Lanczos works in the Bloch basis: psi holds R (n_bands complex
entries at the perturbation q-point) and the a', b' blocks of every unique
q-pair; the anharmonic operator is the ensemble average of
Modules/tdscha_qspace.jl:455-712, here the float64 complex kernels of
csrc/qspace.cu behind tdscha_qapply_full_L; the Hermitian Lanczos runs on the
device (tdscha_qlanczos_run).  Only the Wigner formalism exists, as in the
reference.

Pairing rule.  The reference pairs q1 with q2 such that q1 + q2 = q_pert
(build_q_pair_map, :298-333) and this class does the same by default.  With
the kernel's products conj(x_q1) alpha x_q2 and real supercell data
(X_{-q} = conj(X_q)), the pairing that commutes with lattice translations is
q2 - q1 = q_pert; the two coincide when every q-point of the grid equals its
own inverse (2x2x2 grids and Gamma).  pairing="difference" selects the
translation-invariant one; it reproduces the real-space Wigner Lanczos of the
same supercell averaged over all translations.
"""
import os
import time

import numpy as np

from . import _native as nat
from .DynamicalLanczos import Lanczos, MODE_GB300, _torch, __EPSILON__

RY_TO_K = 157887.32400374097


def find_q_index(q_target, q_points, bg, tol=1e-6):
    """Index of the q-point equal to q_target modulo the reciprocal lattice
    (QSpaceLanczos.py:94-117).  bg: reciprocal vectors / (2 pi) as rows; q in
    the same Cartesian units."""
    q_points = np.asarray(q_points, dtype=np.float64)
    bg = np.asarray(bg, dtype=np.float64)
    inv = np.linalg.inv(bg.T)
    for iq, q in enumerate(q_points):
        d = inv @ (np.asarray(q_target) - q)
        if np.abs(d - np.round(d)).max() < tol:
            return iq
    raise ValueError("q-point %s not found in the grid" % (q_target,))


class QSpaceLanczos(Lanczos):
    """Hermitian q-space Lanczos on the GPU (QSpaceLanczos.py:120)."""

    def __init__(self, ensemble=None, lo_to_split=None, **kwargs):
        kwargs["mode"] = MODE_GB300
        kwargs["use_wigner"] = True
        kwargs.pop("unwrap_symmetries", None)
        super().__init__(None, **{k: v for k, v in kwargs.items()
                                  if k in ("mode", "use_wigner", "select_modes", "precision")})
        self.use_wigner = True
        self.q_points = None
        self.n_q = 0
        self.n_bands = 0
        self.w_q = None
        self.pols_q = None
        self.valid_modes_q = None
        self.X_q = None
        self.Y_q = None
        self.iq_pert = None
        self.q_pair_map = None
        self.unique_pairs = None
        self.pairing = "sum"
        self.bg = None
        self._psi_size = None
        self._block_offsets_a = None
        self._block_offsets_b = None
        self._block_sizes = None
        self._qspace_syms = None
        self.n_syms_qspace = 0
        self._qctx = None
        self._qctx_key = None
        self._qpert_key = None
        if ensemble is not None:
            self._init_qspace_from_ensemble(ensemble, lo_to_split)

    # ------------------------------------------------------------------ setup
    @classmethod
    def from_arrays(cls, X_q, Y_q, w_q, rho, T, q_points=None, valid_modes_q=None, bg=None,
                    pols_q=None, m=None, pairing="sum", precision="fp64"):
        """Bloch-transformed ensemble: X_q, Y_q (n_q, N, n_bands) complex in the q
        mode basis (the arrays _bloch_transform_ensemble builds, :221-296), w_q
        (n_bands, n_q) in Ry.  q_points (n_q, 3) and bg (reciprocal vectors /
        2 pi, rows) locate partners; without bg, q_points are taken in crystal
        coordinates.  precision "mixed": the averages in fp32 on the CUDA
        cores (24-bit operands, float64 partial sums), the recurrence in
        float64."""
        self = cls(precision=precision)
        X_q = np.ascontiguousarray(X_q, dtype=np.complex128)
        Y_q = np.ascontiguousarray(Y_q, dtype=np.complex128)
        if X_q.ndim != 3 or X_q.shape != Y_q.shape:
            raise ValueError("X_q and Y_q must have the same (n_q, N, n_bands) shape")
        self.X_q, self.Y_q = X_q, Y_q
        self.n_q, self.N, self.n_bands = X_q.shape
        self.w_q = np.asarray(w_q, dtype=np.float64).copy()
        if self.w_q.shape != (self.n_bands, self.n_q):
            raise ValueError("w_q must be (n_bands, n_q)")
        self.rho = np.asarray(rho, dtype=np.float64).copy()
        self.N_eff = np.sum(self.rho)
        self.T = float(T)
        self.q_points = (np.zeros((self.n_q, 3)) if q_points is None
                         else np.asarray(q_points, dtype=np.float64))
        self.bg = np.eye(3) if bg is None else np.asarray(bg, dtype=np.float64)
        self.valid_modes_q = (np.ones((self.n_bands, self.n_q), dtype=bool) if valid_modes_q is None
                              else np.asarray(valid_modes_q, dtype=bool).copy())
        self.pols_q = pols_q
        self.m = np.ones(self.n_bands) if m is None else np.asarray(m, dtype=np.float64)
        self.n_modes = self.n_q * self.n_bands
        self.pairing = pairing
        return self

    def _init_qspace_from_ensemble(self, ensemble, lo_to_split):
        """Bloch transform of a sscha Ensemble (QSpaceLanczos.py:129-296); needs
        cellconstructor, which the GPU path itself does not."""
        try:
            import cellconstructor as CC
            import cellconstructor.symmetries  # noqa: F401
            import cellconstructor.Methods  # noqa: F401
        except ImportError as e:
            raise ImportError("building from a sscha Ensemble needs cellconstructor; use "
                              "QSpaceLanczos.from_arrays with the Bloch-transformed arrays") from e
        dyn = ensemble.current_dyn
        self.dyn = dyn
        self.uci_structure = dyn.structure
        self.T = ensemble.current_T
        ws_sc, pols_sc, w_q, pols_q = dyn.DiagonalizeSupercell(return_qmodes=True,
                                                                lo_to_split=lo_to_split)
        self.q_points = np.array(dyn.q_tot)
        self.n_q = len(self.q_points)
        self.n_bands = 3 * dyn.structure.N_atoms
        self.w_q, self.pols_q = w_q, pols_q
        masses_uc = dyn.structure.get_masses_array()
        self.m = np.repeat(masses_uc, 3)
        self.valid_modes_q = np.ones((self.n_bands, self.n_q), dtype=bool)
        trans = CC.Methods.get_translations(np.real(pols_q[:, :, 0]), masses_uc)
        self.valid_modes_q[:, 0] = ~trans
        if ensemble.ignore_small_w:
            for iq in range(self.n_q):
                self.valid_modes_q[:, iq] &= ~(np.abs(w_q[:, iq]) < CC.Phonons.__EPSILON_W__)
        self.bg = dyn.structure.get_reciprocal_vectors() / (2 * np.pi)
        self.rho = np.asarray(ensemble.rho, dtype=np.float64)
        self.N = len(self.rho)
        self.N_eff = np.sum(self.rho)
        if ensemble.u_disps_qspace is None:
            ensemble.fourier_gradient = True
            ensemble.init()
        u_conv, f_conv = 1.0, 1.0
        if ensemble.units == "default":
            u_conv = CC.Units.A_TO_BOHR
            f_conv = 1.0 / CC.Units.A_TO_BOHR
        elif ensemble.units == "hartree":
            f_conv = 2.0
        sqrt_m3 = np.repeat(np.sqrt(masses_uc), 3)
        f_mean = ensemble.get_average_forces(get_error=False)
        qe_sym = CC.symmetries.QE_Symmetry(dyn.structure)
        qe_sym.SetupQPoint()
        qe_sym.SymmetrizeVector(f_mean)
        n_cell = np.prod(dyn.GetSupercell())
        f_mean_g = np.sqrt(n_cell) * f_mean.ravel()
        # projection on the q modes on the GPU (:271-296)
        from .preprocessing import project_bloch
        u_q = np.transpose(ensemble.u_disps_qspace, (2, 0, 1))
        f_q = np.transpose(ensemble.forces_qspace - ensemble.sscha_forces_qspace, (2, 0, 1))
        self.X_q, self.Y_q = project_bloch(u_q, f_q, sqrt_m3 ** 2, np.transpose(pols_q, (2, 0, 1)),
                                           f_mean_gamma=f_mean_g, u_scale=u_conv, f_scale=f_conv)
        self.n_modes = self.n_q * self.n_bands

    # --------------------------------------------------------- pair layout
    def build_q_pair_map(self, iq_pert, pairing=None):
        """Partner of every q-point (QSpaceLanczos.py:298-333): q1 + q2 = q_pert
        (pairing "sum", the reference's rule) or q2 - q1 = q_pert ("difference",
        defined where that map is an involution: 2 q_pert = 0)."""
        pairing = self.pairing if pairing is None else pairing
        if pairing not in ("sum", "difference"):
            raise ValueError("pairing must be 'sum' or 'difference'")
        q = np.asarray(self.q_points, dtype=np.float64)
        inv = np.linalg.inv(np.asarray(self.bg, dtype=np.float64).T)
        self.iq_pert = int(iq_pert)
        self.q_pair_map = np.zeros(self.n_q, dtype=np.int32)
        for iq1 in range(self.n_q):
            target = (q[iq_pert] - q[iq1]) if pairing == "sum" else (q[iq1] + q[iq_pert])
            d = (inv @ (q - target).T).T
            hit = np.where(np.abs(d - np.round(d)).max(1) < 1e-6)[0]
            if len(hit) == 0:
                raise ValueError("Could not find partner for q1={} with q_pert={}".format(
                    q[iq1], q[iq_pert]))
            self.q_pair_map[iq1] = hit[0]
        qm = self.q_pair_map
        if np.any(qm[qm] != np.arange(self.n_q)):
            # q1 -> q1 + q_pert pairs each q-point with itself only when
            # 2 q_pert is a reciprocal lattice vector
            raise ValueError("pairing 'difference' needs 2 q_pert = 0 modulo the reciprocal "
                             "lattice (q_pert = %s)" % (q[iq_pert],))
        self.set_q_pair_map(iq_pert, qm)

    def set_q_pair_map(self, iq_pert, q_pair_map):
        """Use an explicit pairing (an involution on the q-points)."""
        qm = np.asarray(q_pair_map, dtype=np.int32)
        if qm.shape != (self.n_q,) or np.any(qm[qm] != np.arange(self.n_q)):
            raise ValueError("q_pair_map must be an involution of the n_q q-points")
        self.iq_pert = int(iq_pert)
        self.q_pair_map = qm
        self.unique_pairs = [(iq1, int(qm[iq1])) for iq1 in range(self.n_q) if iq1 <= qm[iq1]]
        self._compute_block_layout()
        self._qpert_key = None

    def _compute_block_layout(self):
        nb = self.n_bands
        self._block_sizes = [nb * nb if a < b else nb * (nb + 1) // 2 for a, b in self.unique_pairs]
        off = nb
        self._block_offsets_a = []
        for s in self._block_sizes:
            self._block_offsets_a.append(off)
            off += s
        self._block_offsets_b = []
        for s in self._block_sizes:
            self._block_offsets_b.append(off)
            off += s
        self._psi_size = off

    def get_psi_size(self):
        if self._psi_size is None:
            raise ValueError("Must call build_q_pair_map first")
        return self._psi_size

    def get_static_psi_size(self):
        return self._block_offsets_b[0]

    def get_block_offset(self, pair_idx, sector="a"):
        return self._block_offsets_a[pair_idx] if sector == "a" else self._block_offsets_b[pair_idx]

    def get_block_size(self, pair_idx):
        return self._block_sizes[pair_idx]

    def get_R1_q(self):
        return np.asarray(self.psi)[:self.n_bands].copy()

    @staticmethod
    def _unpack_upper_triangle(flat_data, n):
        iu = np.triu_indices(n)
        m = np.zeros((n, n), dtype=np.complex128)
        m[iu] = flat_data
        low = np.tril_indices(n, -1)
        m[low] = np.conj(m.T[low])
        return m

    @staticmethod
    def _pack_upper_triangle(mat, n):
        return np.asarray(mat)[np.triu_indices(n)]

    def get_block(self, pair_idx, sector="a", source=None):
        src = self.psi if source is None else source
        iq1, iq2 = self.unique_pairs[pair_idx]
        off = self.get_block_offset(pair_idx, sector)
        raw = np.asarray(src)[off:off + self._block_sizes[pair_idx]]
        nb = self.n_bands
        return raw.reshape(nb, nb).copy() if iq1 < iq2 else self._unpack_upper_triangle(raw, nb)

    def get_a1_block(self, pair_idx):
        return self.get_block(pair_idx, "a")

    def get_b1_block(self, pair_idx):
        return self.get_block(pair_idx, "b")

    def set_block_in_psi(self, pair_idx, matrix, sector, target_psi):
        iq1, iq2 = self.unique_pairs[pair_idx]
        off = self.get_block_offset(pair_idx, sector)
        n = self._block_sizes[pair_idx]
        target_psi[off:off + n] = (np.asarray(matrix).ravel() if iq1 < iq2
                                   else self._pack_upper_triangle(matrix, self.n_bands))

    def mask_dot_wigner(self, debug=False):
        """1 on the R sector and on diagonal entries of self-paired blocks, 2
        elsewhere (QSpaceLanczos.py:494-535)."""
        mask = np.ones(self.get_psi_size(), dtype=np.float64)
        nb = self.n_bands
        diag = np.zeros(nb * (nb + 1) // 2, dtype=bool)
        idx = 0
        for i in range(nb):
            diag[idx] = True
            idx += nb - i
        for p, (iq1, iq2) in enumerate(self.unique_pairs):
            for off in (self._block_offsets_a[p], self._block_offsets_b[p]):
                n = self._block_sizes[p]
                mask[off:off + n] = 2.0
                if iq1 == iq2:
                    mask[off:off + n][diag] = 1.0
        return mask

    # ------------------------------------------------------- coefficients
    def _safe_bose_and_mask(self, iq):
        w = self.w_q[:, iq]
        v = self.valid_modes_q[:, iq]
        n = np.zeros_like(w)
        if self.T > __EPSILON__:
            n[v] = 1.0 / (np.exp(w[v] * RY_TO_K / self.T) - 1.0)
        return n, v

    def _chi(self, sign):
        out = []
        for iq1, iq2 in self.unique_pairs:
            n1, v1 = self._safe_bose_and_mask(iq1)
            n2, v2 = self._safe_bose_and_mask(iq2)
            w1, w2 = self.w_q[:, iq1][:, None], self.w_q[:, iq2][None, :]
            vm = np.outer(v1, v2)
            den = np.where(vm, 2 * w1 * w2, 1.0)
            if sign < 0:
                val = (w1 - w2) * (n1[:, None] - n2[None, :]) / den
            else:
                val = (w1 + w2) * (1 + n1[:, None] + n2[None, :]) / den
            out.append(np.where(vm, val, 0.0))
        return out

    def get_chi_minus_q(self):
        """chi- per pair block (QSpaceLanczos.py:599-625)."""
        return self._chi(-1)

    def get_chi_plus_q(self):
        """chi+ per pair block (QSpaceLanczos.py:627-651)."""
        return self._chi(+1)

    def get_alpha1_beta1_wigner_q(self, get_alpha=True):
        """alpha1 (or beta1) blocks from psi (QSpaceLanczos.py:653-707)."""
        cm, cp = self.get_chi_minus_q(), self.get_chi_plus_q()
        out = []
        for p, (iq1, iq2) in enumerate(self.unique_pairs):
            n1, v1 = self._safe_bose_and_mask(iq1)
            n2, v2 = self._safe_bose_and_mask(iq2)
            w1, w2 = self.w_q[:, iq1][:, None], self.w_q[:, iq2][None, :]
            vm = np.outer(v1, v2)
            X = (1 + 2 * n1[:, None]) * (1 + 2 * n2[None, :]) / 8
            w2X = np.where(vm, w1 * w2 / np.where(vm, X, 1.0), 0.0)
            a = self.get_block(p, "a")
            b = self.get_block(p, "b")
            if get_alpha:
                out.append(w2X * np.sqrt(-0.5 * cm[p]) * a - w2X * np.sqrt(0.5 * cp[p]) * b)
            else:
                out.append(-np.sqrt(-0.5 * cm[p]) * a - np.sqrt(0.5 * cp[p]) * b)
        return out

    # ------------------------------------------------------------ operator
    def _qcontext(self):
        key = (id(self.X_q), id(self.Y_q), self.N, self.T, id(self._qspace_syms),
               self.valid_modes_q.tobytes(), self.w_q.tobytes(), self.rho.tobytes())
        if self._qctx is None or self._qctx_key != key:
            if self._qctx is not None:
                self._qctx.close()
            self._qctx = nat.QContext(self.X_q, self.Y_q, self.w_q, self.rho, self.T,
                                      valid=self.valid_modes_q, symmetries=self._qspace_syms)
            self._qctx_key = key
            self._qpert_key = None
        if self.q_pair_map is None:
            raise ValueError("Must call build_q_pair_map (or prepare_mode_q) first")
        pkey = (self.iq_pert, self.q_pair_map.tobytes(), bool(self.ignore_harmonic),
                bool(self.ignore_v3), bool(self.ignore_v4))
        if self._qpert_key != pkey:
            P = self._qctx.set_pert(self.iq_pert, self.q_pair_map, self.ignore_harmonic,
                                    self.ignore_v3, self.ignore_v4)
            if P != self.get_psi_size():
                raise AssertionError("psi layout mismatch")
            self._qpert_key = pkey
        self._qctx.set_precision(self.precision)
        return self._qctx

    def _invalidate(self):
        super()._invalidate()
        if getattr(self, "_qctx", None) is not None:
            self._qctx.close()
        self._qctx = None
        self._qctx_key = None
        self._qpert_key = None

    def get_perturb_averages_q(self, R1, alpha1_blocks, apply_v4=True):
        """(f_pert, d2v blocks) of get_perturb_averages_qspace (tdscha_qspace.jl:639-712)."""
        ctx = self._qcontext()
        nb = self.n_bands
        R1 = np.ascontiguousarray(R1, dtype=np.complex128)
        al = np.ascontiguousarray(np.stack(alpha1_blocks), dtype=np.complex128)
        if R1.shape != (nb,) or al.shape != (ctx.n_pairs, nb, nb):
            raise ValueError("R1 must be (n_bands,) and alpha1 (n_pairs, n_bands, n_bands)")
        f = np.zeros(nb, dtype=np.complex128)
        d2v = np.zeros_like(al)
        nat.check(nat.load().tdscha_qperturb_averages(ctx.handle, R1.ctypes.data, al.ctypes.data,
                                                      1 if apply_v4 else 0, f.ctypes.data,
                                                      d2v.ctypes.data, 0, None))
        return f, [d2v[p] for p in range(len(d2v))]

    def apply_L1_FT(self, transpose=False):
        """Harmonic part (QSpaceLanczos.py:537-580)."""
        psi = np.asarray(self.psi, dtype=np.complex128)
        out = np.zeros(self.get_psi_size(), dtype=np.complex128)
        if self.ignore_harmonic:
            return out
        nb = self.n_bands
        out[:nb] = -(self.w_q[:, self.iq_pert] ** 2) * psi[:nb] * self.valid_modes_q[:, self.iq_pert]
        for p, (iq1, iq2) in enumerate(self.unique_pairs):
            w1, w2 = self.w_q[:, iq1], self.w_q[:, iq2]
            vm = np.outer(self.valid_modes_q[:, iq1], self.valid_modes_q[:, iq2])
            self.set_block_in_psi(p, -np.subtract.outer(w1, w2) ** 2 * self.get_block(p, "a") * vm,
                                  "a", out)
            self.set_block_in_psi(p, -np.add.outer(w1, w2) ** 2 * self.get_block(p, "b") * vm,
                                  "b", out)
        return out

    def apply_anharmonic_FT(self, transpose=False, **kwargs):
        """Anharmonic part (QSpaceLanczos.py:730-773): alpha1 from psi on the host,
        the ensemble average on the GPU."""
        out = np.zeros(self.get_psi_size(), dtype=np.complex128)
        if self.ignore_v3 and self.ignore_v4:
            return out
        R1 = self.get_R1_q()
        if self.ignore_v3:
            R1[:] = 0
        f, d2v = self.get_perturb_averages_q(R1, self.get_alpha1_beta1_wigner_q(True),
                                             not self.ignore_v4)
        out[:self.n_bands] = f
        cm, cp = self.get_chi_minus_q(), self.get_chi_plus_q()
        for p in range(len(self.unique_pairs)):
            self.set_block_in_psi(p, np.sqrt(-0.5 * cm[p]) * d2v[p], "a", out)
            self.set_block_in_psi(p, -np.sqrt(0.5 * cp[p]) * d2v[p], "b", out)
        return out

    def apply_full_L(self, target=None, force_t_0=False, force_FT=True, transpose=False,
                     fast_lanczos=True):
        """L psi in one device call (QSpaceLanczos.py:941-961)."""
        if target is not None:
            self.psi = np.asarray(target, dtype=np.complex128).copy()
        torch = _torch()
        ctx = self._qcontext()
        psi = torch.from_numpy(np.ascontiguousarray(self.psi, dtype=np.complex128)).cuda()
        out = torch.empty_like(psi)
        st = torch.cuda.current_stream().cuda_stream
        nat.check(nat.load().tdscha_qapply_full_L(ctx.handle, psi.data_ptr(), out.data_ptr(), st))
        return out.cpu().numpy()

    # ------------------------------------------------------- perturbations
    def reset_q(self):
        n = self.get_psi_size()
        self.psi = np.zeros(n, dtype=np.complex128)
        self.eigvals = None
        self.eigvects = None
        self.a_coeffs, self.b_coeffs, self.c_coeffs = [], [], []
        self.krilov_basis = []
        self.s_norm = []
        self._Qd = self._Pd = None
        self._basis_host = ([], [])

    def prepare_mode_q(self, iq, band_index):
        """Unit perturbation on mode (q, nu) (QSpaceLanczos.py:1187-1203)."""
        if band_index < 0 or band_index >= self.n_bands:
            raise ValueError("Invalid band index for perturbation: {}".format(band_index))
        self.build_q_pair_map(iq)
        self.reset_q()
        self.psi[band_index] = 1.0 + 0j
        self.perturbation_modulus = 1.0

    def prepare_perturbation_q(self, iq, vector, add=False):
        """Cartesian vector (3 n_at_uc) projected on the q modes (:1428-1451)."""
        if self.pols_q is None:
            raise ValueError("prepare_perturbation_q needs the q polarisation vectors (pols_q)")
        if not add:
            self.build_q_pair_map(iq)
            self.reset_q()
        v = np.asarray(vector) / np.sqrt(np.asarray(self.m)[: len(vector)])
        R1 = np.conj(np.asarray(self.pols_q)[:, :, iq]).T @ v
        self.psi[:self.n_bands] += R1
        self.perturbation_modulus = float(np.real(np.conj(R1) @ R1))

    # ------------------------------------------ IR / Raman perturbations (at Gamma)
    def _gamma_cells(self, n_supercell):
        """Cells of the supercell: the dynamical matrix's, n_supercell, or the q grid size."""
        if self.dyn is not None:
            return int(np.prod(self.dyn.GetSupercell()))
        if n_supercell is not None:
            return int(n_supercell)
        return int(self.n_q)

    def prepare_ir(self, effective_charges=None, pol_vec=np.array([1.0, 0.0, 0.0]),
                   n_supercell=None):
        """IR perturbation at Gamma (QSpaceLanczos.py:1205-1237): the effective charges
        contracted with the light polarisation, times sqrt(cells), projected on the
        q = 0 modes by prepare_perturbation_q."""
        ec = effective_charges
        if ec is None and self.dyn is not None:
            ec = self.dyn.effective_charges
        if ec is None:
            raise AssertionError("Error, no effective charge found. Cannot initialize IR responce")
        z_eff = np.einsum("abc, b", np.asarray(ec, dtype=np.double), pol_vec)
        self.prepare_perturbation_q(0, z_eff.ravel() * np.sqrt(self._gamma_cells(n_supercell)))

    def prepare_raman(self, pol_vec_in=np.array([1.0, 0.0, 0.0]),
                      pol_vec_out=np.array([1.0, 0.0, 0.0]), mixed=False, pol_in_2=None,
                      pol_out_2=None, unpolarized=None, raman_tensor=None, n_supercell=None):
        """Raman perturbation at Gamma (QSpaceLanczos.py:1239-1355): the Raman vector of
        the two polarisations (plus the second pair when mixed), or the terms of
        unpolarised component 0..6 summed, each times sqrt(cells)."""
        vec_fn, _ = self._raman_vector_fn(raman_tensor)
        root = np.sqrt(self._gamma_cells(n_supercell))
        if unpolarized is None:
            raman_v = np.array(vec_fn(pol_vec_in, pol_vec_out), dtype=np.double)
            if mixed:
                raman_v += vec_fn(pol_in_2, pol_out_2)
            self.prepare_perturbation_q(0, raman_v.ravel() * root)
            return
        if unpolarized not in self._UNPOL:
            raise ValueError("Error, unpolarized must be between [0, ..., 6] got invalid {}."
                             .format(unpolarized))
        e = np.eye(3)
        for k, (i, j, scale) in enumerate(self._UNPOL[unpolarized]):
            v = np.asarray(vec_fn(e[i], e[j]), dtype=np.double).ravel() * root
            self.prepare_perturbation_q(0, scale(v), add=k > 0)

    def prepare_unpolarized_raman(self, index=0, debug=False, raman_tensor=None,
                                  n_supercell=None):
        """Unpolarised Raman component `index` at Gamma (QSpaceLanczos.py:1357-1426),
        without the prefactor of get_prefactors_unpolarized_raman."""
        vec_fn, _ = self._raman_vector_fn(raman_tensor)
        if index not in range(7):
            raise ValueError('{} should be in {}'.format(index, list(range(7))))
        e = np.eye(3)
        raman_v = None
        for i, j, sgn in self._UNPOL_SUM[index]:
            v = np.asarray(vec_fn(e[i], e[j]), dtype=np.double)
            raman_v = v.copy() if raman_v is None else (raman_v + v if sgn > 0 else raman_v - v)
        if debug:
            np.save('raman_v_{}'.format(index), raman_v)
        self.prepare_perturbation_q(0, raman_v.ravel() * np.sqrt(self._gamma_cells(n_supercell)))

    def prepare_symmetrization(self, no_sym=False, verbose=True, symmetries=None):
        """q-space symmetry matrices (:1472-1531).  symmetries: list of (n_q n_bands)^2
        complex matrices (dense or scipy.sparse) acting on vectors indexed
        iq * n_bands + nu; no_sym or None keeps the identity only.  Building them
        from the crystal (spglib) needs cellconstructor and is not done here."""
        self.initialized = True
        if no_sym or symmetries is None:
            self._qspace_syms = None
            self.n_syms_qspace = 1
        else:
            self._qspace_syms = list(symmetries)
            self.n_syms_qspace = len(self._qspace_syms)

    def init(self, use_symmetries=True, symmetries=None):
        self.prepare_symmetrization(no_sym=not use_symmetries, symmetries=symmetries)
        self.initialized = True

    # -------------------------------------------------------------- Krylov
    def _sync_basis(self, drop_device=False):
        if getattr(self, "_Qd", None) is not None:
            n = self._nbasis
            Q = self._Qd[:n].cpu().numpy().view(np.complex128)
            Pm = self._Pd[:n].cpu().numpy().view(np.complex128)
            self._basis_host = ([q for q in Q], [p for p in Pm])
            if drop_device:
                self._Qd = self._Pd = None
        elif getattr(self, "_basis_host", None) is None:
            self._basis_host = ([], [])

    def run_FT(self, n_iter, save_dir=None, save_each=5, verbose=True, n_rep_orth=0, n_ortho=10,
               flush_output=True, debug=False, prefix="LANCZOS", run_simm=None, optimized=False,
               reorthogonalize=True):
        """Hermitian Lanczos on the GPU (QSpaceLanczos.py:967-1182).

        reorthogonalize=True (the default, as in the reference) runs the Gram-
        Schmidt against every stored Q vector with P = Q; False runs the plain
        recurrence (the reference's n_rep_orth = 0 branch); its biconjugate
        n_rep_orth > 0 variant is not provided.
        """
        self.verbose = verbose
        if not self.initialized:
            self.prepare_symmetrization()
        err = ("Error, you must initialize a perturbation to start the Lanczos.\n"
               "Use prepare_mode_q or prepare_perturbation_q before calling run_FT.")
        if self.psi is None or self._psi_size is None or len(self.psi) != self._psi_size:
            raise ValueError(err)
        if not reorthogonalize and n_rep_orth > 0:
            raise NotImplementedError("the biconjugate n_rep_orth > 0 Gram-Schmidt is not "
                                      "provided; use reorthogonalize=True")
        mask = self.mask_dot_wigner(debug)
        psi = np.asarray(self.psi, dtype=np.complex128)
        psi_norm = np.real(np.conj(psi).dot(psi * mask))
        if np.isnan(psi_norm) or psi_norm == 0:
            raise ValueError(err)
        if save_dir is not None and not os.path.exists(save_dir):
            os.makedirs(save_dir)
        setup = self._ft_setup(n_iter, 1 if reorthogonalize else 0)
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
            nat.check(nat.load().tdscha_qlanczos_run(
                setup["ctx"], self._Qd.data_ptr(), self._Pd.data_ptr(), setup["cap"], start, todo,
                setup["reorth"], nat.dp(setup["hist"]), nat.ctypes.byref(steps_done),
                nat.ctypes.byref(conv), st))
            n = steps_done.value
            self._ft_collect(setup["hist"], start, n, bool(conv.value))
            converged = bool(conv.value)
            done += n
            if verbose:
                print("Q-space Lanczos steps %d-%d in %.3f s" % (start + 1, start + n,
                                                                time.time() - t0))
            if save_dir is not None and not converged and (start + n) % save_each == 0:
                self.save_status("%s/%s_STEP%d" % (save_dir, prefix, start + n))
        if converged and verbose:
            print("   last a coeff = {}".format(self.a_coeffs[-1]))

    def _ft_setup(self, n_iter, reorth):
        """Device basis (interleaved complex rows) with room for n_iter more
        steps and the coefficient history in the C-ABI layout."""
        torch = _torch()
        ctx = self._qcontext()
        n2 = 2 * ctx.P
        i_step = len(self.a_coeffs)
        dev = torch.device("cuda")
        cap = i_step + n_iter + 2
        if i_step == 0:
            mask = self.mask_dot_wigner()
            psi = np.asarray(self.psi, dtype=np.complex128)
            first = psi / np.sqrt(np.real(np.conj(psi).dot(psi * mask)))
            self.s_norm = [1]
        if i_step == 0 or self._Qd is None or self._Qd.shape[0] < cap:
            Qd = torch.empty((cap, n2), dtype=torch.float64, device=dev)
            Pd = torch.empty((cap, n2), dtype=torch.float64, device=dev)
            if i_step == 0:
                row = torch.from_numpy(np.ascontiguousarray(first).view(np.float64))
                Qd[0].copy_(row)
                Pd[0].copy_(row)
            elif self._Qd is not None:
                Qd[: self._nbasis].copy_(self._Qd[: self._nbasis])
                Pd[: self._nbasis].copy_(self._Pd[: self._nbasis])
            else:
                Qh = np.ascontiguousarray(self._basis_host[0], dtype=np.complex128)
                Ph = np.ascontiguousarray(self._basis_host[1], dtype=np.complex128)
                Qd[: len(Qh)].copy_(torch.from_numpy(Qh.view(np.float64).reshape(len(Qh), n2)))
                Pd[: len(Ph)].copy_(torch.from_numpy(Ph.view(np.float64).reshape(len(Ph), n2)))
            self._Qd, self._Pd = Qd, Pd
        self._nbasis = i_step + 1
        self._basis_host = None
        hist = np.zeros(4 * cap, dtype=np.float64)
        hist[0:4 * len(self.a_coeffs):4] = self.a_coeffs
        hist[1:4 * len(self.b_coeffs):4] = self.b_coeffs
        hist[2:4 * len(self.c_coeffs):4] = self.c_coeffs
        s_prev = list(self.s_norm)[: i_step + 1]
        hist[3:4 * len(s_prev):4] = s_prev
        return {"ctx": ctx.handle, "cap": cap, "start": i_step, "hist": hist, "kind": 1,
                "run_simm": 0, "precision": 0, "reorth": reorth}

    # ------------------------------------------------------------------ I/O
    def save_status(self, file):
        if ".npz" not in file.lower():
            file += ".npz"
        np.savez_compressed(
            file, T=self.T, n_q=self.n_q, n_bands=self.n_bands, w_q=self.w_q, q_points=self.q_points,
            bg=self.bg, valid_modes_q=self.valid_modes_q, X_q=self.X_q, Y_q=self.Y_q, rho=self.rho,
            N=self.N, m=self.m, ignore_v3=self.ignore_v3, ignore_v4=self.ignore_v4,
            ignore_harmonic=self.ignore_harmonic, iq_pert=self.iq_pert,
            q_pair_map=self.q_pair_map, psi=self.psi, a_coeffs=self.a_coeffs,
            b_coeffs=self.b_coeffs, c_coeffs=self.c_coeffs,
            basis_Q=np.asarray(self.basis_Q), basis_P=np.asarray(self.basis_P),
            s_norm=self.s_norm, perturbation_modulus=self.perturbation_modulus,
            use_wigner=True, pairing=self.pairing)

    def load_status(self, file, is_file_instance=False):
        if not is_file_instance:
            if ".npz" not in file.lower():
                file += ".npz"
            if not os.path.exists(file):
                raise IOError("Error while loading %s" % file)
        d = dict(np.load(file, allow_pickle=True))
        self.T = float(d["T"])
        self.n_q, self.n_bands = int(d["n_q"]), int(d["n_bands"])
        self.w_q, self.q_points, self.bg = d["w_q"], d["q_points"], d["bg"]
        self.valid_modes_q = d["valid_modes_q"].astype(bool)
        self.X_q = np.ascontiguousarray(d["X_q"])
        self.Y_q = np.ascontiguousarray(d["Y_q"])
        self.rho = d["rho"]
        self.N = int(d["N"])
        self.N_eff = np.sum(self.rho)
        self.m = d["m"]
        self.n_modes = self.n_q * self.n_bands
        self.ignore_v3, self.ignore_v4 = bool(d["ignore_v3"]), bool(d["ignore_v4"])
        self.ignore_harmonic = bool(d["ignore_harmonic"])
        self.pairing = str(d["pairing"])
        self._invalidate()
        self.set_q_pair_map(int(d["iq_pert"]), d["q_pair_map"])
        self.psi = d["psi"]
        self.a_coeffs = list(d["a_coeffs"])
        self.b_coeffs = list(d["b_coeffs"])
        self.c_coeffs = list(d["c_coeffs"])
        self.s_norm = list(d["s_norm"])
        self.perturbation_modulus = float(d["perturbation_modulus"])
        self._Qd = self._Pd = None
        self._basis_host = (list(d["basis_Q"]), list(d["basis_P"]))
