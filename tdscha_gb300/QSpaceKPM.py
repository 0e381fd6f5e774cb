"""Drop-in for tdscha.QSpaceKPM (Modules/QSpaceKPM.py) on the GPU.

Chebyshev moments of the q-space operator with the two-moments-per-application
recurrence of run_KPM; the loop runs on the device (tdscha_qkpm_run: operator
application, Chebyshev update and the Wigner-metric dot products, moments kept
in device memory and read once at the end).
"""
import time

import numpy as np

from . import _native as nat
from .DynamicalLanczos import _torch, __EPSILON__
from .QSpaceLanczos import QSpaceLanczos

RY_TO_CM = 109691.40235


class QSpaceKPM(QSpaceLanczos):
    """Kernel Polynomial Method with the q-space Liouvillian (QSpaceKPM.py:17)."""

    def __init__(self, ensemble=None, lo_to_split=None, **kwargs):
        super().__init__(ensemble, lo_to_split=lo_to_split, **kwargs)
        self.use_wigner = True
        self._init_kpm_attributes()

    def _init_kpm_attributes(self):
        self.kpm_moments = None
        self.kpm_vector_norm = None
        self.kpm_n_moments = 0
        self.kpm_lambda_min = None
        self.kpm_lambda_max = None
        self.kpm_rescale_a = None
        self.kpm_rescale_b = None
        self.kpm_bound_factor = None
        self.kpm_chebyshev_vm = None
        self.kpm_chebyshev_v = None

    _invalidate_kpm_cache = _init_kpm_attributes

    @classmethod
    def from_qspace_lanczos(cls, qlanc):
        """A QSpaceKPM sharing the data of a QSpaceLanczos (:561-632)."""
        kpm = cls()
        for k, v in vars(qlanc).items():
            if k.startswith("_qctx") or k in ("_ctx", "_ctx_key", "_Qd", "_Pd"):
                continue
            setattr(kpm, k, v)
        kpm._qctx = None
        kpm._qctx_key = None
        kpm._qpert_key = None
        kpm._init_kpm_attributes()
        return kpm

    def reset_q(self):
        super().reset_q()
        self._invalidate_kpm_cache()

    def _metric_dot(self, v1, v2, mask=None):
        if mask is None:
            mask = self.mask_dot_wigner(False)
        return np.real(np.conj(v1).dot(v2 * mask))

    def _get_kpm_bounds(self, lambda_min=None, lambda_max=None, bound_factor=2.5,
                        edge_buffer=1e-8):
        """Spectral bounds (:156-176): from the largest valid frequency unless given."""
        if (lambda_min is None) != (lambda_max is None):
            raise ValueError("lambda_min and lambda_max must be both specified or both omitted")
        if lambda_min is None:
            max_w = np.max(np.abs(self.w_q[self.valid_modes_q]))
            width = (2 * max_w) ** 2
            margin = (bound_factor - 1) * width
            if self.use_wigner:
                lmin, lmax = -width - margin, margin
            else:
                lmin, lmax = -margin, width + margin
            span = lmax - lmin
            return lmin - edge_buffer * span, lmax + edge_buffer * span
        if lambda_min >= lambda_max:
            raise ValueError("Invalid KPM bounds: lambda_min must be smaller than lambda_max")
        span = lambda_max - lambda_min
        return lambda_min - edge_buffer * span, lambda_max + edge_buffer * span

    def estimate_kpm_steps(self, precision_cm, bound_factor=1.2, regularization="jackson"):
        """Moments for a frequency resolution precision_cm at the smallest valid
        frequency of the perturbation q-point (:178-255)."""
        if precision_cm <= 0:
            raise ValueError("precision_cm must be positive")
        if bound_factor <= 1.0:
            raise ValueError("bound_factor must be > 1.0")
        if self.iq_pert is None:
            raise ValueError("Must prepare a perturbation before estimating KPM steps")
        w_at_q = self.w_q[:, self.iq_pert]
        valid_at_q = self.valid_modes_q[:, self.iq_pert]
        w_min = np.min(np.abs(w_at_q[valid_at_q]))
        if w_min < __EPSILON__:
            raise ValueError("Smallest frequency at q-point is effectively zero; cannot estimate steps")
        delta_omega = precision_cm / RY_TO_CM
        lmin, lmax = self._get_kpm_bounds(bound_factor=bound_factor, edge_buffer=1e-8)
        rescale_a = 0.5 * (lmax - lmin)
        n_moments = int(np.ceil(np.pi * rescale_a / (2.0 * w_min * delta_omega)))
        return max(n_moments, 8)

    # ----------------------------------------------------------------- run
    def _dev_loop(self, vm, v, n_start, moments):
        """tdscha_qkpm_run from T_{n_start-1}, T_{n_start}; returns (vm, v) host."""
        torch = _torch()
        ctx = self._qcontext()
        dev = torch.device("cuda")
        to_dev = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=np.complex128)
                                            .view(np.float64)).to(dev)
        A, B = to_dev(vm), to_dev(v)
        W = torch.empty_like(A)
        mom = torch.from_numpy(np.ascontiguousarray(moments)).to(dev)
        sw = nat.ctypes.c_int(0)
        st = torch.cuda.current_stream().cuda_stream
        nat.check(nat.load().tdscha_qkpm_run(ctx.handle, A.data_ptr(), B.data_ptr(), W.data_ptr(),
                                             int(n_start), int(self.kpm_n_moments),
                                             float(self.kpm_rescale_a), float(self.kpm_rescale_b),
                                             mom.data_ptr(), nat.ctypes.byref(sw), st))
        if sw.value:
            A, B = B, A
        moments[:] = mom.cpu().numpy()
        cpl = lambda t: t.cpu().numpy().view(np.complex128).copy()
        return cpl(A), cpl(B)

    def _rescaled_L(self, vec):
        return (self.apply_full_L(vec) - self.kpm_rescale_b * vec) / self.kpm_rescale_a

    def run_KPM(self, n_moments, lambda_min=None, lambda_max=None, bound_factor=1.2,
                edge_buffer=1e-8, verbose=True):
        """Chebyshev moments, two per operator application (:260-454); continues
        from saved recurrence vectors when they exist."""
        if n_moments < 1:
            raise ValueError("n_moments must be positive")
        if self.psi is None or self._psi_size is None:
            raise ValueError("Prepare a perturbation before running KPM")
        mask = self.mask_dot_wigner(False)
        existing = self.kpm_n_moments
        can_continue = (existing > 0 and self.kpm_moments is not None
                        and self.kpm_chebyshev_v is not None)
        if can_continue and n_moments <= existing:
            if verbose:
                print("KPM: already have {} moments, {} requested. Nothing to do.".format(
                    existing, n_moments))
            return
        t0 = time.time()
        if can_continue:
            if verbose:
                print("KPM: continuing from {} to {} moments".format(existing, n_moments))
            moments = np.zeros(n_moments, dtype=np.float64)
            moments[:existing] = self.kpm_moments[:existing]
            vm = np.array(self.kpm_chebyshev_vm, dtype=np.complex128)
            v = np.array(self.kpm_chebyshev_v, dtype=np.complex128)
            if existing == 1:
                v1 = self._rescaled_L(v)
                moments[1] = self._metric_dot(vm, v1, mask)
                vm, v = v, v1
                n_start = 1
            elif existing % 2 == 0:
                n_start = existing // 2
            else:
                n_half = existing // 2
                vp = 2 * self._rescaled_L(v) - vm
                moments[2 * n_half + 1] = 2 * self._metric_dot(vp, v, mask) - moments[1]
                vm, v = v, vp
                n_start = n_half + 1
            self.kpm_n_moments = int(n_moments)
            if 2 * n_start < self.kpm_n_moments:
                vm, v = self._dev_loop(vm, v, n_start, moments)
        else:
            psi0 = np.array(self.psi, dtype=np.complex128)
            norm_sq = self._metric_dot(psi0, psi0, mask)
            if norm_sq <= __EPSILON__ or np.isnan(norm_sq):
                raise ValueError("Prepare a non-zero perturbation before running KPM")
            self.kpm_lambda_min, self.kpm_lambda_max = self._get_kpm_bounds(
                lambda_min=lambda_min, lambda_max=lambda_max, bound_factor=bound_factor,
                edge_buffer=edge_buffer)
            self.kpm_rescale_a = 0.5 * (self.kpm_lambda_max - self.kpm_lambda_min)
            self.kpm_rescale_b = 0.5 * (self.kpm_lambda_max + self.kpm_lambda_min)
            self.kpm_vector_norm = np.sqrt(norm_sq)
            self.kpm_n_moments = int(n_moments)
            self.kpm_bound_factor = bound_factor
            v0 = psi0 / self.kpm_vector_norm
            moments = np.zeros(self.kpm_n_moments, dtype=np.float64)
            moments[0] = 1.0
            vm, v = v0, v0
            if self.kpm_n_moments > 1:
                v1 = self._rescaled_L(v0)
                moments[1] = self._metric_dot(v0, v1, mask)
                vm, v = v0, v1
                if 2 < self.kpm_n_moments:
                    vm, v = self._dev_loop(vm, v, 1, moments)
            self.psi = psi0
        self.kpm_chebyshev_vm = vm.copy()
        self.kpm_chebyshev_v = v.copy()
        self.kpm_moments = moments
        if verbose:
            print("KPM completed: {} moments in {:.3f} s".format(self.kpm_n_moments,
                                                                time.time() - t0))

    # -------------------------------------------------------------- output
    @staticmethod
    def _jackson_kernel(n_moments):
        n = np.arange(n_moments, dtype=np.float64)
        phi = np.pi / (n_moments + 1)
        return ((n_moments - n + 1) * np.cos(n * phi) + np.sin(n * phi) / np.tan(phi)) / (n_moments + 1)

    def _get_kpm_damping(self, regularization="jackson", damping_factors=None):
        if self.kpm_moments is None:
            raise ValueError("Run run_KPM before requesting the spectral function")
        if damping_factors is not None:
            g = np.asarray(damping_factors, dtype=np.float64)
        elif regularization is None or str(regularization).lower() == "none":
            g = np.ones(self.kpm_n_moments, dtype=np.float64)
        elif str(regularization).lower() == "jackson":
            g = self._jackson_kernel(self.kpm_n_moments)
        else:
            raise ValueError("Unknown KPM regularization: {}".format(regularization))
        if len(g) != self.kpm_n_moments:
            raise ValueError("Damping factors must have length {}".format(self.kpm_n_moments))
        return g

    def get_spectral_function_KPM(self, w_array, regularization="jackson", damping_factors=None):
        """Spectral function from the moments (:536-559)."""
        g = self._get_kpm_damping(regularization=regularization, damping_factors=damping_factors)
        w_array = np.asarray(w_array, dtype=np.float64)
        lambdas = -(w_array ** 2) if self.use_wigner else (w_array ** 2)
        x = (lambdas - self.kpm_rescale_b) / self.kpm_rescale_a
        inside = np.abs(x) < 1
        spectral = np.zeros_like(w_array, dtype=np.float64)
        if not np.any(inside):
            return spectral
        xin = np.clip(x[inside], -1 + 1e-15, 1 - 1e-15)
        t0 = np.ones_like(xin)
        rho = g[0] * self.kpm_moments[0] * t0
        if self.kpm_n_moments > 1:
            t1 = xin.copy()
            rho += 2 * g[1] * self.kpm_moments[1] * t1
            for i in range(2, self.kpm_n_moments):
                t2 = 2 * xin * t1 - t0
                rho += 2 * g[i] * self.kpm_moments[i] * t2
                t0, t1 = t1, t2
        rho /= np.pi * self.kpm_rescale_a * np.sqrt(1 - xin ** 2)
        rho *= self.kpm_vector_norm ** 2
        spectral[inside] = np.pi * rho
        return spectral

    # ----------------------------------------------------------------- I/O
    def save_status(self, file):
        """KPM state for continuation (:80-111)."""
        if self.kpm_moments is None:
            raise ValueError("Run run_KPM before saving status")
        if ".npz" not in file.lower():
            file += ".npz"
        d = dict(kpm_n_moments=self.kpm_n_moments, kpm_vector_norm=self.kpm_vector_norm,
                 kpm_lambda_min=self.kpm_lambda_min, kpm_lambda_max=self.kpm_lambda_max,
                 kpm_rescale_a=self.kpm_rescale_a, kpm_rescale_b=self.kpm_rescale_b,
                 kpm_bound_factor=self.kpm_bound_factor, kpm_moments=self.kpm_moments)
        if self.kpm_chebyshev_vm is not None:
            d["kpm_chebyshev_vm"] = self.kpm_chebyshev_vm
        if self.kpm_chebyshev_v is not None:
            d["kpm_chebyshev_v"] = self.kpm_chebyshev_v
        np.savez_compressed(file, **d)

    def load_status(self, file):
        """Restore a state written by save_status (:113-145)."""
        if ".npz" not in file.lower():
            file += ".npz"
        d = np.load(file, allow_pickle=True)
        self.kpm_n_moments = int(d["kpm_n_moments"])
        self.kpm_vector_norm = float(d["kpm_vector_norm"])
        self.kpm_lambda_min = float(d["kpm_lambda_min"])
        self.kpm_lambda_max = float(d["kpm_lambda_max"])
        self.kpm_rescale_a = float(d["kpm_rescale_a"])
        self.kpm_rescale_b = float(d["kpm_rescale_b"])
        bf = d["kpm_bound_factor"]
        self.kpm_bound_factor = None if bf.dtype == object else float(bf)
        self.kpm_moments = np.array(d["kpm_moments"], dtype=np.float64)
        self.kpm_chebyshev_vm = np.array(d["kpm_chebyshev_vm"]) if "kpm_chebyshev_vm" in d else None
        self.kpm_chebyshev_v = np.array(d["kpm_chebyshev_v"]) if "kpm_chebyshev_v" in d else None

    def save_kpm(self, file):
        """Moments as text with the parameters in the header line (:456-471)."""
        if self.kpm_moments is None:
            raise ValueError("Run run_KPM before saving")
        header = ("kpm_n_moments={} kpm_vector_norm={} kpm_lambda_min={} kpm_lambda_max={} "
                  "kpm_rescale_a={} kpm_rescale_b={}").format(
            self.kpm_n_moments, self.kpm_vector_norm, self.kpm_lambda_min, self.kpm_lambda_max,
            self.kpm_rescale_a, self.kpm_rescale_b)
        np.savetxt(file, self.kpm_moments, header=header)

    def load_kpm(self, file):
        """Read a save_kpm file (:473-514)."""
        with open(file, "r") as f:
            header = f.readline()
        if not header.startswith("#"):
            raise ValueError("Invalid KPM save file: missing header")
        params = {}
        for part in header[1:].strip().split():
            if "=" in part:
                key, val = part.split("=")
                try:
                    params[key] = float(val)
                except ValueError:
                    params[key] = int(val)
        self.kpm_n_moments = int(params["kpm_n_moments"])
        self.kpm_vector_norm = params["kpm_vector_norm"]
        self.kpm_lambda_min = params["kpm_lambda_min"]
        self.kpm_lambda_max = params["kpm_lambda_max"]
        self.kpm_rescale_a = params["kpm_rescale_a"]
        self.kpm_rescale_b = params["kpm_rescale_b"]
        self.kpm_moments = np.atleast_1d(np.loadtxt(file))
