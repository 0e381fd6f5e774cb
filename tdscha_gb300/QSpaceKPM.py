"""Drop-in for tdscha.QSpaceKPM (Modules/QSpaceKPM.py) on the GPU.

Kernel polynomial method on the q-space Liouvillian L.  With the spectrum
mapped into (-1, 1) by L~ = (L - b) / a and the start vector normalised in the
Wigner metric <u, v>_M, the moments are mu_n = <v0, T_n(L~) v0>_M.  Because L
is self-adjoint in that metric, T_m T_n = (T_{m+n} + T_|m-n|) / 2 gives two
moments per operator application from t_n = T_n(L~) v0:

    mu_2n   = 2 <t_n, t_n>_M     - mu_0,
    mu_2n+1 = 2 <t_n+1, t_n>_M   - mu_1.

A run is a sequence of moment counts; after k moments the recurrence keeps
(t_{n-1}, t_n) with n = k // 2 (for k = 1: (t_0, t_0)), so any count can be
continued -- an odd count first completes its pending odd moment.  The bulk of
the loop runs on the device (tdscha_qkpm_run: operator application, Chebyshev
update and metric dots, moments kept on the device, one read-back per run).

Spectral function: the Jackson-damped Chebyshev series (Weisse, Wellein,
Alvermann, Fehske, Rev. Mod. Phys. 78, 275 (2006), eq. 71 for the kernel)
summed with Clenshaw's backward recurrence.
"""
import os
import time

import numpy as np

from . import _native as nat
from .DynamicalLanczos import _torch, __EPSILON__
from .QSpaceLanczos import QSpaceLanczos

RY_TO_CM = 109691.40235

_STATE_FIELDS = ("kpm_n_moments", "kpm_vector_norm", "kpm_lambda_min", "kpm_lambda_max",
                 "kpm_rescale_a", "kpm_rescale_b")


def jackson_damping(n):
    """g_k, k = 0..n-1, of the Jackson kernel for an n-moment expansion."""
    theta = np.pi / (n + 1)
    k = np.arange(n, dtype=np.float64)
    return ((n + 1 - k) * np.cos(k * theta) + np.sin(k * theta) / np.tan(theta)) / (n + 1)


def chebyshev_series(coeffs, x):
    """sum_k coeffs[k] T_k(x) for every x (Clenshaw's recurrence)."""
    b1 = np.zeros_like(x)
    b2 = np.zeros_like(x)
    for c in coeffs[:0:-1]:
        b1, b2 = c + 2.0 * x * b1 - b2, b1
    return coeffs[0] + x * b1 - b2


def spectral_window(w_q, valid, use_wigner, bound_factor, edge_buffer):
    """Eigenvalue interval of L enclosing the two-phonon band.

    L's eigenvalues lie within [-(2 w_max)^2, 0] in the Wigner representation
    and [0, (2 w_max)^2] otherwise.  The window extends that band by
    (bound_factor - 1) of its width on both sides, then by edge_buffer of the
    resulting span."""
    width = (2.0 * np.max(np.abs(w_q[valid]))) ** 2
    lo, hi = (-width, 0.0) if use_wigner else (0.0, width)
    pad = (bound_factor - 1.0) * width
    lo, hi = lo - pad, hi + pad
    return _buffered(lo, hi, edge_buffer)


def _buffered(lo, hi, edge_buffer):
    span = hi - lo
    return lo - edge_buffer * span, hi + edge_buffer * span


class QSpaceKPM(QSpaceLanczos):
    """Chebyshev moments of the q-space operator (Modules/QSpaceKPM.py:17)."""

    def __init__(self, ensemble=None, lo_to_split=None, **kwargs):
        super().__init__(ensemble, lo_to_split=lo_to_split, **kwargs)
        self.use_wigner = True
        self._clear_kpm()

    def _clear_kpm(self):
        for name in _STATE_FIELDS + ("kpm_bound_factor", "kpm_moments", "kpm_chebyshev_vm",
                                     "kpm_chebyshev_v"):
            setattr(self, name, None)
        self.kpm_n_moments = 0

    _init_kpm_attributes = _clear_kpm
    _invalidate_kpm_cache = _clear_kpm

    @classmethod
    def from_qspace_lanczos(cls, qlanc):
        """A QSpaceKPM on the data of a QSpaceLanczos (the arrays are shared;
        device contexts are rebuilt on first use)."""
        kpm = cls()
        device_state = ("_ctx", "_ctx_key", "_Qd", "_Pd")
        for name, value in vars(qlanc).items():
            if not name.startswith("_qctx") and name not in device_state:
                setattr(kpm, name, value)
        kpm._qctx = kpm._qctx_key = kpm._qpert_key = None
        kpm._clear_kpm()
        return kpm

    def reset_q(self):
        super().reset_q()
        self._clear_kpm()

    # -------------------------------------------------------------- helpers
    def _metric_dot(self, v1, v2, mask=None):
        m = self.mask_dot_wigner(False) if mask is None else mask
        return float(np.real(np.vdot(v1, m * v2)))

    def _get_kpm_bounds(self, lambda_min=None, lambda_max=None, bound_factor=2.5,
                        edge_buffer=1e-8):
        """(lambda_min, lambda_max) of the expansion, given or estimated."""
        if (lambda_min is None) != (lambda_max is None):
            raise ValueError("lambda_min and lambda_max must be both specified or both omitted")
        if lambda_min is None:
            return spectral_window(self.w_q, self.valid_modes_q, self.use_wigner, bound_factor,
                                   edge_buffer)
        if not lambda_min < lambda_max:
            raise ValueError("Invalid KPM bounds: lambda_min must be smaller than lambda_max")
        return _buffered(lambda_min, lambda_max, edge_buffer)

    def estimate_kpm_steps(self, precision_cm, bound_factor=1.2, regularization="jackson"):
        """Moments that resolve precision_cm at the lowest valid frequency of
        the perturbation q-point.  The Jackson-damped expansion resolves about
        pi a / n in eigenvalue (a the half-width of the window), and an
        eigenvalue -w^2 moves by 2 w dw, so n = ceil(pi a / (2 w_min dw)),
        at least 8.  Without damping the same estimate is used."""
        if precision_cm <= 0:
            raise ValueError("precision_cm must be positive")
        if bound_factor <= 1.0:
            raise ValueError("bound_factor must be > 1.0")
        if self.iq_pert is None:
            raise ValueError("Must prepare a perturbation before estimating KPM steps")
        here = self.valid_modes_q[:, self.iq_pert]
        w_min = np.min(np.abs(self.w_q[:, self.iq_pert][here]))
        if w_min < __EPSILON__:
            raise ValueError("Smallest frequency at q-point is effectively zero; "
                             "cannot estimate steps")
        lo, hi = self._get_kpm_bounds(bound_factor=bound_factor, edge_buffer=1e-8)
        half_width = 0.5 * (hi - lo)
        resolution = 2.0 * w_min * (precision_cm / RY_TO_CM)
        return max(8, int(np.ceil(np.pi * half_width / resolution)))

    def _rescaled_L(self, vec):
        return (self.apply_full_L(vec) - self.kpm_rescale_b * vec) / self.kpm_rescale_a

    # ------------------------------------------------------------ the loop
    def _device_pairs(self, prev, cur, n_from, moments):
        """Moment pairs (2n, 2n+1) for n = n_from, ... up to the requested
        count, on the device (tdscha_qkpm_run); returns the final (prev, cur)."""
        torch = _torch()
        ctx = self._qcontext()
        dev = torch.device("cuda")

        def upload(v):
            return torch.from_numpy(np.ascontiguousarray(v, dtype=np.complex128)
                                    .view(np.float64)).to(dev)

        A, B = upload(prev), upload(cur)
        work = torch.empty_like(A)
        mom = torch.from_numpy(np.ascontiguousarray(moments)).to(dev)
        swapped = nat.ctypes.c_int(0)
        nat.check(nat.load().tdscha_qkpm_run(
            ctx.handle, A.data_ptr(), B.data_ptr(), work.data_ptr(), int(n_from),
            int(self.kpm_n_moments), float(self.kpm_rescale_a), float(self.kpm_rescale_b),
            mom.data_ptr(), nat.ctypes.byref(swapped), torch.cuda.current_stream().cuda_stream))
        moments[:] = mom.cpu().numpy()
        if swapped.value:
            A, B = B, A
        back = lambda t: t.cpu().numpy().view(np.complex128).copy()
        return back(A), back(B)

    def _start_fresh(self, n_moments, lambda_min, lambda_max, bound_factor, edge_buffer, mask):
        psi0 = np.array(self.psi, dtype=np.complex128)
        nrm2 = self._metric_dot(psi0, psi0, mask)
        if not nrm2 > __EPSILON__:
            raise ValueError("Prepare a non-zero perturbation before running KPM")
        lo, hi = self._get_kpm_bounds(lambda_min=lambda_min, lambda_max=lambda_max,
                                      bound_factor=bound_factor, edge_buffer=edge_buffer)
        self.kpm_lambda_min, self.kpm_lambda_max = lo, hi
        self.kpm_rescale_a, self.kpm_rescale_b = 0.5 * (hi - lo), 0.5 * (hi + lo)
        self.kpm_vector_norm = np.sqrt(nrm2)
        self.kpm_bound_factor = bound_factor
        v0 = psi0 / self.kpm_vector_norm
        moments = np.zeros(n_moments)
        moments[0] = 1.0
        return psi0, moments, v0, v0.copy(), 1

    def run_KPM(self, n_moments, lambda_min=None, lambda_max=None, bound_factor=1.2,
                edge_buffer=1e-8, verbose=True):
        """Compute n_moments Chebyshev moments, continuing a previous run (from
        memory or load_status) when its recurrence vectors are available;
        bounds and norm of a continued run are those of the first one."""
        if n_moments < 1:
            raise ValueError("n_moments must be positive")
        if self.psi is None or self._psi_size is None:
            raise ValueError("Prepare a perturbation before running KPM")
        mask = self.mask_dot_wigner(False)
        have = int(self.kpm_n_moments or 0)
        resumable = have > 0 and self.kpm_moments is not None and self.kpm_chebyshev_v is not None
        if resumable and n_moments <= have:
            if verbose:
                print("KPM: already have {} moments, {} requested. Nothing to do.".format(
                    have, n_moments))
            return
        t0 = time.time()
        psi0 = None
        if resumable:
            if verbose:
                print("KPM: continuing from {} to {} moments".format(have, n_moments))
            moments = np.zeros(n_moments)
            moments[:have] = np.asarray(self.kpm_moments)[:have]
            prev = np.array(self.kpm_chebyshev_vm, dtype=np.complex128)
            cur = np.array(self.kpm_chebyshev_v, dtype=np.complex128)
            k = have
        else:
            psi0, moments, prev, cur, k = self._start_fresh(n_moments, lambda_min, lambda_max,
                                                           bound_factor, edge_buffer, mask)
        self.kpm_n_moments = int(n_moments)
        # bring the recurrence to an even count: (t_{n-1}, t_n) with 2n moments
        if k < n_moments and k % 2 == 1:
            if k == 1:            # (t0, t0) -> (t0, t1), mu_1 = <t0, t1>
                nxt = self._rescaled_L(cur)
                moments[1] = self._metric_dot(cur, nxt, mask)
            else:                 # pending odd moment of a run stopped after mu_{k-1}
                nxt = 2.0 * self._rescaled_L(cur) - prev
                moments[k] = 2.0 * self._metric_dot(nxt, cur, mask) - moments[1]
            prev, cur = cur, nxt
            k += 1
        if k < n_moments:
            prev, cur = self._device_pairs(prev, cur, k // 2, moments)
        if psi0 is not None:
            self.psi = psi0
        self.kpm_chebyshev_vm, self.kpm_chebyshev_v = prev.copy(), cur.copy()
        self.kpm_moments = moments
        if verbose:
            print("KPM completed: {} moments in {:.3f} s".format(self.kpm_n_moments,
                                                                time.time() - t0))

    # -------------------------------------------------------------- output
    _jackson_kernel = staticmethod(jackson_damping)

    def _get_kpm_damping(self, regularization="jackson", damping_factors=None):
        if self.kpm_moments is None:
            raise ValueError("Run run_KPM before requesting the spectral function")
        n = self.kpm_n_moments
        if damping_factors is not None:
            g = np.asarray(damping_factors, dtype=np.float64)
        else:
            kind = "none" if regularization is None else str(regularization).lower()
            known = {"none": lambda: np.ones(n), "jackson": lambda: jackson_damping(n)}
            if kind not in known:
                raise ValueError("Unknown KPM regularization: {}".format(regularization))
            g = known[kind]()
        if g.shape != (n,):
            raise ValueError("Damping factors must have length {}".format(n))
        return g

    def get_spectral_function_KPM(self, w_array, regularization="jackson", damping_factors=None):
        """Spectral weight at the frequencies w_array (Ry): the damped series
        [g_0 mu_0 + 2 sum g_k mu_k T_k(x)] / (pi a sqrt(1 - x^2)) at
        x = (lambda - b) / a, lambda = -w^2 (Wigner) or w^2, times pi |v|^2;
        zero outside the expansion window."""
        g = self._get_kpm_damping(regularization=regularization, damping_factors=damping_factors)
        w = np.asarray(w_array, dtype=np.float64)
        lam = -w * w if self.use_wigner else w * w
        x = (lam - self.kpm_rescale_b) / self.kpm_rescale_a
        out = np.zeros_like(w)
        inside = np.abs(x) < 1.0
        if inside.any():
            c = 2.0 * g * np.asarray(self.kpm_moments, dtype=np.float64)
            c[0] *= 0.5
            xi = x[inside]
            series = chebyshev_series(c, xi)
            out[inside] = series * self.kpm_vector_norm ** 2 / (
                self.kpm_rescale_a * np.sqrt((1.0 - xi) * (1.0 + xi)))
        return out

    # ----------------------------------------------------------------- I/O
    def save_status(self, file):
        """Moments, parameters and recurrence vectors for continuation, under
        the reference's npz keys."""
        if self.kpm_moments is None:
            raise ValueError("Run run_KPM before saving status")
        payload = {k: getattr(self, k) for k in _STATE_FIELDS}
        payload.update(kpm_bound_factor=self.kpm_bound_factor, kpm_moments=self.kpm_moments)
        for k in ("kpm_chebyshev_vm", "kpm_chebyshev_v"):
            if getattr(self, k) is not None:
                payload[k] = getattr(self, k)
        np.savez_compressed(_with_npz(file), **payload)

    def load_status(self, file):
        """Restore a state written by save_status."""
        file = _with_npz(file)
        if not os.path.exists(file):
            raise IOError("KPM status file not found: {}".format(file))
        with np.load(file, allow_pickle=True) as d:
            data = {k: d[k] for k in d.files}
        self._set_parameters(data)
        bf = data.get("kpm_bound_factor")
        self.kpm_bound_factor = None if bf is None or bf.dtype == object else float(bf)
        self.kpm_moments = np.array(data["kpm_moments"], dtype=np.float64)
        self.kpm_chebyshev_vm = data.get("kpm_chebyshev_vm")
        self.kpm_chebyshev_v = data.get("kpm_chebyshev_v")

    def _set_parameters(self, params):
        self.kpm_n_moments = int(params["kpm_n_moments"])
        for k in _STATE_FIELDS[1:]:
            setattr(self, k, float(params[k]))

    def save_kpm(self, file):
        """Moments as text; the first line carries the parameters as key=value."""
        if self.kpm_moments is None:
            raise ValueError("Run run_KPM before saving")
        header = " ".join("{}={}".format(k, getattr(self, k)) for k in _STATE_FIELDS)
        np.savetxt(file, self.kpm_moments, header=header)

    def load_kpm(self, file):
        """Read a save_kpm file (enough for get_spectral_function_KPM)."""
        with open(file) as fh:
            first = fh.readline()
        if not first.startswith("#"):
            raise ValueError("Invalid KPM save file: missing header")
        params = dict(item.split("=", 1) for item in first[1:].split() if "=" in item)
        self._set_parameters(params)
        self.kpm_moments = np.atleast_1d(np.loadtxt(file))


def _with_npz(name):
    return name if ".npz" in name.lower() else name + ".npz"
