"""ORACLE -- test infrastructure only.

A CPU restatement of the reference's hot path (float64), used by `tests/`,
`__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` as the
checker.  Nothing on the product path (`tdscha_gb300`) imports this package.

* `perturb_averages`: ctypes wrapper of `perturb_avg.c` (a restatement of
  `GetPerturbAverageSym`, CModules/odd_corr_module.c:491-634).
* `OracleLanczos`: numpy restatement of the `Lanczos` driver
  (Modules/DynamicalLanczos.py): `apply_L1_FT` :2287-2445,
  `apply_anharmonic_FT` :2951-3363, `apply_full_L` :3549-3651,
  `mask_dot_wigner` :5905-5954, `run_FT` :5958-6497 and
  `get_green_function_continued_fraction` :5032-5162.

Pinning: tests/test_oracle.py checks this oracle against fixtures generated
by the reference itself (its C module compiled from source, its Python
driver imported with stubbed physics deps; tests/golden/make_golden.py),
and against the reference's own saved run tests/test_julia/LANCZOS_STEP5.npz
(first coefficient; the later ones need symmetry tables the fixture lacks).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
RY_TO_K = 157887.32400374097
EPS = 1e-12

_lib = None


def build(force=False):
    """Compile perturb_avg.c (plain C, no FMA contraction: same bits on x86 and Arm)."""
    src = os.path.join(HERE, "perturb_avg.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                           "-pthread", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        d = ctypes.POINTER(ctypes.c_double)
        i = ctypes.POINTER(ctypes.c_int)
        lib.oracle_perturb_averages.argtypes = [
            d, d, d, d, d, d, ctypes.c_double, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, i, i, d, i, d, d, ctypes.c_int]
        lib.oracle_perturb_averages.restype = ctypes.c_int
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def flatten_symmetries(symmetries, degenerate_space):
    """Reference per-block lists -> (n_deg, deg_space_flat, sym_flat)."""
    n_deg = np.array([len(b) for b in degenerate_space], dtype=np.intc)
    deg = np.ascontiguousarray(np.concatenate([np.asarray(b, dtype=np.intc) for b in degenerate_space]))
    sym = np.ascontiguousarray(np.concatenate([np.asarray(s, dtype=np.float64).ravel() for s in symmetries]))
    return n_deg, deg, sym


def identity_symmetries(M):
    """The no-symmetry tables (Modules/DynamicalLanczos.py:727-732)."""
    return ([np.ones((1, 1, 1))] * M, [np.array([i], dtype=np.intc) for i in range(M)],
            np.arange(M, dtype=np.intc))


def perturb_averages(X, Y, w, rho, R1, Y1, T, apply_d4, symmetries, degenerate_space,
                     blocks_ids, n_threads=1):
    """(f_pert_av[M], d2v_pert_av[M, M]) exactly as GetPerturbAverageSym returns them."""
    lib = _load()
    X = np.ascontiguousarray(X, dtype=np.float64)
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    R1 = np.ascontiguousarray(R1, dtype=np.float64)
    Y1 = np.ascontiguousarray(Y1, dtype=np.float64)
    blocks_ids = np.ascontiguousarray(blocks_ids, dtype=np.intc)
    N, M = X.shape
    n_deg, deg, sym = flatten_symmetries(symmetries, degenerate_space)
    S = int(np.asarray(symmetries[0]).shape[0])
    f = np.zeros(M)
    d2v = np.zeros((M, M))
    rc = lib.oracle_perturb_averages(_dp(X), _dp(Y), _dp(w), _dp(rho), _dp(R1), _dp(Y1),
                                     float(T), int(apply_d4), M, N, S, len(n_deg),
                                     _ip(n_deg), _ip(deg), _dp(sym), _ip(blocks_ids),
                                     _dp(f), _dp(d2v), int(n_threads))
    if rc != 0:
        raise ValueError("oracle_perturb_averages: bad arguments")
    return f, d2v


def bose(w, T):
    if T <= 0:
        return np.zeros_like(w)
    return 1.0 / (np.exp(w * RY_TO_K / T) - 1.0)


class OracleLanczos:
    """Numpy restatement of the reference `Lanczos` driver on the fast path."""

    def __init__(self, ens, use_wigner=True, apply_d4=True, ignore_v3=False,
                 ignore_harmonic=False, n_threads=1):
        self.X = np.ascontiguousarray(ens["X"], dtype=np.float64)
        self.Y = np.ascontiguousarray(ens["Y"], dtype=np.float64)
        self.w = np.asarray(ens["w"], dtype=np.float64)
        self.rho = np.asarray(ens["rho"], dtype=np.float64)
        self.T = float(ens["T"])
        self.N, self.n_modes = self.X.shape
        M = self.n_modes
        if ens.get("symmetries") is None:
            self.symmetries, self.degenerate_space, self.sym_block_id = identity_symmetries(M)
        else:
            self.symmetries = ens["symmetries"]
            self.degenerate_space = ens["degenerate_space"]
            self.sym_block_id = np.asarray(ens["sym_block_id"], dtype=np.intc)
        self.use_wigner = use_wigner
        self.ignore_v3 = ignore_v3
        self.ignore_v4 = not apply_d4
        self.ignore_harmonic = ignore_harmonic
        self.reverse_L = False
        self.shift_value = 0.0
        self.perturbation_modulus = 1.0
        self.n_threads = n_threads
        self.psi = np.zeros(M + M * (M + 1))
        self.a_coeffs, self.b_coeffs, self.c_coeffs = [], [], []
        self.basis_Q, self.basis_P, self.s_norm = [], [], []
        # upper triangle, row-major, i <= j (DynamicalLanczos.py:2338-2343)
        self.iu_row, self.iu_col = np.triu_indices(M)

    # --- psi layout helpers ------------------------------------------------
    def _pair_w(self):
        return self.w[self.iu_col], self.w[self.iu_row]     # (w_a, w_b)

    def _sym_from_triangle(self, v):
        M = self.n_modes
        A = np.zeros((M, M))
        A[self.iu_row, self.iu_col] = v
        A[self.iu_col, self.iu_row] = v
        return A

    def prepare_perturbation_R(self, v):
        """psi = (v, 0, 0), modulus v.v (DynamicalLanczos.py:2058-2070)."""
        self.reset()
        self.psi[:] = 0
        self.psi[: self.n_modes] = v
        self.perturbation_modulus = float(np.dot(v, v))

    def reset(self):
        self.a_coeffs, self.b_coeffs, self.c_coeffs = [], [], []
        self.basis_Q, self.basis_P, self.s_norm = [], [], []

    def mask_dot_wigner(self):
        M = self.n_modes
        mask = np.ones(M + M * (M + 1))
        off = (self.iu_row < self.iu_col)
        h = M * (M + 1) // 2
        mask[M:M + h][off] = 2
        mask[M + h:][off] = 2
        return mask

    # --- operator ------------------------------------------------------------
    def apply_L1_FT(self, psi, transpose=False):
        M = self.n_modes
        out = np.zeros_like(psi)
        if self.ignore_harmonic:
            return out
        w_a, w_b = self._pair_w()
        h = len(w_a)
        sY, sA = M, M + h
        if not self.use_wigner:
            out[:M] = (psi[:M] * self.w) * self.w
        else:
            out[:M] = -(psi[:M] * self.w) * self.w
        n_a = np.zeros_like(w_a)
        n_b = np.zeros_like(w_a)
        if self.T > 0:
            n_a = 1 / (np.exp(w_a / np.double(self.T / RY_TO_K)) - 1)
            n_b = 1 / (np.exp(w_b / np.double(self.T / RY_TO_K)) - 1)
        if not self.use_wigner:
            X_ab = -w_a**2 - w_b**2 - (2 * w_a * w_b) / ((2 * n_a + 1) * (2 * n_b + 1))
            out[sY:sA] = -X_ab * psi[sY:sA]
            Y_ab = -(8 * w_a * w_b) / ((2 * n_a + 1) * (2 * n_b + 1))
            if not transpose:
                out[sY:sA] += -Y_ab * psi[sA:]
            else:
                out[sA:] += -Y_ab * psi[sY:sA]
            X1_ab = -(2 * n_a * n_b + n_a + n_b) * (2 * n_a * n_b + n_a + n_b + 1) * (2 * w_a * w_b) / ((2 * n_a + 1) * (2 * n_b + 1))
            if not transpose:
                out[sA:] += -X1_ab * psi[sY:sA]
            else:
                out[sY:sA] += -X1_ab * psi[sA:]
            Y1_ab = -w_a**2 - w_b**2 + (2 * w_a * w_b) / ((2 * n_a + 1) * (2 * n_b + 1))
            out[sA:] += -Y1_ab * psi[sA:]
        else:
            out[sY:sA] = -(w_a**2 + w_b**2 - 2. * w_a * w_b) * psi[sY:sA]
            out[sA:] = -(w_a**2 + w_b**2 + 2. * w_a * w_b) * psi[sA:]
        return out

    def _wigner_factors(self):
        w_a, w_b = self._pair_w()
        n_a = np.zeros(()); n_b = np.zeros(())
        if self.T > 0:
            n_a = 1 / (np.exp(w_a / np.double(self.T / RY_TO_K)) - 1)
            n_b = 1 / (np.exp(w_b / np.double(self.T / RY_TO_K)) - 1)
        Xf = ((1 + 2 * n_a) * (1 + 2 * n_b) / 8)
        w2_on_X = (w_a * w_b) / Xf
        chi_m = ((w_a - w_b) * (n_a - n_b)) / (2 * w_a * w_b)
        chi_p = ((w_a + w_b) * (1 + n_a + n_b)) / (2 * w_a * w_b)
        return w2_on_X, chi_m, chi_p

    def _chi_matrices(self):
        M = self.n_modes
        w = np.tile(self.w, (M, 1))
        n = np.zeros((M, M))
        if self.T > 1e-12:
            n = 1.0 / (np.exp(w * 157887.32400374097 / self.T) - 1.0)
        chi_m = (w - w.T) * (n - n.T) / (2. * w * w.T)
        chi_p = (w + w.T) * (1 + n + n.T) / (2. * w * w.T)
        return chi_m, chi_p

    def get_R1_Y1(self, psi, transpose=False):
        """(R1, Y1) fed to the perturbation averages (DynamicalLanczos.py:3009-3053)."""
        M = self.n_modes
        h = M * (M + 1) // 2
        R1 = psi[:M].copy()
        if not self.use_wigner:
            Y1 = self._sym_from_triangle(psi[M:M + h])
            if transpose:
                Y1[~np.eye(M, dtype=bool)] /= 2
                ReA1 = self._sym_from_triangle(psi[M + h:])
                ReA1[~np.eye(M, dtype=bool)] /= 2
                n_mu = 0
                if self.T > 1e-12:
                    n_mu = 1.0 / (np.exp(self.w * 157887.32400374097 / self.T) - 1.0)
                Y_w = 2 * self.w / (2 * n_mu + 1)
                ReA_w = 2 * self.w * n_mu * (n_mu + 1) / (2 * n_mu + 1)
                cY = np.einsum("a,b,b->ab", Y_w, Y_w, Y_w) + np.einsum("a,a,b->ab", Y_w, Y_w, Y_w)
                cY *= 2
                cRA = np.einsum("a,b,b->ab", Y_w, ReA_w, Y_w) + np.einsum("a,a,b->ab", Y_w, ReA_w, Y_w)
                cRA *= 2
                Y1 = Y1 * cY + ReA1 * cRA
        else:
            w2_on_X, chi_m, chi_p = self._wigner_factors()
            new_a = w2_on_X * np.sqrt(-0.5 * chi_m) * psi[M:M + h]
            new_b = w2_on_X * np.sqrt(+0.5 * chi_p) * psi[M + h:]
            Y1 = self._sym_from_triangle(new_a - new_b)
        if self.ignore_v3:
            R1[:] = 0.
        return R1, Y1

    def perturb(self, R1, Y1):
        return perturb_averages(self.X, self.Y, self.w, self.rho, R1, Y1, self.T,
                                0 if self.ignore_v4 else 1, self.symmetries,
                                self.degenerate_space, self.sym_block_id, self.n_threads)

    def apply_anharmonic_FT(self, psi, transpose=False):
        M = self.n_modes
        R1, Y1 = self.get_R1_Y1(psi, transpose)
        f, d2v = self.perturb(R1, Y1)
        if getattr(self, "trans", None) is not None:
            f, d2v = translation_project(f, d2v, *self.trans)
        return self.repack(f, d2v, transpose)

    def repack(self, f, d2v, transpose=False):
        """(f, d2v) -> psi' (DynamicalLanczos.py:3281-3363)."""
        M = self.n_modes
        out = np.zeros(M + M * (M + 1))
        out[:M] = f
        if not self.use_wigner:
            n_mu = 0
            if self.T > 1e-12:
                n_mu = 1.0 / (np.exp(self.w * 157887.32400374097 / self.T) - 1.0)
            Y_w = 2 * self.w / (2 * n_mu + 1)
            ReA_w = 2 * self.w * n_mu * (n_mu + 1) / (2 * n_mu + 1)
            if not transpose:
                pY = np.einsum("ab,a->ab", d2v, Y_w) + np.einsum("ab,b->ab", d2v, Y_w)
                pRA = np.einsum("ab,a->ab", d2v, ReA_w) + np.einsum("ab,b->ab", d2v, ReA_w)
            else:
                Yi = 1 / Y_w
                pY = 0.5 * np.einsum("a,ab,b->ab", Yi, d2v, Yi)
                pRA = np.zeros_like(pY)
                mask = np.ones(pY.shape) * 2
                np.fill_diagonal(mask, 1)
                pY *= mask
                pRA *= mask
        else:
            chi_m, chi_p = self._chi_matrices()
            pY = np.sqrt(-0.5 * chi_m) * d2v
            pRA = -np.sqrt(+0.5 * chi_p) * d2v
        h = M * (M + 1) // 2
        out[M:M + h] = pY[self.iu_row, self.iu_col]
        out[M + h:] = pRA[self.iu_row, self.iu_col]
        return -out if not self.use_wigner else out

    def apply_full_L(self, psi, transpose=False):
        out = self.apply_L1_FT(psi, transpose)
        if not self.ignore_v3:
            out = out + self.apply_anharmonic_FT(psi, transpose)
        if self.reverse_L:
            out *= -1
        out += self.shift_value * psi
        return out

    # --- Krylov driver (no Gram-Schmidt: the reference default n_rep_orth=0) --
    def run_FT(self, n_iter, run_simm=None):
        if run_simm is None:
            run_simm = self.use_wigner
        if run_simm and not self.use_wigner:
            raise NotImplementedError("symmetric Lanczos needs use_wigner")
        mask = self.mask_dot_wigner() if run_simm else None

        def dot(x, y):
            return x.dot(y * mask) if run_simm else x.dot(y)

        psi = self.psi
        nrm = np.sum(psi ** 2)
        if np.isnan(nrm) or nrm == 0:
            raise ValueError("zero or NaN start vector")
        if len(self.a_coeffs) == 0:
            first = psi / np.sqrt(dot(psi, psi))
            self.basis_Q = [first]
            self.basis_P = [first]
            self.s_norm = [1]
        psi_q = self.basis_Q[-1]
        psi_p = self.basis_P[-1]
        for _ in range(n_iter):
            L_q = self.apply_full_L(psi_q)
            if not self.use_wigner or not run_simm:
                p_L = self.apply_full_L(psi_p, transpose=True)
            else:
                p_L = L_q.copy()
            c_old = self.c_coeffs[-1] if len(self.c_coeffs) > 0 else 1
            p_norm = self.s_norm[-1] / c_old
            a = dot(psi_p, L_q) * p_norm
            if np.isnan(a):
                raise ValueError("NaN in the Lanczos coefficients")
            rk = L_q - a * psi_q
            if len(self.basis_Q) > 1:
                rk -= self.c_coeffs[-1] * self.basis_Q[-2]
            sk = p_L - a * psi_p
            if len(self.basis_P) > 1:
                if len(self.c_coeffs) < 2:
                    old_p_norm = self.s_norm[-2]
                else:
                    old_p_norm = self.s_norm[-2] / self.c_coeffs[-2]
                sk -= self.b_coeffs[-1] * self.basis_P[-2] * (old_p_norm / p_norm)
            s_norm = np.sqrt(dot(sk, sk))
            sk_tilde = sk / s_norm
            s_norm *= p_norm
            b = np.sqrt(dot(rk, rk))
            c = dot(sk_tilde, rk / b) * s_norm
            self.a_coeffs.append(a)
            if abs(b) < EPS or abs(c) < EPS:
                break
            psi_q = rk / b
            psi_p = sk_tilde.copy()
            self.basis_Q.append(psi_q.copy())
            self.basis_P.append(psi_p.copy())
            self.b_coeffs.append(b)
            self.c_coeffs.append(c)
            self.s_norm.append(s_norm)
        return self.a_coeffs, self.b_coeffs, self.c_coeffs

    def get_green_function_continued_fraction(self, w_array, use_terminator=True,
                                              last_average=1, smearing=0.0, smooth_ramp=0):
        return continued_fraction(self.a_coeffs, self.b_coeffs, self.c_coeffs, w_array,
                                  self.use_wigner, self.perturbation_modulus,
                                  self.reverse_L, self.shift_value, use_terminator,
                                  last_average, smearing, smooth_ramp)


def continued_fraction(a_coeffs, b_coeffs, c_coeffs, w_array, use_wigner, modulus=1.0,
                       reverse_L=False, shift_value=0.0, use_terminator=True,
                       last_average=1, smearing=0.0, smooth_ramp=0):
    """G(w) by backward recurrence (DynamicalLanczos.py:5032-5162)."""
    n = len(a_coeffs)
    w_array = np.asarray(w_array, dtype=np.float64)
    gf = np.zeros(w_array.shape, dtype=np.complex128)
    sign = -1 if reverse_L else 1
    nonsym = len(c_coeffs) == len(b_coeffs)
    if use_terminator:
        a_av = np.mean(a_coeffs[-last_average:])
        b_av = np.mean(b_coeffs[-last_average:])
        c_av = np.mean(c_coeffs[-last_average:]) if nonsym else b_av
        a_m = a_av * sign - sign * shift_value
        b_m = b_av * sign
        c_m = c_av * sign
        d = a_m - w_array ** 2 if not use_wigner else a_m + w_array ** 2
        disc = d ** 2 - 4 * b_m * c_m
        sq = np.sqrt(disc + 0j)
        gp = (d + sq) / (2 * b_m * c_m)
        gm = (d - sq) / (2 * b_m * c_m)
        gf[:] = np.where(np.abs(gp) < np.abs(gm), gp, gm)
    else:
        a = a_coeffs[-1] * sign - sign * shift_value
        if not use_wigner:
            gf[:] = 1 / (a - w_array ** 2 + 2j * w_array * smearing)
        else:
            gf[:] = 1 / (a + w_array ** 2 + 2j * w_array * smearing)
    for i in range(n - 2, -1, -1):
        a = a_coeffs[i] * sign - sign * shift_value
        b = b_coeffs[i] * sign
        c = c_coeffs[i] * sign if nonsym else b
        if use_terminator and smooth_ramp > 0 and i >= n - smooth_ramp:
            al = (i - n + smooth_ramp + 1) / smooth_ramp
            a = (1 - al) * a + al * a_m
            b = (1 - al) * b + al * b_m
            c = (1 - al) * c + al * c_m
        if not use_wigner:
            gf = 1. / (a - w_array ** 2 + 2j * w_array * smearing - b * c * gf)
        else:
            gf = 1. / (a + w_array ** 2 + 2j * w_array * smearing - b * c * gf)
    if not use_wigner:
        return gf * modulus
    return (-np.real(gf) + 1j * np.imag(gf)) * modulus


# --- static response (free-energy Hessian) ----------------------------------
def static_lambda(w, T):
    """Pair factor Lambda of apply_L1_static (DynamicalLanczos.py:2588-2622), one
    value per upper-triangle pair (row i, column j): w_a = w[j], w_b = w[i];
    both population masks from w_a (:2603-2604); on w_a == w_b the derivative
    term multiplies n_equal^2, read before the occupations are set (:2608-2619)."""
    M = len(w)
    iu_r, iu_c = np.triu_indices(M)
    wa, wb = w[iu_c], w[iu_r]
    na = np.zeros_like(wa)
    nb = np.zeros_like(wa)
    unpop = 0.01 * wa * RY_TO_K > T
    equal = np.abs(wa - wb) < 1e-8
    diff = np.zeros_like(wa)
    if T > 0:
        beta = RY_TO_K / T
        na = 1 / (np.exp(wa * beta) - 1)
        nb = 1 / (np.exp(wb * beta) - 1)
        na[unpop] = 0
        nb[unpop] = 0
        with np.errstate(divide="ignore", invalid="ignore"):
            diff = (na - nb) / (wa - wb)
        diff[equal] = -beta * np.exp(wa[equal] * beta) * 0.0
    lam = (na + nb + 1) / (wa + wb) - diff
    return lam / (4 * wa * wb)


def static_L1(w, T, psi, inverse=False, power=1):
    """apply_L1_static (DynamicalLanczos.py:2562-2624)."""
    M = len(w)
    if inverse:
        power = -power
    out = np.zeros(len(psi))
    out[:M] = psi[:M] * w ** (2 * power)
    out[M:] = psi[M:] / static_lambda(w, T) ** power
    return out


def upsilon(w, T):
    n = np.zeros_like(w) if T <= 1e-12 else 1.0 / (np.exp(w * RY_TO_K / T) - 1.0)
    return 2 * w / (2 * n + 1)


def static_anharmonic(ol, psi):
    """apply_anharmonic_static (DynamicalLanczos.py:3369-3430) on an OracleLanczos:
    R1 = psi_R, Y1 = -2 Upsilon psi_W Upsilon, output [-f | d2v upper rows]."""
    M = ol.n_modes
    Y1 = ol._sym_from_triangle(psi[M:])
    Yw = upsilon(ol.w, ol.T)
    Y1 = -2 * np.einsum("ab, a, b -> ab", Y1, Yw, Yw)
    f, d2v = ol.perturb(np.ascontiguousarray(psi[:M]), np.ascontiguousarray(Y1))
    out = np.zeros(len(psi))
    out[:M] = -f
    out[M:] = d2v[ol.iu_row, ol.iu_col]
    return out


def minimum_residual(apply_A, b, x0, max_iters=100, conv_thr=1e-6):
    """The minimal-residual iteration of Tools.minimum_residual_algorithm
    (Modules/Tools.py:265-414) without preconditioner; returns (x, iterations,
    converged)."""
    r1 = b - apply_A(x0)
    b_norm = np.sqrt(b.dot(b))
    r1_bar = apply_A(r1)
    z1 = r1.copy()
    p1 = r1.copy()
    p1_bar = r1_bar.copy()
    x = x0.copy()
    iters, converged = 1, False
    while iters < max_iters and not converged:
        Ap = p1_bar
        Ap_bar = apply_A(p1_bar)
        alpha = r1_bar.dot(z1) / p1_bar.dot(Ap)
        x = x + alpha * p1
        r = r1 - alpha * Ap
        rbar = r1_bar - alpha * Ap_bar
        r_norm = np.sqrt(r.dot(r)) / b_norm
        beta = rbar.dot(r) / r1_bar.dot(z1)
        p1 = r + beta * p1
        p1_bar = rbar + beta * p1_bar
        r1, r1_bar, z1 = r, rbar, r
        converged = r_norm < conv_thr
        iters += 1
    return x, iters, converged


def run_hessian_calculation(ol, eigen_shift=1.0, max_iters=1000, use_preconditioning=True):
    """Lanczos.run_hessian_calculation with the 'cg' algorithm
    (DynamicalLanczos.py:4054-4330): one minimal-residual solve per unit vector,
    G_ij = x_i[j], returns inv((G + G^T) / 2)."""
    M = ol.n_modes
    Ps = M + M * (M + 1) // 2

    def L(psi):
        p = psi.copy()
        p[M:] *= eigen_shift
        ret = static_L1(ol.w, ol.T, p) + static_anharmonic(ol, p)
        ret[M:] *= eigen_shift
        return ret

    def P(x):
        return static_L1(ol.w, ol.T, x, inverse=True, power=0.5)

    G = np.zeros((M, M))
    for i in range(M):
        b = np.zeros(Ps)
        b[i] = 1
        if use_preconditioning:
            bt = P(b)
            xt, _, _ = minimum_residual(lambda x: P(L(P(x))), bt, bt.copy(), max_iters)
            res = P(xt)
        else:
            res, _, _ = minimum_residual(L, b, b.copy(), max_iters)
        G[i, :] = res[:M]
    G = 0.5 * (G + G.T)
    return np.linalg.inv(G)


# --- ensemble preprocessing and gamma_only -----------------------------------
def project_modes(u, f, masses, pols, f_mean=None, u_scale=1.0, f_scale=1.0):
    """X, Y of Lanczos.__init__ (DynamicalLanczos.py:392-452) from Cartesian data."""
    sq = np.sqrt(masses)
    uu = u * u_scale
    ff = f * f_scale
    if f_mean is not None:
        ff = ff - f_mean * f_scale
    return (uu * sq).dot(pols), (ff / sq).dot(pols)


def translation_projector(pols, perms):
    """trans_projector = mean_R pols^T P_R pols (DynamicalLanczos.py:764-785)."""
    return np.mean([pols.T @ pols[p, :] for p in perms], axis=0)


def translation_project(f, d2v, pols, perms):
    """gamma_only projection of the averages (DynamicalLanczos.py:3173-3191)."""
    f = translation_projector(pols, perms) @ f
    d2v_cart = pols @ d2v @ pols.T
    avg = np.zeros_like(d2v_cart)
    for p in perms:
        avg += d2v_cart[np.ix_(p, p)]
    avg /= len(perms)
    return f, pols.T @ avg @ pols
