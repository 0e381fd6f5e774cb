"""ORACLE -- test infrastructure only: q-space (Bloch basis) restatement.

numpy restatement of the reference's q-space perturbation averages
(`get_perturb_averages_qspace_fused`, Modules/tdscha_qspace.jl:455-628, entry
:639-712) and of the QSpaceLanczos operator and Hermitian Lanczos
(Modules/QSpaceLanczos.py: block layout :298-364, mask :494-535, L1 :537-580,
chi :599-651, alpha1 :653-707, apply_anharmonic_FT :730-773, run_FT
:967-1182).  Used by tests/ as the checker of the GPU q-space path.

Pinning: the reference's q-space kernel is Julia and cannot run here (no
Julia); with one q-point and real data the q-space operator reduces to the
real-space Wigner operator, and tests/test_oracle_qspace.py checks this
restatement against the reference's own real-space fixtures in that limit.
Beyond that limit the q-space parity is unpinned.

Ensemble layout as the reference: X_q, Y_q complex (n_q, N, n_bands); w_q,
valid (n_bands, n_q); symmetries: list of (n_q*n_bands)^2 complex matrices
(dense or scipy.sparse) acting on vectors indexed iq*n_bands + nu.
"""
import numpy as np

RY_TO_K = 157887.32400374097
EPS = 1e-12


def pair_layout(q_pair_map):
    """unique pairs (iq1 <= iq2) and the psi layout (QSpaceLanczos.py:298-364)."""
    n_q = len(q_pair_map)
    pairs = [(iq1, int(q_pair_map[iq1])) for iq1 in range(n_q) if iq1 <= q_pair_map[iq1]]
    return pairs


def perturb_averages_qspace(X_q, Y_q, w_q, rho, R1, alpha1_blocks, T, apply_v4, iq_pert,
                            pairs, symmetries=None, valid=None):
    """(f_pert[n_bands], [d2v blocks]) as get_perturb_averages_qspace returns them.

    The configuration loop of the reference is vectorised over configurations;
    the (symmetry, pair) structure and every formula follow tdscha_qspace.jl.
    """
    n_q, N, nb = X_q.shape
    if valid is None:
        valid = np.ones((nb, n_q), dtype=bool)
    fY = np.zeros((nb, n_q))
    fpsi = np.zeros((nb, n_q))
    for iq in range(n_q):
        for nu in range(nb):
            if not valid[nu, iq]:
                continue
            w = w_q[nu, iq]
            nw = 1.0 / (np.exp(w * RY_TO_K / T) - 1.0) if T > 0 else 0.0
            fY[nu, iq] = 2.0 * w / (1.0 + 2.0 * nw)
            fpsi[nu, iq] = (1.0 + 2.0 * nw) / (2.0 * w)
    if symmetries is None:
        symmetries = [None]
    S = len(symmetries)
    # rows: config-major, (N, n_q*nb)
    xb = np.ascontiguousarray(np.transpose(X_q, (1, 0, 2)).reshape(N, n_q * nb))
    yb = np.ascontiguousarray(np.transpose(Y_q, (1, 0, 2)).reshape(N, n_q * nb))
    f_pert = np.zeros(nb, dtype=np.complex128)
    d2v = [np.zeros((nb, nb), dtype=np.complex128) for _ in pairs]
    N_eff = np.sum(rho)
    sl = lambda iq: slice(iq * nb, (iq + 1) * nb)
    for sym in symmetries:
        if sym is None:
            xr, yr = xb, yb
        else:
            Sm = sym.toarray() if hasattr(sym, "toarray") else np.asarray(sym)
            xr = xb @ Sm.T
            yr = yb @ Sm.T
        xp, yp = xr[:, sl(iq_pert)], yr[:, sl(iq_pert)]
        weight_R = (xp * fY[:, iq_pert] * np.conj(R1)).sum(1) * rho / 3.0
        weight_Rf = (np.conj(R1) * yp).sum(1) * rho / 3.0
        buf_u = np.zeros((N, n_q, nb), dtype=np.complex128)
        total = np.zeros(N, dtype=np.complex128)
        for p, (iq1, iq2) in enumerate(pairs):
            a = alpha1_blocks[p]
            x1, x2 = xr[:, sl(iq1)], xr[:, sl(iq2)]
            buf_u[:, iq1, :] += x2 @ a.T
            if iq1 != iq2:
                buf_u[:, iq2, :] += x1 @ np.conj(a)
            lw = np.einsum("ri,ij,rj->r", np.conj(x1), a, x2)
            total += (lw + np.conj(lw)) if iq1 < iq2 else lw
        g = yr.reshape(N, n_q, nb) * fpsi.T[None, :, :]
        bfw = (np.conj(buf_u) * g).sum((1, 2))
        w1 = -total / 2.0 * rho / 3.0
        w2 = -bfw * rho / 3.0
        f_pert += (w1[:, None] * yp).sum(0) + (w2[:, None] * fY[:, iq_pert] * xp).sum(0)
        wD4 = -total * rho / 8.0 if apply_v4 else 0.0
        wb = -bfw * rho / 4.0 if apply_v4 else 0.0
        w_cross = weight_R + wD4
        w_diag = weight_Rf + wb
        for p, (iq1, iq2) in enumerate(pairs):
            r1_1 = fY[:, iq1] * xr[:, sl(iq1)]
            r2_1 = yr[:, sl(iq1)]
            r1_2 = fY[:, iq2] * xr[:, sl(iq2)]
            r2_2 = yr[:, sl(iq2)]
            d2v[p] -= np.einsum("r,ri,rj->ij", w_cross, r1_1, np.conj(r2_2))
            d2v[p] -= np.einsum("r,ri,rj->ij", w_cross, r2_1, np.conj(r1_2))
            d2v[p] -= np.einsum("r,ri,rj->ij", w_diag, r1_1, np.conj(r1_2))
    norm = S * N_eff
    return f_pert / norm, [b / norm for b in d2v]


class OracleQSpaceLanczos:
    """numpy restatement of QSpaceLanczos on the fast path (Wigner only)."""

    def __init__(self, X_q, Y_q, w_q, rho, T, q_pair_map, iq_pert, symmetries=None,
                 valid=None, apply_d4=True, ignore_v3=False, ignore_harmonic=False):
        self.X_q, self.Y_q = np.asarray(X_q), np.asarray(Y_q)
        self.n_q, self.N, self.nb = self.X_q.shape
        self.w_q = np.asarray(w_q, dtype=np.float64)
        self.rho = np.asarray(rho, dtype=np.float64)
        self.T = float(T)
        self.symmetries = symmetries
        self.valid = np.ones((self.nb, self.n_q), dtype=bool) if valid is None else np.asarray(valid)
        self.ignore_v4 = not apply_d4
        self.ignore_v3 = ignore_v3
        self.ignore_harmonic = ignore_harmonic
        self.iq_pert = iq_pert
        self.q_pair_map = np.asarray(q_pair_map)
        self.pairs = pair_layout(self.q_pair_map)
        nb = self.nb
        self.sizes = [nb * nb if a < b else nb * (nb + 1) // 2 for a, b in self.pairs]
        self.off_a, off = [], nb
        for s in self.sizes:
            self.off_a.append(off)
            off += s
        self.off_b = []
        for s in self.sizes:
            self.off_b.append(off)
            off += s
        self.P = off
        self.psi = np.zeros(self.P, dtype=np.complex128)
        self.a_coeffs, self.b_coeffs, self.c_coeffs = [], [], []
        self.basis_Q, self.basis_P, self.s_norm = [], [], []
        self.perturbation_modulus = 1.0

    # layout helpers (QSpaceLanczos.py:402-491)
    def _unpack(self, flat, n):
        m = np.zeros((n, n), dtype=np.complex128)
        idx = 0
        for i in range(n):
            m[i, i:] = flat[idx:idx + n - i]
            idx += n - i
        for i in range(n):
            m[i + 1:, i] = np.conj(m[i, i + 1:])
        return m

    def _pack(self, mat, n):
        return np.concatenate([mat[i, i:] for i in range(n)])

    def get_block(self, p, sector, src):
        iq1, iq2 = self.pairs[p]
        off = self.off_a[p] if sector == "a" else self.off_b[p]
        raw = src[off:off + self.sizes[p]]
        return raw.reshape(self.nb, self.nb).copy() if iq1 < iq2 else self._unpack(raw, self.nb)

    def set_block(self, p, mat, sector, dst):
        iq1, iq2 = self.pairs[p]
        off = self.off_a[p] if sector == "a" else self.off_b[p]
        dst[off:off + self.sizes[p]] = mat.ravel() if iq1 < iq2 else self._pack(mat, self.nb)

    def mask_dot_wigner(self):
        mask = np.ones(self.P)
        nb = self.nb
        for p, (iq1, iq2) in enumerate(self.pairs):
            for off in (self.off_a[p], self.off_b[p]):
                if iq1 < iq2:
                    mask[off:off + self.sizes[p]] = 2
                else:
                    idx = off
                    for i in range(nb):
                        mask[idx] = 1
                        idx += 1
                        for _ in range(i + 1, nb):
                            mask[idx] = 2
                            idx += 1
        return mask

    def _bose(self, iq):
        w = self.w_q[:, iq]
        v = self.valid[:, iq]
        n = np.zeros_like(w)
        if self.T > EPS:
            n[v] = 1.0 / (np.exp(w[v] * RY_TO_K / self.T) - 1.0)
        return n, v

    def _pair_mats(self, iq1, iq2):
        w1, w2 = self.w_q[:, iq1], self.w_q[:, iq2]
        n1, v1 = self._bose(iq1)
        n2, v2 = self._bose(iq2)
        vm = np.outer(v1, v2)
        nb = self.nb
        w1m, w2m = np.tile(w1, (nb, 1)).T, np.tile(w2, (nb, 1))
        n1m, n2m = np.tile(n1, (nb, 1)).T, np.tile(n2, (nb, 1))
        den = 2.0 * w1m * w2m
        cm = np.where(vm, (w1m - w2m) * (n1m - n2m) / np.where(vm, den, 1.0), 0.0)
        cp = np.where(vm, (w1m + w2m) * (1 + n1m + n2m) / np.where(vm, den, 1.0), 0.0)
        X = (1 + 2 * n1m) * (1 + 2 * n2m) / 8
        w2X = np.where(vm, (w1m * w2m) / np.where(vm, X, 1.0), 0.0)
        return w1, w2, vm, cm, cp, w2X

    def apply_L1_FT(self, psi):
        out = np.zeros(self.P, dtype=np.complex128)
        if self.ignore_harmonic:
            return out
        nb = self.nb
        wqp = self.w_q[:, self.iq_pert]
        out[:nb] = -(wqp ** 2) * psi[:nb]
        out[:nb] *= self.valid[:, self.iq_pert]
        for p, (iq1, iq2) in enumerate(self.pairs):
            w1, w2 = self.w_q[:, iq1], self.w_q[:, iq2]
            vm = np.outer(self.valid[:, iq1], self.valid[:, iq2])
            a = self.get_block(p, "a", psi)
            b = self.get_block(p, "b", psi)
            self.set_block(p, -np.subtract.outer(w1, w2) ** 2 * a * vm, "a", out)
            self.set_block(p, -np.add.outer(w1, w2) ** 2 * b * vm, "b", out)
        return out

    def alpha1_blocks(self, psi):
        blocks = []
        for p, (iq1, iq2) in enumerate(self.pairs):
            _, _, vm, cm, cp, w2X = self._pair_mats(iq1, iq2)
            a = self.get_block(p, "a", psi)
            b = self.get_block(p, "b", psi)
            blocks.append(w2X * np.sqrt(-0.5 * cm) * a - w2X * np.sqrt(+0.5 * cp) * b)
        return blocks

    def apply_anharmonic_FT(self, psi):
        if self.ignore_v3 and self.ignore_v4:
            return np.zeros(self.P, dtype=np.complex128)
        R1 = psi[:self.nb].copy()
        if self.ignore_v3:
            R1[:] = 0
        f, d2v = perturb_averages_qspace(self.X_q, self.Y_q, self.w_q, self.rho, R1,
                                         self.alpha1_blocks(psi), self.T, not self.ignore_v4,
                                         self.iq_pert, self.pairs, self.symmetries, self.valid)
        out = np.zeros(self.P, dtype=np.complex128)
        out[:self.nb] = f
        for p, (iq1, iq2) in enumerate(self.pairs):
            _, _, _, cm, cp, _ = self._pair_mats(iq1, iq2)
            self.set_block(p, np.sqrt(-0.5 * cm) * d2v[p], "a", out)
            self.set_block(p, -np.sqrt(+0.5 * cp) * d2v[p], "b", out)
        return out

    def apply_full_L(self, psi):
        return self.apply_L1_FT(psi) + self.apply_anharmonic_FT(psi)

    def run_FT(self, n_iter, reorthogonalize=True):
        """Hermitian Lanczos (QSpaceLanczos.py:967-1182)."""
        mask = self.mask_dot_wigner()
        dot = lambda x, y: np.real(np.conj(x).dot(y * mask))
        if len(self.a_coeffs) == 0:
            first = self.psi / np.sqrt(dot(self.psi, self.psi))
            self.basis_Q, self.basis_P, self.s_norm = [first], [first], [1]
        psi_q, psi_p = self.basis_Q[-1], self.basis_P[-1]
        for _ in range(n_iter):
            L_q = self.apply_full_L(psi_q)
            p_L = L_q.copy()
            c_old = self.c_coeffs[-1] if self.c_coeffs else 1
            p_norm = self.s_norm[-1] / c_old
            a = dot(psi_p, L_q) * p_norm
            rk = L_q - a * psi_q
            if len(self.basis_Q) > 1:
                rk -= self.c_coeffs[-1] * self.basis_Q[-2]
            sk = p_L - a * psi_p
            if len(self.basis_P) > 1:
                old = self.s_norm[-2]
                if len(self.c_coeffs) >= 2:
                    old = self.s_norm[-2] / self.c_coeffs[-2]
                sk -= self.b_coeffs[-1] * self.basis_P[-2] * (old / p_norm)
            s_norm = np.sqrt(dot(sk, sk))
            sk_t = sk / s_norm
            s_norm *= p_norm
            b = np.sqrt(dot(rk, rk))
            c = dot(sk_t, rk / b) * s_norm
            self.a_coeffs.append(a)
            if abs(b) < EPS or abs(c) < EPS:
                break
            psi_q = rk / b
            psi_p = sk_t.copy()
            if reorthogonalize:
                nq = psi_q.copy()
                for qj in self.basis_Q:
                    nq -= dot(qj, nq) * qj
                nq /= np.sqrt(dot(nq, nq))
                new_q, new_p, s_norm = nq, nq.copy(), c
            else:
                new_q, new_p = psi_q.copy(), psi_p.copy()
            self.basis_Q.append(new_q)
            self.basis_P.append(new_p)
            psi_q, psi_p = new_q.copy(), new_p.copy()
            self.b_coeffs.append(b)
            self.c_coeffs.append(c)
            self.s_norm.append(s_norm)
        return self.a_coeffs, self.b_coeffs, self.c_coeffs


def q_pair_map_grid(q_crys, iq_pert, tol=1e-6):
    """iq2 with q1 + q2 = q_pert (mod reciprocal lattice), crystal coordinates."""
    q = np.asarray(q_crys, dtype=np.float64)
    out = np.zeros(len(q), dtype=np.int32)
    for i in range(len(q)):
        t = q[iq_pert] - q[i]
        d = q - t
        d -= np.round(d)
        j = np.where(np.abs(d).max(1) < tol)[0]
        if len(j) == 0:
            raise ValueError("no partner for q-point %d" % i)
        out[i] = j[0]
    return out


# --- kernel polynomial method (Modules/QSpaceKPM.py) -------------------------
def kpm_bounds(w_q, valid, bound_factor=1.2, edge_buffer=1e-8, use_wigner=True):
    """_get_kpm_bounds without explicit bounds (QSpaceKPM.py:156-176)."""
    max_w = np.max(np.abs(np.asarray(w_q)[np.asarray(valid, dtype=bool)]))
    width = (2 * max_w) ** 2
    margin = (bound_factor - 1) * width
    lmin, lmax = (-width - margin, margin) if use_wigner else (-margin, width + margin)
    span = lmax - lmin
    return lmin - edge_buffer * span, lmax + edge_buffer * span


def kpm_moments(apply_L, psi, mask, n_moments, lmin, lmax):
    """run_KPM's fresh path (QSpaceKPM.py:377-440): returns (moments, norm, vm, v)."""
    dot = lambda x, y: np.real(np.conj(x).dot(y * mask))
    a = 0.5 * (lmax - lmin)
    b = 0.5 * (lmax + lmin)
    resc = lambda v: (apply_L(v) - b * v) / a
    norm = np.sqrt(dot(psi, psi))
    v0 = psi / norm
    mom = np.zeros(n_moments)
    mom[0] = 1.0
    vm, v = v0, v0
    if n_moments > 1:
        v1 = resc(v0)
        mom[1] = dot(v0, v1)
        vm, v = v0, v1
        n = 1
        while 2 * n < n_moments:
            mom[2 * n] = 2 * dot(v, v) - mom[0]
            if 2 * n + 1 >= n_moments:
                break
            vp = 2 * resc(v) - vm
            mom[2 * n + 1] = 2 * dot(vp, v) - mom[1]
            vm, v = v, vp
            n += 1
    return mom, norm, vm, v


def jackson_kernel(n_moments):
    """QSpaceKPM._jackson_kernel (:516-519)."""
    n = np.arange(n_moments, dtype=np.float64)
    phi = np.pi / (n_moments + 1)
    return ((n_moments - n + 1) * np.cos(n * phi) + np.sin(n * phi) / np.tan(phi)) / (n_moments + 1)


def kpm_spectral(w_array, moments, norm, lmin, lmax, g=None, use_wigner=True):
    """get_spectral_function_KPM (QSpaceKPM.py:536-559)."""
    n_m = len(moments)
    g = jackson_kernel(n_m) if g is None else g
    a = 0.5 * (lmax - lmin)
    b = 0.5 * (lmax + lmin)
    w = np.asarray(w_array, dtype=np.float64)
    lam = -(w ** 2) if use_wigner else w ** 2
    x = (lam - b) / a
    inside = np.abs(x) < 1
    out = np.zeros_like(w)
    if not np.any(inside):
        return out
    xin = np.clip(x[inside], -1 + 1e-15, 1 - 1e-15)
    t0 = np.ones_like(xin)
    rho = g[0] * moments[0] * t0
    if n_m > 1:
        t1 = xin.copy()
        rho += 2 * g[1] * moments[1] * t1
        for i in range(2, n_m):
            t2 = 2 * xin * t1 - t0
            rho += 2 * g[i] * moments[i] * t2
            t0, t1 = t1, t2
    rho /= np.pi * a * np.sqrt(1 - xin ** 2)
    rho *= norm ** 2
    out[inside] = np.pi * rho
    return out


def moments_from_tridiagonal(a_c, b_c, c_c, n_moments, lmin, lmax):
    """Chebyshev moments e0^T T_n((T - b)/a) e0 of the Lanczos tridiagonal
    (diagonal a_k, T[k+1,k] = b_k, T[k,k+1] = c_k): equal to the KPM moments of
    the start vector for n < 2 (number of steps) + 1 in exact arithmetic."""
    k = len(a_c)
    T = np.diag(np.asarray(a_c, dtype=np.float64))
    for i in range(k - 1):
        T[i + 1, i] = b_c[i]
        T[i, i + 1] = c_c[i]
    a = 0.5 * (lmax - lmin)
    b = 0.5 * (lmax + lmin)
    Ts = (T - b * np.eye(k)) / a
    e0 = np.zeros(k)
    e0[0] = 1
    mom = np.zeros(n_moments)
    t_prev, t_cur = e0, Ts @ e0
    mom[0] = 1.0
    if n_moments > 1:
        mom[1] = t_cur[0]
    for n in range(2, n_moments):
        t_next = 2 * Ts @ t_cur - t_prev
        mom[n] = t_next[0]
        t_prev, t_cur = t_cur, t_next
    return mom
