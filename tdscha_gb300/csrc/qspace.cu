// q-space (Bloch basis) perturbation averages and operator, float64 complex.
//
// Restates get_perturb_averages_qspace_fused (Modules/tdscha_qspace.jl:455-628,
// entry :639-712) and the QSpaceLanczos operator (Modules/QSpaceLanczos.py:
// layout :298-364, mask :494-535, L1 :537-580, chi :599-651, alpha1 :653-707,
// apply_anharmonic_FT :730-773) on the GPU.  For image row r (configuration
// i, symmetry j): x = S_j x_i, y = S_j y_i over all (q, band) pairs;
//   u[q]   = A_q x[partner(q)]       (A_q = alpha_p, or alpha_p^H for the second
//                                      member of pair p)
//   total  = x^H u                    q of the real-space path
//   bfw    = u^H (f_psi * y)          p
//   wR     = sum f_Y x[q_pert] conj(R1),  wRf = sum conj(R1) y[q_pert]
//   f      = sum_r w1_r y[q_pert] + w2_r f_Y x[q_pert]
//   d2v_p  = -sum_r w_cross (u1 f2^H + f1 u2^H) + w_diag u1 u2^H
// with u = f_Y x, f = y on the two q-points of pair p.  Complex numbers are
// double2 (re, im), interleaved in every host and device array.
#include <cmath>
#include <vector>

#include "common.cuh"



namespace tdscha {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {   // a * conj(b)
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// acc + a b and acc + conj(a) b as four explicit FMAs each
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
    return acc;
}
__device__ __forceinline__ double2 cfma_conj(double2 a, double2 b, double2 acc) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
    return acc;
}

// The same complex helpers on float2: the mixed-precision operator does its
// arithmetic in fp32 on the CUDA cores (see q_perturb).
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 acc) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
    return acc;
}
__device__ __forceinline__ float2 cfma_conj(float2 a, float2 b, float2 acc) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
    return acc;
}
template <typename T2> struct CReal;
template <> struct CReal<double2> { using type = double; };
template <> struct CReal<float2> { using type = float; };
template <typename T2> __device__ __forceinline__ T2 czero() { T2 z; z.x = 0; z.y = 0; return z; }
__device__ __forceinline__ double2 to_d2(double2 a) { return a; }
__device__ __forceinline__ double2 to_d2(float2 a) { return make_double2(a.x, a.y); }

// float copies for the mixed-precision operator
__global__ void k_q_to32(const double *__restrict__ a, long n, float *__restrict__ b) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        b[e] = (float)a[e];
}

// x_rot = S_j x_i for every image row, S_j in CSR (identity when n_syms == 0).
// bad = 1 if any of the n entries of a or b is not finite
__global__ void k_q_finite(const double *__restrict__ a, const double *__restrict__ b, long n,
                           int *__restrict__ bad) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        if (!isfinite(a[e]) || !isfinite(b[e])) *bad = 1;
}

__global__ void k_q_expand(const double2 *__restrict__ X, const double2 *__restrict__ Y, int N,
                           int n_q, int nb, int S, int has_syms, const int *__restrict__ rowptr,
                           const int *__restrict__ col, const double2 *__restrict__ val,
                           double2 *__restrict__ Xr, double2 *__restrict__ Yr) {
    const int L = n_q * nb;
    long total = (long)N * S * L;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e % L);
        long r = e / L;
        int i = (int)(r / S), j = (int)(r % S);
        // source element (q, nu) = a of configuration i: X is [q][config][nu]
        double2 xs = make_double2(0, 0), ys = make_double2(0, 0);
        if (!has_syms) {
            int q = a / nb, nu = a % nb;
            xs = X[((long)q * N + i) * nb + nu];
            ys = Y[((long)q * N + i) * nb + nu];
        } else {
            const int *rp = rowptr + (long)j * (L + 1);
            for (int t = rp[a]; t < rp[a + 1]; ++t) {
                int b = col[t];
                int q = b / nb, nu = b % nb;
                double2 v = val[t];
                xs = cadd(xs, cmul(v, X[((long)q * N + i) * nb + nu]));
                ys = cadd(ys, cmul(v, Y[((long)q * N + i) * nb + nu]));
            }
        }
        Xr[e] = xs;
        Yr[e] = ys;
    }
}

// alpha1 blocks from psi (Wigner change of variables per pair element).
// pcoef layout per pair element: [0] -(w1-w2)^2 vm, [1] -(w1+w2)^2 vm,
// [2] w2X sqrt(-chi-/2), [3] w2X sqrt(chi+/2), [4] sqrt(-chi-/2), [5] -sqrt(chi+/2)
__device__ __forceinline__ long q_store(int p, int i, int j, int nb, int full, const long *off) {
    if (full) return off[p] + (long)i * nb + j;
    // upper triangle rows from the diagonal, i <= j
    return off[p] + (long)i * nb - (long)i * (i - 1) / 2 + (j - i);
}

__global__ void k_q_unpack(const double2 *__restrict__ psi, const int *__restrict__ pair_q,
                           const long *__restrict__ off_a, const long *__restrict__ off_b,
                           const double *__restrict__ pcoef, int n_pairs, int nb,
                           int ignore_v3, double2 *__restrict__ R1, double2 *__restrict__ alpha) {
    long n = (long)n_pairs * nb * nb;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int p = (int)(e / (nb * nb));
        int i = (int)((e / nb) % nb), j = (int)(e % nb);
        int full = pair_q[2 * p] < pair_q[2 * p + 1];
        double2 a, b;
        if (full || i <= j) {
            a = psi[q_store(p, i, j, nb, full, off_a)];
            b = psi[q_store(p, i, j, nb, full, off_b)];
        } else {   // lower triangle of a Hermitian block
            a = cconj(psi[q_store(p, j, i, nb, 0, off_a)]);
            b = cconj(psi[q_store(p, j, i, nb, 0, off_b)]);
        }
        const double *c = pcoef + e * 6;
        alpha[e] = make_double2(c[2] * a.x - c[3] * b.x, c[2] * a.y - c[3] * b.y);
        if (e < nb) R1[e] = ignore_v3 ? make_double2(0, 0) : psi[e];
    }
}

// Per image row: q-space row scalars.  A block of 256 threads takes
// rows_per_block rows; the lw = 256 / rows_per_block threads of a row stride
// over its n_q nb entries and reduce through warp shuffles + shared memory.
// One row per block when n_q nb >= 128 (the grid is then many waves deep).
inline int q_rows_per_block(int L) {
    int lw = std::min(256, ((L + 31) / 32) * 32);
    return 256 / lw;
}
// T2 = double2: float64 throughout (the reference's precision); T2 = float2:
// fp32 products and per-row sums (24 significant bits), the block sums and the
// row weights in float64, written to rowc as T2.
template <typename T2>
__global__ void __launch_bounds__(256, 4) k_q_rows(
        const T2 *__restrict__ Xr, const T2 *__restrict__ Yr,
        const typename CReal<T2>::type *__restrict__ fY,
        const typename CReal<T2>::type *__restrict__ fpsi,
        const double *__restrict__ rho, const T2 *__restrict__ R1,
        const T2 *__restrict__ alpha, const int *__restrict__ qpair,
        const int *__restrict__ qrole, const int *__restrict__ qpartner,
        int n_q, int nb, int S, long R, int iq_pert, int apply_d4, int rpb,
        T2 *__restrict__ rowc) {
    using T = typename CReal<T2>::type;
    __shared__ double red[8][8];   // per warp: tot, bfw, wR, wRf (re, im)
    const int lw = blockDim.x / rpb;
    const int g = threadIdx.x / lw, t = threadIdx.x % lw;
    long r = (long)blockIdx.x * rpb + g;
    const bool live = r < R;
    const int L = n_q * nb;
    T2 tot = czero<T2>(), bfw = czero<T2>();
    T2 wR = czero<T2>(), wRf = czero<T2>();
    if (live) {
        const T2 *x = Xr + r * L, *y = Yr + r * L;
        for (int a = t; a < L; a += lw) {
            int q = a / nb, nu = a - q * nb;
            int p = qpair[q], role = qrole[q], q2 = qpartner[q];
            const T2 *blk = alpha + (long)p * nb * nb;
            const T2 *xp = x + q2 * nb;
            T2 u = czero<T2>(), u2 = czero<T2>();
            // role 0: alpha[nu][k]; role 1: conj(alpha[k][nu])
            if (role == 0) {
                const T2 *ar = blk + nu * nb;
                int k = 0;
                for (; k + 1 < nb; k += 2) {
                    u = cfma(ar[k], xp[k], u);
                    u2 = cfma(ar[k + 1], xp[k + 1], u2);
                }
                if (k < nb) u = cfma(ar[k], xp[k], u);
            } else {
                int k = 0;
                for (; k + 1 < nb; k += 2) {
                    u = cfma_conj(blk[k * nb + nu], xp[k], u);
                    u2 = cfma_conj(blk[(k + 1) * nb + nu], xp[k + 1], u2);
                }
                if (k < nb) u = cfma_conj(blk[k * nb + nu], xp[k], u);
            }
            u = cadd(u, u2);
            tot = cfma_conj(x[a], u, tot);                        // conj(x) u
            bfw = cfma_conj(u, cscale(y[a], fpsi[a]), bfw);       // conj(u) g
        }
        for (int nu = t; nu < nb; nu += lw) {
            int a = iq_pert * nb + nu;
            wR = cadd(wR, cmulc(cscale(x[a], fY[a]), R1[nu]));    // fY x conj(R1)
            wRf = cadd(wRf, cmulc(y[a], R1[nu]));                   // conj(R1) y
        }
    }
    T v[8] = {tot.x, tot.y, bfw.x, bfw.y, wR.x, wR.y, wRf.x, wRf.y};
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 8; ++k) red[wid][k] = v[k];
    __syncthreads();
    if (live && t == 0) {
        // the warps of this row: lw / 32 consecutive warps starting at its first
        const int w0 = (g * lw) >> 5, nw = lw >> 5;
        double s[8];
        for (int k = 0; k < 8; ++k) {
            s[k] = 0;
            for (int w = 0; w < nw; ++w) s[k] += red[w0 + w][k];
        }
        double2 dtot = make_double2(s[0], s[1]);
        double2 dbfw = make_double2(s[2], s[3]);
        double2 dwR = make_double2(s[4], s[5]);
        double2 dwRf = make_double2(s[6], s[7]);
        double rw = rho[r / S];
        double d4 = apply_d4 ? 1.0 : 0.0;
        double2 w[4] = {cscale(dtot, -0.5 * rw / 3.0), cscale(dbfw, -rw / 3.0),
                        cadd(cscale(dwR, rw / 3.0), cscale(dtot, -d4 * rw / 8.0)),
                        cadd(cscale(dwRf, rw / 3.0), cscale(dbfw, -d4 * rw / 4.0))};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            rowc[4 * r + k].x = (T)w[k].x;
            rowc[4 * r + k].y = (T)w[k].y;
        }
    }
}

// f partials: fpart[chunk][nu] = sum_r w1 y[q_pert][nu] + w2 f_Y x[q_pert][nu]
template <typename T2>
__global__ void k_q_favg(const T2 *__restrict__ Xr, const T2 *__restrict__ Yr,
                         const typename CReal<T2>::type *__restrict__ fY,
                         const T2 *__restrict__ rowc, int L, int nb, int iq_pert, long R,
                         long chunk, double2 *__restrict__ fpart) {
    using T = typename CReal<T2>::type;
    __shared__ double sh[2][32];
    int nu = blockIdx.x;
    long rb = (long)blockIdx.y * chunk, re = min(R, rb + chunk);
    int a = iq_pert * nb + nu;
    T fy = fY[a];
    T2 acc = czero<T2>();
    for (long r = rb + threadIdx.x; r < re; r += blockDim.x) {
        acc = cadd(acc, cmul(rowc[4 * r], Yr[r * L + a]));
        acc = cadd(acc, cmul(rowc[4 * r + 1], cscale(Xr[r * L + a], fy)));
    }
    double2 dacc = to_d2(acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dacc.x += __shfl_xor_sync(0xffffffffu, dacc.x, o);
        dacc.y += __shfl_xor_sync(0xffffffffu, dacc.y, o);
    }
    if ((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = dacc.x; sh[1][threadIdx.x >> 5] = dacc.y; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 s = make_double2(0, 0);
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s.x += sh[0][w]; s.y += sh[1][w]; }
        fpart[(long)blockIdx.y * nb + nu] = s;
    }
}

// d2v partials per pair: block (pair, chunk).  Rows are staged kQRows at a
// time as A1 = -w_cross u1, A2 = -(w_cross f1 + w_diag u1), conj(f2), conj(u2),
// so every block element takes two complex FMAs per row:
//   d2v_ij += A1_i conj(f2_j) + A2_i conj(u2_j)
// Thread t owns element t % nbb for the rows of phase t / nbb (blocks with
// nbb <= blockDim / 2 run several phases), phases summed in a fixed order.
constexpr int kQRows = 16;   // rows staged in shared memory per pass
inline int q_d2v_threads(int nb) {
    int nbb = nb * nb;
    return nbb <= 128 ? 256 : ((nbb + 31) / 32) * 32;
}
template <typename T2>
__global__ void k_q_d2v(const T2 *__restrict__ Xr, const T2 *__restrict__ Yr,
                        const typename CReal<T2>::type *__restrict__ fY,
                        const T2 *__restrict__ rowc, const int *__restrict__ pair_q, int L, int nb,
                        long R, long chunk, int n_pairs, double2 *__restrict__ dpart) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T2 *sm = reinterpret_cast<T2 *>(sm_raw);   // kQRows x 4 nb, reused for the phase sum
    const int p = blockIdx.x;
    const int q1 = pair_q[2 * p], q2 = pair_q[2 * p + 1];
    const int stride = 4 * nb;
    const int nbb = nb * nb;
    const int nph = max(1, (int)blockDim.x / nbb);
    const int e = threadIdx.x % nbb, ph = threadIdx.x / nbb;
    const bool active = ph < nph && (int)threadIdx.x < nph * nbb;
    const int i = e / nb, j = e % nb;
    long rb = (long)blockIdx.y * chunk, re = min(R, rb + chunk);
    // two accumulators (the A1 and A2 products) to shorten the FMA chains
    T2 acc = czero<T2>(), acc2 = czero<T2>();
    for (long r0 = rb; r0 < re; r0 += kQRows) {
        int nr = (int)min((long)kQRows, re - r0);
        __syncthreads();
        for (int t = threadIdx.x; t < nr * 2 * nb; t += blockDim.x) {
            int rr = t / (2 * nb), c = t % (2 * nb);
            long r = r0 + rr;
            T2 *s = sm + rr * stride;
            if (c < nb) {
                T2 x1 = Xr[r * L + q1 * nb + c], f1 = Yr[r * L + q1 * nb + c];
                T2 u1 = cscale(x1, fY[q1 * nb + c]);
                T2 wc = rowc[4 * r + 2], wd = rowc[4 * r + 3];
                T2 a1 = cmul(wc, u1);
                T2 a2 = cadd(cmul(wc, f1), cmul(wd, u1));
                s[c] = cscale(a1, -1);
                s[nb + c] = cscale(a2, -1);
            } else {
                int cc = c - nb;
                T2 x2 = Xr[r * L + q2 * nb + cc], f2 = Yr[r * L + q2 * nb + cc];
                s[2 * nb + cc] = cconj(f2);
                s[3 * nb + cc] = cconj(cscale(x2, fY[q2 * nb + cc]));
            }
        }
        __syncthreads();
        if (active) {
            for (int rr = ph; rr < nr; rr += nph) {
                const T2 *s = sm + rr * stride;
                T2 a1 = s[i], a2 = s[nb + i], cf = s[2 * nb + j], cu = s[3 * nb + j];
                acc = cfma(a1, cf, acc);
                acc2 = cfma(a2, cu, acc2);
            }
        }
    }
    double2 dacc = cadd(to_d2(acc), to_d2(acc2));
    __syncthreads();
    double2 *smd = reinterpret_cast<double2 *>(sm_raw);
    if (nph > 1) {
        if (active) smd[threadIdx.x] = dacc;
        __syncthreads();
        if (ph == 0 && active) {
            for (int k = 1; k < nph; ++k) dacc = cadd(dacc, smd[k * nbb + e]);
        }
    }
    if (ph == 0 && active) dpart[((long)blockIdx.y * n_pairs + p) * nbb + e] = dacc;
}

__global__ void k_q_finalize(const double2 *__restrict__ fpart, int nfchunk,
                             const double2 *__restrict__ dpart, int nbchunk, int nb, int n_pairs,
                             double inv_norm, double2 *__restrict__ f, double2 *__restrict__ d2v) {
    long n = (long)n_pairs * nb * nb;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        double2 s = make_double2(0, 0);
        for (int c = 0; c < nbchunk; ++c) s = cadd(s, dpart[(long)c * n + e]);
        d2v[e] = cscale(s, inv_norm);
        if (e < nb) {
            double2 t = make_double2(0, 0);
            for (int c = 0; c < nfchunk; ++c) t = cadd(t, fpart[(long)c * nb + e]);
            f[e] = cscale(t, inv_norm);
        }
    }
}

// psi' = L1 psi + anharmonic repack (q-space Wigner operator, no sign flip).
// elem[e]: sector (0 R, 1 a', 2 b') << 28 | pair << 16 | nu1 << 8 | nu2
__global__ void k_q_assemble(const double2 *__restrict__ psi, const double2 *__restrict__ f,
                             const double2 *__restrict__ d2v, const int *__restrict__ elem,
                             const double *__restrict__ pcoef, const double *__restrict__ wpert,
                             long P, int nb, int with_harm, int with_anh,
                             double2 *__restrict__ out) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < P; e += (long)gridDim.x * blockDim.x) {
        int code = elem[e];
        int sector = code >> 28, p = (code >> 16) & 0xfff, i = (code >> 8) & 0xff, j = code & 0xff;
        double2 v = psi[e], o = make_double2(0, 0);
        if (sector == 0) {
            if (with_harm) o = cscale(v, wpert[i]);                // -(w^2) valid
            if (with_anh) o = cadd(o, f[i]);
        } else {
            long be = ((long)p * nb + i) * nb + j;
            const double *c = pcoef + be * 6;
            if (with_harm) o = cscale(v, sector == 1 ? c[0] : c[1]);
            if (with_anh) o = cadd(o, cscale(d2v[be], sector == 1 ? c[4] : c[5]));
        }
        out[e] = o;
    }
}

static int q_build_layout(tdscha_qctx *c, const int *q_pair_map) {
    const int n_q = c->n_q, nb = c->nb;
    std::vector<int> pq;      // pair q1, q2
    std::vector<int> qpair(n_q, -1), qrole(n_q, 0), qpartner(n_q, 0);
    for (int q1 = 0; q1 < n_q; ++q1) {
        int q2 = q_pair_map[q1];
        if (q2 < 0 || q2 >= n_q || q_pair_map[q2] != q1) {
            set_error("qspace: q_pair_map is not an involution at q=%d", q1);
            return TDSCHA_ERR_ARG;
        }
        if (q1 <= q2) {
            int p = (int)pq.size() / 2;
            pq.push_back(q1);
            pq.push_back(q2);
            qpair[q1] = p; qrole[q1] = 0; qpartner[q1] = q2;
            if (q2 != q1) { qpair[q2] = p; qrole[q2] = 1; qpartner[q2] = q1; }
        }
    }
    const int n_pairs = (int)pq.size() / 2;
    if (n_pairs >= 4096 || nb > 255) { set_error("qspace: too many pairs or bands"); return TDSCHA_ERR_ARG; }
    std::vector<long> size(n_pairs), off_a(n_pairs), off_b(n_pairs);
    long off = nb;
    for (int p = 0; p < n_pairs; ++p) {
        size[p] = pq[2 * p] < pq[2 * p + 1] ? (long)nb * nb : (long)nb * (nb + 1) / 2;
        off_a[p] = off;
        off += size[p];
    }
    for (int p = 0; p < n_pairs; ++p) { off_b[p] = off; off += size[p]; }
    const long P = off;
    std::vector<int> elem(P);
    std::vector<double> mask(2 * P, 1.0);
    for (int i = 0; i < nb; ++i) elem[i] = i << 8;
    for (int s = 1; s <= 2; ++s) {
        for (int p = 0; p < n_pairs; ++p) {
            long o = s == 1 ? off_a[p] : off_b[p];
            bool full = pq[2 * p] < pq[2 * p + 1];
            for (int i = 0; i < nb; ++i)
                for (int j = full ? 0 : i; j < nb; ++j, ++o) {
                    elem[o] = (s << 28) | (p << 16) | (i << 8) | j;
                    double m = (full || i != j) ? 2.0 : 1.0;
                    mask[2 * o] = mask[2 * o + 1] = m;
                }
        }
    }
    // per pair element coefficients (QSpaceLanczos.py:537-707)
    const double T = c->T;
    auto bose = [&](int iq, int nu, bool &v) {
        v = c->valid[nu * n_q + iq] != 0;
        if (!v || !(T > kEps)) return 0.0;
        return 1.0 / (exp(c->w_q[nu * n_q + iq] * kRyToK / T) - 1.0);
    };
    std::vector<double> pc((size_t)n_pairs * nb * nb * 6);
    for (int p = 0; p < n_pairs; ++p) {
        int q1 = pq[2 * p], q2 = pq[2 * p + 1];
        for (int i = 0; i < nb; ++i)
            for (int j = 0; j < nb; ++j) {
                bool v1, v2;
                double n1 = bose(q1, i, v1), n2 = bose(q2, j, v2);
                double w1 = c->w_q[i * n_q + q1], w2 = c->w_q[j * n_q + q2];
                bool vm = v1 && v2;
                double den = 2.0 * w1 * w2;
                double cm = vm ? (w1 - w2) * (n1 - n2) / den : 0.0;
                double cp = vm ? (w1 + w2) * (1 + n1 + n2) / den : 0.0;
                double X = (1 + 2 * n1) * (1 + 2 * n2) / 8;
                double w2X = vm ? (w1 * w2) / X : 0.0;
                double *o = &pc[(((size_t)p * nb + i) * nb + j) * 6];
                o[0] = vm ? -((w1 - w2) * (w1 - w2)) : 0.0;
                o[1] = vm ? -((w1 + w2) * (w1 + w2)) : 0.0;
                o[2] = w2X * sqrt(-0.5 * cm);
                o[3] = w2X * sqrt(+0.5 * cp);
                o[4] = sqrt(-0.5 * cm);
                o[5] = -sqrt(+0.5 * cp);
            }
    }
    std::vector<double> wpert(nb);
    for (int i = 0; i < nb; ++i) {
        double w = c->w_q[i * n_q + c->iq_pert];
        wpert[i] = c->valid[i * n_q + c->iq_pert] ? -(w * w) : 0.0;
    }
    // upload
    auto up = [&](auto **dst, const auto &src) -> int {
        if (*dst) cudaFree(*dst);
        *dst = nullptr;
        TDS_CUDA(cudaMalloc((void **)dst, sizeof(src[0]) * std::max<size_t>(1, src.size())));
        TDS_CUDA(cudaMemcpy(*dst, src.data(), sizeof(src[0]) * src.size(), cudaMemcpyHostToDevice));
        return TDSCHA_OK;
    };
    TDS_TRY(up(&c->qpair, qpair));
    TDS_TRY(up(&c->qrole, qrole));
    TDS_TRY(up(&c->qpartner, qpartner));
    TDS_TRY(up(&c->pair_q, pq));
    TDS_TRY(up(&c->elem, elem));
    TDS_TRY(up(&c->pcoef, pc));
    TDS_TRY(up(&c->mask, mask));
    std::vector<long> offs(2 * n_pairs + 1);
    for (int p = 0; p < n_pairs; ++p) { offs[p] = off_a[p]; offs[n_pairs + p] = off_b[p]; }
    offs[2 * n_pairs] = 0;
    TDS_TRY(up(&c->q_off, offs));
    c->n_pairs = n_pairs;
    c->P = P;
    // scratch sized by the layout
    double2 **bufs2[] = {&c->alpha, &c->d2v, &c->dpart};
    for (double2 **b : bufs2)
        if (*b) { cudaFree(*b); *b = nullptr; }
    TDS_CUDA(cudaMalloc(&c->alpha, sizeof(double2) * (size_t)n_pairs * nb * nb));
    if (c->alpha32) { cudaFree(c->alpha32); c->alpha32 = nullptr; }
    if (c->precision == TDSCHA_PREC_MIXED)
        TDS_CUDA(cudaMalloc(&c->alpha32, sizeof(float2) * (size_t)n_pairs * nb * nb));
    TDS_CUDA(cudaMalloc(&c->d2v, sizeof(double2) * (size_t)n_pairs * nb * nb));
    // d2v split over configurations: about four waves of eight blocks per SM
    // over all pairs (a short last wave), at least 64 image rows per block
    c->nbchunk = (int)std::max<long>(1, std::min<long>((152L * 8 * 4 + n_pairs - 1) / n_pairs,
                                                       (c->R + 63) / 64));
    TDS_CUDA(cudaMalloc(&c->dpart, sizeof(double2) * (size_t)c->nbchunk * n_pairs * nb * nb));
    double **bufs[] = {&c->Lq, &c->rk, &c->sk};
    for (double **b : bufs) {
        if (*b) cudaFree(*b);
        TDS_CUDA(cudaMalloc(b, sizeof(double) * 2 * P));
    }
    TDS_TRY(up(&c->wpert, wpert));
    return TDSCHA_OK;
}

}  // namespace tdscha

namespace tdscha {

// perturbation averages into c->f, c->d2v from c->R1, c->alpha.  Float64, or
// with precision mixed the row, force and d2v kernels in fp32 on the CUDA
// cores over float copies of the image rows (their partial sums and the
// finalisation stay float64).  The q-pair blocks are n_b x n_b with K = N*S:
// a 128-row tensor-core tile would compute mostly unused blocks (the row
// products are block diagonal with K = n_b), while GB300's fp32 pipe runs at
// about 64 times its float64 rate.
template <typename T2>
static int q_perturb_t(tdscha_qctx *c, int apply_d4, const T2 *Xr, const T2 *Yr,
                       const typename CReal<T2>::type *fY, const typename CReal<T2>::type *fpsi,
                       const T2 *R1, const T2 *alpha, T2 *rowc, cudaStream_t st) {
    const int nb = c->nb, L = c->L;
    const long R = c->R;
    const int rpb = q_rows_per_block(L);
    k_q_rows<T2><<<ceil_div(R, rpb), 256, 0, st>>>(Xr, Yr, fY, fpsi, c->rho, R1, alpha, c->qpair,
                                                    c->qrole, c->qpartner, c->n_q, nb, c->S, R,
                                                    c->iq_pert, apply_d4, rpb, rowc);
    TDS_CHECK_LAUNCH();
    long fchunk = (R + c->nfchunk - 1) / c->nfchunk;
    k_q_favg<T2><<<dim3(nb, c->nfchunk), 256, 0, st>>>(Xr, Yr, fY, rowc, L, nb, c->iq_pert, R,
                                                       fchunk, c->fpart);
    TDS_CHECK_LAUNCH();
    long bchunk = (R + c->nbchunk - 1) / c->nbchunk;
    const int dthreads = q_d2v_threads(nb);
    size_t smem = sizeof(double2) * std::max(kQRows * 4 * nb, dthreads);
    k_q_d2v<T2><<<dim3(c->n_pairs, c->nbchunk), dthreads, smem, st>>>(
        Xr, Yr, fY, rowc, c->pair_q, L, nb, R, bchunk, c->n_pairs, c->dpart);
    TDS_CHECK_LAUNCH();
    long n = (long)c->n_pairs * nb * nb;
    k_q_finalize<<<std::max(1, std::min(ceil_div(n, 256), 1024)), 256, 0, st>>>(
        c->fpart, c->nfchunk, c->dpart, c->nbchunk, nb, c->n_pairs, 1.0 / (c->sum_rho * c->S),
        c->f, c->d2v);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

static int q_perturb(tdscha_qctx *c, int apply_d4, cudaStream_t st) {
    if (c->precision != TDSCHA_PREC_MIXED)
        return q_perturb_t<double2>(c, apply_d4, c->Xr, c->Yr, c->fY, c->fpsi, c->R1, c->alpha,
                                    c->rowc, st);
    const long na = 2L * c->n_pairs * c->nb * c->nb, nr = 2L * c->nb;
    k_q_to32<<<std::max(1, std::min(ceil_div(na, 256), 256)), 256, 0, st>>>(
        reinterpret_cast<const double *>(c->alpha), na, reinterpret_cast<float *>(c->alpha32));
    TDS_CHECK_LAUNCH();
    k_q_to32<<<1, 64, 0, st>>>(reinterpret_cast<const double *>(c->R1), nr,
                               reinterpret_cast<float *>(c->R1_32));
    TDS_CHECK_LAUNCH();
    return q_perturb_t<float2>(c, apply_d4, c->Xr32, c->Yr32, c->fY32, c->fpsi32, c->R1_32,
                               c->alpha32, c->rowc32, st);
}

int q_apply_full_L_dev(tdscha_qctx *c, const double *psi_in, double *psi_out, cudaStream_t st) {
    const int nb = c->nb;
    const double2 *psi = reinterpret_cast<const double2 *>(psi_in);
    int with_anh = !(c->ignore_v3 && c->ignore_v4);
    if (with_anh) {
        long n = (long)c->n_pairs * nb * nb;
        k_q_unpack<<<std::max(1, std::min(ceil_div(n, 256), 1024)), 256, 0, st>>>(
            psi, c->pair_q, c->q_off, c->q_off + c->n_pairs, c->pcoef, c->n_pairs, nb, c->ignore_v3,
            c->R1, c->alpha);
        TDS_CHECK_LAUNCH();
        TDS_TRY(q_perturb(c, c->ignore_v4 ? 0 : 1, st));
    }
    k_q_assemble<<<std::max(1, std::min(ceil_div(c->P, 256), 4096)), 256, 0, st>>>(
        psi, c->f, c->d2v, c->elem, c->pcoef, c->wpert, c->P, nb, !c->ignore_harmonic, with_anh,
        reinterpret_cast<double2 *>(psi_out));
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

static void q_free(tdscha_qctx *c) {
    if (!c) return;
    void *bufs[] = {c->Xr, c->Yr, c->fY, c->fpsi, c->rho, c->qpair, c->qrole, c->qpartner,
                    c->pair_q, c->elem, c->pcoef, c->mask, c->q_off, c->wpert, c->R1, c->alpha,
                    c->f, c->d2v, c->rowc, c->fpart, c->dpart, c->Lq, c->rk, c->sk, c->dots,
                    c->scal, c->hist_dev, c->stat_dev, c->pqn, c->rcoef, c->Xr32, c->Yr32,
                    c->fY32, c->fpsi32, c->R1_32, c->alpha32, c->rowc32};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (c->stat_host) cudaFreeHost(c->stat_host);
    delete c;
}

}  // namespace tdscha

using namespace tdscha;

extern "C" int tdscha_qctx_create(tdscha_qctx **out, int n_q, int nb, int N, const double *X_q,
                                  const double *Y_q, const double *w_q, const int *valid,
                                  const double *rho, double T, int n_syms, const int *sym_rowptr,
                                  const int *sym_col, const double *sym_val) {
    set_error("");
    if (!out) { set_error("qctx_create: null output pointer"); return TDSCHA_ERR_ARG; }
    *out = nullptr;
    if (n_q <= 0 || nb <= 0 || nb > 32 || N <= 0 || n_syms < 0) {
        set_error("qctx_create: bad sizes n_q=%d nb=%d (1..32) N=%d n_syms=%d", n_q, nb, N, n_syms);
        return TDSCHA_ERR_ARG;
    }
    if (!X_q || !Y_q || !w_q || !rho || (n_syms > 0 && (!sym_rowptr || !sym_col || !sym_val))) {
        set_error("qctx_create: null input pointer");
        return TDSCHA_ERR_ARG;
    }
    if (!(T >= 0) || !std::isfinite(T)) { set_error("qctx_create: bad temperature %g", T); return TDSCHA_ERR_ARG; }
    const int L = n_q * nb;
    long nnz = 0;
    if (n_syms > 0) {
        for (int j = 0; j < n_syms; ++j) {
            const int *rp = sym_rowptr + (long)j * (L + 1);
            for (int a = 0; a < L; ++a)
                if (rp[a + 1] < rp[a]) { set_error("qctx_create: symmetry %d row pointers decrease", j); return TDSCHA_ERR_ARG; }
            nnz = std::max<long>(nnz, rp[L]);
            if (rp[0] < 0) { set_error("qctx_create: negative row pointer"); return TDSCHA_ERR_ARG; }
        }
        for (long t = 0; t < nnz; ++t)
            if (sym_col[t] < 0 || sym_col[t] >= L) { set_error("qctx_create: symmetry column %ld out of range", t); return TDSCHA_ERR_ARG; }
    }
    // X_q and Y_q are checked for non-finite entries on the device after the upload
    double sum_rho = 0;
    for (int i = 0; i < N; ++i) sum_rho += rho[i];
    if (!(sum_rho != 0) || !std::isfinite(sum_rho)) { set_error("qctx_create: bad weights"); return TDSCHA_ERR_ARG; }
    tdscha_qctx *c = new tdscha_qctx();
    c->n_q = n_q; c->nb = nb; c->N = N; c->S = n_syms > 0 ? n_syms : 1;
    c->R = (long)N * c->S; c->L = L; c->T = T; c->sum_rho = sum_rho;
    c->w_q.assign(w_q, w_q + (size_t)nb * n_q);
    c->valid.assign((size_t)nb * n_q, 1);
    if (valid)
        for (size_t k = 0; k < c->valid.size(); ++k) c->valid[k] = valid[k] != 0;
    for (size_t k = 0; k < c->valid.size(); ++k)
        if (c->valid[k] && !(c->w_q[k] > 0)) { q_free(c); set_error("qctx_create: valid mode with w <= 0"); return TDSCHA_ERR_ARG; }
    std::vector<double> fy((size_t)L, 0.0), fp((size_t)L, 0.0);
    for (int q = 0; q < n_q; ++q)
        for (int nu = 0; nu < nb; ++nu) {
            if (!c->valid[nu * n_q + q]) continue;
            double w = c->w_q[nu * n_q + q];
            double nw = T > 0 ? 1.0 / (exp(w * kRyToK / T) - 1.0) : 0.0;
            fy[q * nb + nu] = 2.0 * w / (1.0 + 2.0 * nw);
            fp[q * nb + nu] = (1.0 + 2.0 * nw) / (2.0 * w);
        }
    double2 *dX = nullptr, *dY = nullptr, *dval = nullptr;
    int *drp = nullptr, *dcol = nullptr, *dbad = nullptr;
    auto fail = [&](int code) { if (dX) cudaFree(dX); if (dY) cudaFree(dY); if (dval) cudaFree(dval); if (drp) cudaFree(drp); if (dcol) cudaFree(dcol); if (dbad) cudaFree(dbad); q_free(c); return code; };
#define QCU(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { set_error("%s: %s", #x, cudaGetErrorString(_e)); return fail(TDSCHA_ERR_CUDA); } } while (0)
    size_t nX = (size_t)n_q * N * nb;
    QCU(cudaMalloc(&dX, sizeof(double2) * nX));
    QCU(cudaMalloc(&dY, sizeof(double2) * nX));
    QCU(cudaMemcpy(dX, X_q, sizeof(double2) * nX, cudaMemcpyHostToDevice));
    QCU(cudaMemcpy(dY, Y_q, sizeof(double2) * nX, cudaMemcpyHostToDevice));
    {
        int hbad = 0;
        QCU(cudaMalloc(&dbad, sizeof(int)));
        QCU(cudaMemset(dbad, 0, sizeof(int)));
        long n = 2 * (long)nX;
        k_q_finite<<<(int)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 16)), 256>>>(
            reinterpret_cast<const double *>(dX), reinterpret_cast<const double *>(dY), n, dbad);
        QCU(cudaGetLastError());
        QCU(cudaMemcpy(&hbad, dbad, sizeof(int), cudaMemcpyDeviceToHost));
        cudaFree(dbad);
        dbad = nullptr;
        if (hbad) { set_error("qctx_create: non-finite X_q/Y_q"); return fail(TDSCHA_ERR_NAN); }
    }
    if (n_syms > 0) {
        QCU(cudaMalloc(&drp, sizeof(int) * (size_t)n_syms * (L + 1)));
        QCU(cudaMalloc(&dcol, sizeof(int) * std::max<long>(1, nnz)));
        QCU(cudaMalloc(&dval, sizeof(double2) * std::max<long>(1, nnz)));
        QCU(cudaMemcpy(drp, sym_rowptr, sizeof(int) * (size_t)n_syms * (L + 1), cudaMemcpyHostToDevice));
        if (nnz) {
            QCU(cudaMemcpy(dcol, sym_col, sizeof(int) * nnz, cudaMemcpyHostToDevice));
            QCU(cudaMemcpy(dval, sym_val, sizeof(double2) * nnz, cudaMemcpyHostToDevice));
        }
    }
    QCU(cudaMalloc(&c->Xr, sizeof(double2) * (size_t)c->R * L));
    QCU(cudaMalloc(&c->Yr, sizeof(double2) * (size_t)c->R * L));
    {
        long total = c->R * L;
        int blocks = (int)std::min<long>((total + 255) / 256, 152L * 16);
        k_q_expand<<<std::max(1, blocks), 256>>>(dX, dY, N, n_q, nb, c->S, n_syms > 0, drp, dcol, dval,
                                                  c->Xr, c->Yr);
        QCU(cudaGetLastError());
        QCU(cudaDeviceSynchronize());
    }
    cudaFree(dX); cudaFree(dY); dX = dY = nullptr;
    if (drp) { cudaFree(drp); cudaFree(dcol); cudaFree(dval); drp = dcol = nullptr; dval = nullptr; }
    QCU(cudaMalloc(&c->fY, sizeof(double) * L));
    QCU(cudaMalloc(&c->fpsi, sizeof(double) * L));
    QCU(cudaMalloc(&c->rho, sizeof(double) * N));
    QCU(cudaMemcpy(c->fY, fy.data(), sizeof(double) * L, cudaMemcpyHostToDevice));
    QCU(cudaMemcpy(c->fpsi, fp.data(), sizeof(double) * L, cudaMemcpyHostToDevice));
    QCU(cudaMemcpy(c->rho, rho, sizeof(double) * N, cudaMemcpyHostToDevice));
    c->nfchunk = (int)std::min<long>(std::max<long>(1, c->R / 1024), 256);
    QCU(cudaMalloc(&c->R1, sizeof(double2) * nb));
    QCU(cudaMalloc(&c->f, sizeof(double2) * nb));
    QCU(cudaMalloc(&c->rowc, sizeof(double2) * 4 * (size_t)c->R));
    QCU(cudaMalloc(&c->fpart, sizeof(double2) * (size_t)c->nfchunk * nb));
    QCU(cudaMalloc(&c->dots, sizeof(double) * 4 * 296));
    QCU(cudaMalloc(&c->scal, sizeof(double) * 64));
#undef QCU
    *out = c;
    return TDSCHA_OK;
}

extern "C" int tdscha_qctx_destroy(tdscha_qctx *ctx) {
    if (!ctx) return TDSCHA_OK;
    cudaDeviceSynchronize();
    q_free(ctx);
    return TDSCHA_OK;
}

extern "C" int tdscha_qctx_set_pert(tdscha_qctx *ctx, int iq_pert, const int *q_pair_map,
                                    int ignore_harmonic, int ignore_v3, int ignore_v4,
                                    long *psi_size, int *n_pairs) {
    set_error("");
    if (!ctx || !q_pair_map) { set_error("qctx_set_pert: null pointer"); return TDSCHA_ERR_ARG; }
    if (iq_pert < 0 || iq_pert >= ctx->n_q) { set_error("qctx_set_pert: iq_pert %d out of range", iq_pert); return TDSCHA_ERR_ARG; }
    ctx->iq_pert = iq_pert;
    ctx->ignore_harmonic = ignore_harmonic != 0;
    ctx->ignore_v3 = ignore_v3 != 0;
    ctx->ignore_v4 = ignore_v4 != 0;
    TDS_TRY(q_build_layout(ctx, q_pair_map));
    if (psi_size) *psi_size = ctx->P;
    if (n_pairs) *n_pairs = ctx->n_pairs;
    return TDSCHA_OK;
}

extern "C" int tdscha_qperturb_averages(tdscha_qctx *ctx, const double *R1, const double *alpha1,
                                        int apply_d4, double *f_out, double *d2v_out,
                                        int device_ptrs, void *stream) {
    set_error("");
    if (!ctx || !R1 || !alpha1 || !f_out || !d2v_out) { set_error("qperturb_averages: null pointer"); return TDSCHA_ERR_ARG; }
    if (ctx->n_pairs == 0) { set_error("qperturb_averages: call tdscha_qctx_set_pert first"); return TDSCHA_ERR_STATE; }
    if (apply_d4 != 0 && apply_d4 != 1) { set_error("qperturb_averages: apply_d4 must be 0 or 1"); return TDSCHA_ERR_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    const int nb = ctx->nb;
    size_t nbl = (size_t)ctx->n_pairs * nb * nb;
    cudaMemcpyKind in = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaMemcpyKind outk = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    TDS_CUDA(cudaMemcpyAsync(ctx->R1, R1, sizeof(double2) * nb, in, st));
    TDS_CUDA(cudaMemcpyAsync(ctx->alpha, alpha1, sizeof(double2) * nbl, in, st));
    TDS_TRY(q_perturb(ctx, apply_d4, st));
    TDS_CUDA(cudaMemcpyAsync(f_out, ctx->f, sizeof(double2) * nb, outk, st));
    TDS_CUDA(cudaMemcpyAsync(d2v_out, ctx->d2v, sizeof(double2) * nbl, outk, st));
    if (!device_ptrs) TDS_CUDA(cudaStreamSynchronize(st));
    return TDSCHA_OK;
}

extern "C" int tdscha_qapply_full_L(tdscha_qctx *ctx, const double *psi_in, double *psi_out,
                                    void *stream) {
    set_error("");
    if (!ctx || !psi_in || !psi_out || psi_in == psi_out) { set_error("qapply_full_L: bad pointers"); return TDSCHA_ERR_ARG; }
    if (ctx->n_pairs == 0) { set_error("qapply_full_L: call tdscha_qctx_set_pert first"); return TDSCHA_ERR_STATE; }
    return q_apply_full_L_dev(ctx, psi_in, psi_out, (cudaStream_t)stream);
}

extern "C" int tdscha_qctx_set_precision(tdscha_qctx *ctx, int precision) {
    set_error("");
    if (!ctx) { set_error("qctx_set_precision: null context"); return TDSCHA_ERR_ARG; }
    if (precision != TDSCHA_PREC_FP64 && precision != TDSCHA_PREC_MIXED) {
        set_error("qctx_set_precision: unknown precision %d", precision);
        return TDSCHA_ERR_ARG;
    }
    if (precision == TDSCHA_PREC_MIXED && !ctx->Xr32) {
        const long n = ctx->R * (long)ctx->L * 2, nm = (long)ctx->L;
        TDS_CUDA(cudaMalloc(&ctx->Xr32, sizeof(float) * n));
        TDS_CUDA(cudaMalloc(&ctx->Yr32, sizeof(float) * n));
        TDS_CUDA(cudaMalloc(&ctx->fY32, sizeof(float) * nm));
        TDS_CUDA(cudaMalloc(&ctx->fpsi32, sizeof(float) * nm));
        TDS_CUDA(cudaMalloc(&ctx->R1_32, sizeof(float2) * (size_t)ctx->nb));
        TDS_CUDA(cudaMalloc(&ctx->rowc32, sizeof(float2) * 4 * (size_t)ctx->R));
        const int g = (int)std::min<long>(ceil_div(n, 256), 152L * 16);
        k_q_to32<<<g, 256>>>(reinterpret_cast<const double *>(ctx->Xr), n,
                             reinterpret_cast<float *>(ctx->Xr32));
        k_q_to32<<<g, 256>>>(reinterpret_cast<const double *>(ctx->Yr), n,
                             reinterpret_cast<float *>(ctx->Yr32));
        k_q_to32<<<ceil_div(nm, 256), 256>>>(ctx->fY, nm, ctx->fY32);
        k_q_to32<<<ceil_div(nm, 256), 256>>>(ctx->fpsi, nm, ctx->fpsi32);
        TDS_CUDA(cudaGetLastError());
        TDS_CUDA(cudaDeviceSynchronize());
    }
    if (precision == TDSCHA_PREC_MIXED && ctx->n_pairs > 0 && !ctx->alpha32)
        TDS_CUDA(cudaMalloc(&ctx->alpha32, sizeof(float2) * (size_t)ctx->n_pairs * ctx->nb *
                                               ctx->nb));
    ctx->precision = precision;
    return TDSCHA_OK;
}
