// The operator around the perturbation averages and the Krylov driver on the
// GPU (float64 vectors and recurrence scalars; the re-biorthogonalisation
// sweeps of the real-space recurrence in double-float, dfloat.cuh):
//   * psi -> (R1, Y1) unpack: get_Y1 / get_ReA1 / get_alpha1_beta1_wigner
//     and the transpose rescaling (Modules/DynamicalLanczos.py:2773-2948,
//     :3009-3053);
//   * psi' = L1 psi + anharmonic repack + reverse/shift: apply_L1_FT
//     (:2287-2445), the repack of apply_anharmonic_FT (:3281-3363) and
//     apply_full_L (:3549-3651), fused in one elementwise kernel;
//   * the bi-/symmetric Lanczos recurrence of run_FT (:5958-6497) with
//     deterministic block-partial dot products;
//   * the continued fraction (:5032-5162), one thread per frequency.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"

namespace tdscha {

// per-pair coefficient arrays inside ctx->pc (each of length H)
enum { PC_X = 0, PC_Y, PC_X1, PC_Y1, PC_UA, PC_UB, PC_RA, PC_RB, PC_TY, PC_TRA, PC_I, PC_J };

int run_perturb(tdscha_ctx *c, int apply_d4, int precision, cudaStream_t st);
int run_perturb_sym(tdscha_ctx *c, int apply_d4, int precision, cudaStream_t st);

__device__ __forceinline__ long tri_index(int i, int j, int M) {
    return (long)i * M - (long)i * (i - 1) / 2 + (j - i);
}

// Per-pair coefficient arrays, the ψ-layout index tables and the Wigner mask,
// one thread per mode pair (i <= j, row i over blockIdx.y).  Per-mode inputs
// (w, the two Bose-factor forms, f_Y and the ReA weight) come from the host.
__global__ void k_pair_coeffs(const double *__restrict__ w, const double *__restrict__ bdiv,
                              const double *__restrict__ bmul, const double *__restrict__ yw,
                              const double *__restrict__ reaw, int M, long H, int wigner,
                              double *__restrict__ pc, int *__restrict__ tri,
                              double *__restrict__ mask) {
    for (int i = blockIdx.y; i < M; i += gridDim.y)
    for (int j = i + blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x) {
        const long k = tri_index(i, j, M);
        const double wa = w[j], wb = w[i];          // i_a = column, i_b = row (:2338-2346)
        const double na = bdiv[j], nbb = bdiv[i];
        const double den = (2 * na + 1) * (2 * nbb + 1);
        if (!wigner) {
            double X_ab = -wa * wa - wb * wb - (2 * wa * wb) / den;
            double Y_ab = -(8 * wa * wb) / den;
            double X1_ab = -(2 * na * nbb + na + nbb) * (2 * na * nbb + na + nbb + 1) * (2 * wa * wb) / den;
            double Y1_ab = -wa * wa - wb * wb + (2 * wa * wb) / den;
            pc[PC_X * H + k] = -X_ab;
            pc[PC_Y * H + k] = -Y_ab;
            pc[PC_X1 * H + k] = -X1_ab;
            pc[PC_Y1 * H + k] = -Y1_ab;
        } else {
            pc[PC_X * H + k] = -(wa * wa + wb * wb - 2. * wa * wb);
            pc[PC_Y * H + k] = 0.0;
            pc[PC_X1 * H + k] = 0.0;
            pc[PC_Y1 * H + k] = -(wa * wa + wb * wb + 2. * wa * wb);
        }
        // Wigner change of variables a', b' -> alpha (:2818-2839)
        const double Xf = ((1 + 2 * na) * (1 + 2 * nbb) / 8);
        const double w2_on_X = (wa * wb) / Xf;
        const double chi_m = ((wa - wb) * (na - nbb)) / (2 * wa * wb);
        const double chi_p = ((wa + wb) * (1 + na + nbb)) / (2 * wa * wb);
        pc[PC_UA * H + k] = w2_on_X * sqrt(-0.5 * chi_m);
        pc[PC_UB * H + k] = w2_on_X * sqrt(+0.5 * chi_p);
        // repack factors from get_chi_minus / get_chi_plus (row i, column j)
        const double ni = bmul[i], nj = bmul[j];
        const double cm = ((w[j] - w[i]) * (nj - ni)) / ((2. * w[j]) * w[i]);
        const double cp = ((w[j] + w[i]) * (1 + nj + ni)) / ((2. * w[j]) * w[i]);
        pc[PC_RA * H + k] = sqrt(-0.5 * cm);
        pc[PC_RB * H + k] = -sqrt(+0.5 * cp);
        // transpose rescaling coefficients (:3036-3050), [a=i][b=j], times the
        // half weight of an off-diagonal pair (exact: a power of two), so the
        // unpack multiplies each entry once
        const double cY = yw[i] * yw[j] * yw[j] + yw[i] * yw[i] * yw[j];
        const double cRA = yw[i] * reaw[j] * yw[j] + yw[i] * reaw[i] * yw[j];
        const double h = (i != j) ? 0.5 : 1.0;
        pc[PC_TY * H + k] = (cY * 2) * h;
        pc[PC_TRA * H + k] = (cRA * 2) * h;
        pc[PC_I * H + k] = i;
        pc[PC_J * H + k] = j;
        tri[2 * k] = i;
        tri[2 * k + 1] = j;
        // Wigner double-counting mask (mask_dot_wigner, :5905-5954)
        const double m = (i < j) ? 2.0 : 1.0;
        mask[M + k] = m;
        mask[M + H + k] = m;
        if (i == 0) mask[j] = 1.0;
    }
}

int build_pair_coeffs(tdscha_ctx *c) {
    const int M = c->M;
    const long H = c->H;
    std::vector<double> w(M);
    TDS_CUDA(cudaMemcpy(w.data(), c->w, sizeof(double) * M, cudaMemcpyDeviceToHost));
    const double T = c->T;
    // Bose factors as apply_L1_FT writes them (division form, :2363-2366)
    auto nb_div = [&](double x) { return T > 0 ? 1 / (exp(x / (T / kRyToK)) - 1) : 0.0; };
    // and as get_chi_minus/plus write them (multiplication form, :2650-2652)
    auto nb_mul = [&](double x) { return T > kEps ? 1.0 / (exp(x * 157887.32400374097 / T) - 1.0) : 0.0; };
    // per-mode inputs of the pair kernel: [bdiv | bmul | yw | reaw], and 1 / yw
    std::vector<double> pm(4 * (size_t)M), ywinv(M);
    for (int m = 0; m < M; ++m) {
        double n_mu = T > kEps ? 1.0 / (exp(w[m] * 157887.32400374097 / T) - 1.0) : 0.0;
        double yw = 2 * w[m] / (2 * n_mu + 1);
        pm[m] = nb_div(w[m]);
        pm[M + m] = nb_mul(w[m]);
        pm[2 * M + m] = yw;
        pm[3 * M + m] = 2 * w[m] * n_mu * (n_mu + 1) / (2 * n_mu + 1);
        ywinv[m] = 1.0 / yw;
    }
    if (!c->tri) TDS_CUDA(cached_malloc(&c->tri, sizeof(int) * 2 * H));
    if (!c->Ywinv) TDS_CUDA(cached_malloc(&c->Ywinv, sizeof(double) * M));
    // the per-mode inputs go through the 4 M doubles past the 12 H coefficients
    double *d_pm = c->pc + 12 * H;
    TDS_CUDA(cudaMemcpy(d_pm, pm.data(), sizeof(double) * 4 * M, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemcpy(c->Ywinv, ywinv.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    dim3 g(ceil_div(M, 128), std::min(M, 65535));
    k_pair_coeffs<<<g, 128>>>(c->w, d_pm, d_pm + M, d_pm + 2 * M, d_pm + 3 * M, M, H,
                              c->use_wigner, c->pc, c->tri, c->mask);
    TDS_CHECK_LAUNCH();
    TDS_CUDA(cudaDeviceSynchronize());
    c->pc_wigner = c->use_wigner;
    return TDSCHA_OK;
}


__global__ void k_unpack(const double *__restrict__ psi, const double *__restrict__ pc, int M,
                         long H, int wigner, int transpose, int ignore_v3,
                         double *__restrict__ R1, double *__restrict__ Y1) {
    pdl_enter();
    // rows a over blockIdx.y, columns b over the x dimension: no 64-bit
    // division per element
    for (int a = blockIdx.y; a < M; a += gridDim.y)
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < M; b += gridDim.x * blockDim.x) {
        const long e = (long)a * M + b;
        int i = min(a, b), j = max(a, b);
        long k = tri_index(i, j, M);
        double y = psi[M + k], ra = psi[M + H + k], v;
        if (wigner) {
            v = pc[PC_UA * H + k] * y - pc[PC_UB * H + k] * ra;
        } else if (!transpose) {
            v = y;
        } else {
            v = y * pc[PC_TY * H + k] + ra * pc[PC_TRA * H + k];
        }
        Y1[e] = v;
        if (a == 0) R1[b] = ignore_v3 ? 0.0 : psi[b];
    }
}

// out = L1 psi (+ anharmonic repack of f, d2v) then reverse / shift.  One
// thread per mode (the first M entries) or per pair k, which writes both its
// Y entry M + k and its A entry M + H + k: the two share the psi, tri and d2v
// loads, and with the layout (plain, transposed, Wigner) and the reversal as
// template arguments the float64 pipe sees only the products and sums (this
// part runs float64 at two FMA per cycle per SM).  Sign flips are folded into
// the operand order of the final sum.
enum { ASM_PLAIN = 0, ASM_TRANSPOSE = 1, ASM_WIGNER = 2 };

template <bool kRev>
__device__ __forceinline__ double asm_out(double l1, double an_pos, bool minus_an) {
    // o = l1 + (minus_an ? -an_pos : an_pos), negated when reversing
    if (!minus_an) return kRev ? (-l1) - an_pos : l1 + an_pos;
    return kRev ? an_pos - l1 : l1 - an_pos;
}

template <int kMode, bool kRev>
__device__ __forceinline__ void assemble_body(const double *__restrict__ psi, const double *__restrict__ f,
                           const double *__restrict__ d2v, const double *__restrict__ pc,
                           const int *__restrict__ tri, const double *__restrict__ w,
                           const double *__restrict__ Yw, const double *__restrict__ Ywinv,
                           const double *__restrict__ ReAw, int M, long H, int ignore_harmonic,
                           int with_anh, double shift, double *__restrict__ out) {
    constexpr bool kW = kMode == ASM_WIGNER;
    const bool harm = !ignore_harmonic, anh = with_anh != 0, sh = shift != 0.0;
    const long n = M + H;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        if (t < M) {
            const double p = psi[t];
            const double hm = harm ? (p * w[t]) * w[t] : 0.0;
            const double fa = anh ? f[t] : 0.0;
            // plain / transposed: o = hm - f; Wigner: o = -hm + f
            double o = kW ? asm_out<kRev>(fa, hm, true) : asm_out<kRev>(hm, fa, true);
            if (sh) o += shift * p;
            out[t] = o;
            continue;
        }
        const long k = t - M;
        const double pY = psi[M + k], pA = psi[M + H + k];
        double lY = 0.0, lA = 0.0;
        if (harm) {
            if (kMode == ASM_WIGNER) {
                lY = pc[PC_X * H + k] * pY;
                lA = pc[PC_Y1 * H + k] * pA;
            } else if (kMode == ASM_PLAIN) {
                lY = pc[PC_X * H + k] * pY + pc[PC_Y * H + k] * pA;
                lA = pc[PC_X1 * H + k] * pY + pc[PC_Y1 * H + k] * pA;
            } else {
                lY = pc[PC_X * H + k] * pY + pc[PC_X1 * H + k] * pA;
                lA = pc[PC_Y * H + k] * pY + pc[PC_Y1 * H + k] * pA;
            }
        }
        double vY = 0.0, vA = 0.0;
        if (anh) {
            const int i = tri[2 * k], j = tri[2 * k + 1];
            const double dv = d2v[(long)i * M + j];
            if (kMode == ASM_WIGNER) {
                vY = pc[PC_RA * H + k] * dv;
                vA = pc[PC_RB * H + k] * dv;
            } else if (kMode == ASM_PLAIN) {
                vY = dv * Yw[i] + dv * Yw[j];
                vA = dv * ReAw[i] + dv * ReAw[j];
            } else {
                vY = 0.5 * (Ywinv[i] * dv * Ywinv[j]);
                if (i != j) vY *= 2;
            }
        }
        double oY = asm_out<kRev>(lY, vY, !kW);
        double oA = asm_out<kRev>(lA, vA, !kW);
        if (sh) {
            oY += shift * pY;
            oA += shift * pA;
        }
        out[M + k] = oY;
        out[M + H + k] = oA;
    }
}

template <int kMode, bool kRev>
__global__ void k_assemble(const double *__restrict__ psi, const double *__restrict__ f,
                           const double *__restrict__ d2v, const double *__restrict__ pc,
                           const int *__restrict__ tri, const double *__restrict__ w,
                           const double *__restrict__ Yw, const double *__restrict__ Ywinv,
                           const double *__restrict__ ReAw, int M, long H, int ignore_harmonic,
                           int with_anh, double shift, double *__restrict__ out) {
    pdl_enter();
    assemble_body<kMode, kRev>(psi, f, d2v, pc, tri, w, Yw, Ywinv, ReAw, M, H, ignore_harmonic,
                               with_anh, shift, out);
}

// Both outputs of a two-perturbation call in one launch: blockIdx.y = 0
// assembles L q (plain layout), blockIdx.y = 1 L^T p (transposed layout)
template <bool kRev>
__global__ void k_assemble_pair(const double *__restrict__ q, const double *__restrict__ f,
                                const double *__restrict__ d2v, double *__restrict__ Lq,
                                const double *__restrict__ p, const double *__restrict__ f2,
                                const double *__restrict__ d2v2, double *__restrict__ pL,
                                const double *__restrict__ pc, const int *__restrict__ tri,
                                const double *__restrict__ w, const double *__restrict__ Yw,
                                const double *__restrict__ Ywinv, const double *__restrict__ ReAw,
                                int M, long H, int ignore_harmonic, double shift) {
    pdl_enter();
    if (blockIdx.y == 0)
        assemble_body<ASM_PLAIN, kRev>(q, f, d2v, pc, tri, w, Yw, Ywinv, ReAw, M, H,
                                       ignore_harmonic, 1, shift, Lq);
    else
        assemble_body<ASM_TRANSPOSE, kRev>(p, f2, d2v2, pc, tri, w, Yw, Ywinv, ReAw, M, H,
                                           ignore_harmonic, 1, shift, pL);
}

template <int kMode>
static cudaError_t launch_assemble(int nb, cudaStream_t st, int reverse, const double *psi,
                            const double *f, const double *d2v, const double *pc, const int *tri,
                            const double *w, const double *Yw, const double *Ywinv,
                            const double *ReAw, int M, long H, int ignore_harmonic, int with_anh,
                            double shift, double *out) {
    if (reverse)
        return launch_pdl(k_assemble<kMode, true>, nb, 256, 0, st, psi, f, d2v, pc, tri, w, Yw,
                          Ywinv, ReAw, M, H, ignore_harmonic, with_anh, shift, out);
    return launch_pdl(k_assemble<kMode, false>, nb, 256, 0, st, psi, f, d2v, pc, tri, w, Yw, Ywinv,
                      ReAw, M, H, ignore_harmonic, with_anh, shift, out);
}

int apply_full_L_dev(tdscha_ctx *c, const double *psi_in, double *psi_out, int transpose,
                     int precision, cudaStream_t st) {
    int M = c->M;
    long H = c->H;
    int with_anh = !c->ignore_v3;
    if (with_anh) {
        if (precision == TDSCHA_PREC_MIXED && c->with_mixed && !c->use_wigner) {
            // the tensor-core path reads Y1 and R1 straight from psi while it
            // forms the Y1 limbs (no Y1 round trip, one launch fewer)
            TDS_TRY(perturb_mixed_psi(c, c->ignore_v4 ? 0 : 1, psi_in,
                                      transpose ? c->pc + PC_TY * H : nullptr,
                                      transpose ? c->pc + PC_TRA * H : nullptr, st));
        } else {
            dim3 gu(ceil_div(M, 256), std::min(M, 65535));
            TDS_CUDA(launch_pdl(k_unpack, gu, 256, 0, st, psi_in, c->pc, M, H, c->use_wigner,
                                transpose, c->ignore_v3, c->R1, c->Y1));
            // Y1 from the unpack is symmetric by construction: no symmetrise pass
            TDS_TRY(run_perturb_sym(c, c->ignore_v4 ? 0 : 1, precision, st));
        }
        // gamma_only: translation projection of f and d2v (DynamicalLanczos.py:3173-3191)
        if (c->tr_ntrans > 0) TDS_TRY(apply_translation_projection(c, st));
    }
    int nb = std::max(1, std::min(ceil_div(M + H, 256), 4096));
    if (c->use_wigner)
        TDS_CUDA(launch_assemble<ASM_WIGNER>(nb, st, c->reverse_L, psi_in, c->f, c->d2v, c->pc, c->tri, c->w,
                                    c->Yw, c->Ywinv, c->ReAw, M, H, c->ignore_harmonic, with_anh,
                                    c->shift, psi_out));
    else if (transpose)
        TDS_CUDA(launch_assemble<ASM_TRANSPOSE>(nb, st, c->reverse_L, psi_in, c->f, c->d2v, c->pc, c->tri,
                                       c->w, c->Yw, c->Ywinv, c->ReAw, M, H, c->ignore_harmonic,
                                       with_anh, c->shift, psi_out));
    else
        TDS_CUDA(launch_assemble<ASM_PLAIN>(nb, st, c->reverse_L, psi_in, c->f, c->d2v, c->pc, c->tri, c->w,
                                   c->Yw, c->Ywinv, c->ReAw, M, H, c->ignore_harmonic, with_anh,
                                   c->shift, psi_out));
    return TDSCHA_OK;
}

// L q and L^T p of a bi-Lanczos step.  On the tensor-core path (normal
// representation, anharmonic part on, no translation projection) both
// perturbation averages run as one two-perturbation call (perturb_mixed_pair:
// the ensemble read once, one launch per kernel for both) and give the bits of
// two separate applications; otherwise, or with TDSCHA_PAIR_APPLY=0 in the
// environment, two applications.
static bool pair_apply_enabled() {
    const char *e = getenv("TDSCHA_PAIR_APPLY");
    return !(e && atoi(e) == 0);
}

int apply_full_L_pair_dev(tdscha_ctx *c, const double *q, const double *p, double *Lq,
                          double *pL, int precision, cudaStream_t st) {
    const bool pair = pair_apply_enabled() && precision == TDSCHA_PREC_MIXED && c->with_mixed &&
                      !c->use_wigner && !c->ignore_v3 && c->tr_ntrans == 0 && c->f2;
    if (!pair) {
        TDS_TRY(apply_full_L_dev(c, q, Lq, 0, precision, st));
        return apply_full_L_dev(c, p, pL, 1, precision, st);
    }
    const long H = c->H;
    const int M = c->M;
    TDS_TRY(perturb_mixed_pair(c, c->ignore_v4 ? 0 : 1, q, p, c->pc + PC_TY * H,
                               c->pc + PC_TRA * H, st));
    const int nb = std::max(1, std::min(ceil_div(M + H, 256), 4096));
    const dim3 g(nb, 2);
    if (c->reverse_L)
        TDS_CUDA(launch_pdl(k_assemble_pair<true>, g, 256, 0, st, q, c->f, c->d2v, Lq, p, c->f2,
                            c->d2v2, pL, c->pc, c->tri, c->w, c->Yw, c->Ywinv, c->ReAw, M, H,
                            c->ignore_harmonic, c->shift));
    else
        TDS_CUDA(launch_pdl(k_assemble_pair<false>, g, 256, 0, st, q, c->f, c->d2v, Lq, p, c->f2,
                            c->d2v2, pL, c->pc, c->tri, c->w, c->Yw, c->Ywinv, c->ReAw, M, H,
                            c->ignore_harmonic, c->shift));
    return TDSCHA_OK;
}

// ---------------------------------------------------------------------------
// Lanczos recurrence.  Device scalars (ctx->scal):
enum { SC_A = 0, SC_PNORM, SC_CQ, SC_CP, SC_B, SC_C, SC_SNORM, SC_SRAW, SC_CONV, SC_NAN, SC_HALT,
       SC_NEXT,     // SC_NEXT: the last re-orthogonalised vector had zero norm
       SC_IB, SC_IS };   // 1 / b and 1 / s_raw for the normalisation
// per-step status written on the device: 0 running, 1 NaN in a, 2 converged
enum { ST_OK = 0, ST_NAN = 1, ST_CONV = 2 };
// hist_dev rows of 4: a_k, b_k, c_k, s_norm_k.

constexpr int kDotThreads = 256;

__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
    return s;   // valid in thread 0
}

// y * mask[e], or y where there is no mask.  The kernels below take the mask
// test out of their loops (kMasked a compile-time flag): float64 runs at two
// FMA per cycle per SM on this part and a multiplication by 1.0 costs as much
// as the FMA it feeds.  y * 1.0 == y, so both forms give the same bits.
template <bool kMasked>
__device__ __forceinline__ double masked(double y, const double *__restrict__ mask, long e) {
    return kMasked ? y * mask[e] : y;
}

template <bool kMasked>
__device__ __forceinline__ double dot1_range(const double *__restrict__ x,
                                             const double *__restrict__ y,
                                             const double *__restrict__ mask, long n) {
    double acc = 0;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        acc += x[e] * masked<kMasked>(y[e], mask, e);
    return acc;
}

// partial of sum x*y*mask (mask may be null) per block
__global__ void k_dot1(const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ mask, long n, double *__restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    double acc = mask ? dot1_range<true>(x, y, mask, n) : dot1_range<false>(x, y, mask, n);
    double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Sum of nblk block partials by one block (fixed order: thread stride, then tree).
__device__ __forceinline__ double reduce_parts(const double *__restrict__ part, int nblk,
                                               double *sh) {
    double v = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += part[b];
    return block_sum(v, sh);
}

// a = dot * p_norm and the axpy factors of the residuals (run_FT :6167-6232)
// a = dot * p_norm and the axpy factors of the residuals (run_FT :6167-6232);
// thread 0
__device__ __forceinline__ void scal_a_body(double d, const double *__restrict__ hist, int k,
                                            double *__restrict__ scal,
                                            double *__restrict__ status) {
    if (scal[SC_HALT] != 0.0) return;
    double c_old = k >= 1 ? hist[4 * (k - 1) + 2] : 1.0;
    double p_norm = hist[4 * k + 3] / c_old;
    double a = d * p_norm;
    scal[SC_A] = a;
    scal[SC_PNORM] = p_norm;
    scal[SC_NAN] = isnan(a) ? 1.0 : 0.0;
    status[k] = isnan(a) ? ST_NAN : ST_OK;
    if (isnan(a)) scal[SC_HALT] = 1.0;
    double cq = 0, cp = 0;
    if (k >= 1) {
        cq = hist[4 * (k - 1) + 2];
        double old_p_norm = (k < 2) ? hist[4 * (k - 1) + 3] : hist[4 * (k - 1) + 3] / hist[4 * (k - 2) + 2];
        cp = hist[4 * (k - 1) + 1] * (old_p_norm / p_norm);
    }
    scal[SC_CQ] = cq;
    scal[SC_CP] = cp;
}

__global__ void k_scal_a(const double *__restrict__ part, int nblk, const double *__restrict__ hist,
                         int k, double *__restrict__ scal, double *__restrict__ status) {
    pdl_enter();
    __shared__ double sh[32];
    double d = reduce_parts(part, nblk, sh);
    if (threadIdx.x == 0) scal_a_body(d, hist, k, scal, status);
}

// Sum of nblk block partials written by other blocks of the same kernel:
// loads from L2 (this SM's L1 may hold the buffer from an earlier step)
__device__ __forceinline__ double reduce_parts_cg(const double *__restrict__ part, int nblk,
                                                  double *sh) {
    double v = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += __ldcg(part + b);
    return block_sum(v, sh);
}

// Whether this block is the last of the grid to have written its partials
// (thread 0 wrote them): the last block then reduces them in the fixed order
// of the separate reduction kernel and resets the counter for the next launch.
// No block waits for another.
__device__ __forceinline__ bool last_block(unsigned *__restrict__ ctr, bool *flag) {
    if (threadIdx.x == 0) {
        __threadfence();
        *flag = atomicAdd(ctr, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (*flag) __threadfence();
    return *flag;
}

// k_dot1 and k_scal_a in one launch (the real-space recurrence)
__global__ void k_dot1_a(const double *__restrict__ x, const double *__restrict__ y,
                         const double *__restrict__ mask, long n, double *__restrict__ part,
                         const double *__restrict__ hist, int k, double *__restrict__ scal,
                         double *__restrict__ status, unsigned *__restrict__ ctr) {
    pdl_enter();
    __shared__ double sh[32];
    __shared__ bool flag;
    double acc = mask ? dot1_range<true>(x, y, mask, n) : dot1_range<false>(x, y, mask, n);
    double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
    if (!last_block(ctr, &flag)) return;
    const double d = reduce_parts_cg(part, gridDim.x, sh);
    if (threadIdx.x == 0) {
        *ctr = 0u;
        scal_a_body(d, hist, k, scal, status);
    }
}

template <bool kMasked>
__device__ __forceinline__ void resid_range(const double *__restrict__ Lq, const double *__restrict__ pL,
                                            const double *__restrict__ q, const double *__restrict__ p,
                                            const double *__restrict__ qprev,
                                            const double *__restrict__ pprev,
                                            const double *__restrict__ mask,
                                            const double *__restrict__ scal, long n,
                                            double *__restrict__ rk, double *__restrict__ sk,
                                            double &ss, double &rr, double &sr) {
    const double a = scal[SC_A], cq = scal[SC_CQ], cp = scal[SC_CP];
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        double r = Lq[e] - a * q[e];
        double s = pL[e] - a * p[e];
        if (qprev) r -= cq * qprev[e];
        if (pprev) s -= cp * pprev[e];
        rk[e] = r;
        sk[e] = s;
        ss += s * masked<kMasked>(s, mask, e);
        rr += r * masked<kMasked>(r, mask, e);
        sr += s * masked<kMasked>(r, mask, e);
    }
}

// rk = Lq - a q - cq q_prev ; sk = pL - a p - cp p_prev ; partial dots ss, rr, sr
__global__ void k_resid(const double *__restrict__ Lq, const double *__restrict__ pL,
                        const double *__restrict__ q, const double *__restrict__ p,
                        const double *__restrict__ qprev, const double *__restrict__ pprev,
                        const double *__restrict__ mask, const double *__restrict__ scal, long n,
                        double *__restrict__ rk, double *__restrict__ sk, double *__restrict__ part,
                        int nblk) {
    pdl_enter();
    __shared__ double sh[32];
    double ss = 0, rr = 0, sr = 0;
    if (mask)
        resid_range<true>(Lq, pL, q, p, qprev, pprev, mask, scal, n, rk, sk, ss, rr, sr);
    else
        resid_range<false>(Lq, pL, q, p, qprev, pprev, mask, scal, n, rk, sk, ss, rr, sr);
    double t;
    t = block_sum(ss, sh); if (threadIdx.x == 0) part[blockIdx.x] = t;
    t = block_sum(rr, sh); if (threadIdx.x == 0) part[nblk + blockIdx.x] = t;
    t = block_sum(sr, sh); if (threadIdx.x == 0) part[2 * nblk + blockIdx.x] = t;
}

// b, c, the new s_norm and the stop test (run_FT :6233-6306); thread 0
__device__ __forceinline__ void scal_bc_body(double ss, double rr, double sr,
                                             double *__restrict__ hist, int k,
                                             double *__restrict__ scal,
                                             double *__restrict__ status) {
    if (scal[SC_HALT] != 0.0) return;
    double s_raw = sqrt(ss);
    double s_norm = s_raw * scal[SC_PNORM];
    double b = sqrt(rr);
    double c = (sr / (s_raw * b)) * s_norm;
    scal[SC_B] = b;
    scal[SC_C] = c;
    scal[SC_SNORM] = s_norm;
    scal[SC_SRAW] = s_raw;
    scal[SC_IB] = 1.0 / b;
    scal[SC_IS] = 1.0 / s_raw;
    bool conv = fabs(b) < kEps || fabs(c) < kEps || scal[SC_NEXT] != 0.0;
    scal[SC_CONV] = conv ? 1.0 : 0.0;
    if (conv) {
        status[k] = ST_CONV;
        scal[SC_HALT] = 1.0;
    }
    hist[4 * k + 0] = scal[SC_A];
    if (!conv) {
        hist[4 * k + 1] = b;
        hist[4 * k + 2] = c;
        hist[4 * (k + 1) + 3] = s_norm;
    }
}

__global__ void k_scal_bc(const double *__restrict__ part, int nblk, double *__restrict__ hist,
                          int k, double *__restrict__ scal, double *__restrict__ status) {
    pdl_enter();
    __shared__ double sh[32];
    double ss = reduce_parts(part, nblk, sh);
    double rr = reduce_parts(part + nblk, nblk, sh);
    double sr = reduce_parts(part + 2 * nblk, nblk, sh);
    if (threadIdx.x == 0) scal_bc_body(ss, rr, sr, hist, k, scal, status);
}

// k_resid and k_scal_bc in one launch (the real-space recurrence)
__global__ void k_resid_bc(const double *__restrict__ Lq, const double *__restrict__ pL,
                           const double *__restrict__ q, const double *__restrict__ p,
                           const double *__restrict__ qprev, const double *__restrict__ pprev,
                           const double *__restrict__ mask, double *__restrict__ scal, long n,
                           double *__restrict__ rk, double *__restrict__ sk,
                           double *__restrict__ part, double *__restrict__ hist, int k,
                           double *__restrict__ status, unsigned *__restrict__ ctr) {
    pdl_enter();
    __shared__ double sh[32];
    __shared__ bool flag;
    const int nblk = gridDim.x;
    double ss = 0, rr = 0, sr = 0;
    if (mask)
        resid_range<true>(Lq, pL, q, p, qprev, pprev, mask, scal, n, rk, sk, ss, rr, sr);
    else
        resid_range<false>(Lq, pL, q, p, qprev, pprev, mask, scal, n, rk, sk, ss, rr, sr);
    double t;
    t = block_sum(ss, sh); if (threadIdx.x == 0) part[blockIdx.x] = t;
    t = block_sum(rr, sh); if (threadIdx.x == 0) part[nblk + blockIdx.x] = t;
    t = block_sum(sr, sh); if (threadIdx.x == 0) part[2 * nblk + blockIdx.x] = t;
    if (!last_block(ctr, &flag)) return;
    const double a = reduce_parts_cg(part, nblk, sh);
    const double b = reduce_parts_cg(part + nblk, nblk, sh);
    const double c = reduce_parts_cg(part + 2 * nblk, nblk, sh);
    if (threadIdx.x == 0) {
        *ctr = 0u;
        scal_bc_body(a, b, c, hist, k, scal, status);
    }
}

// ---------------------------------------------------------------------------
// The re-biorthogonalisation below runs in double-float (dfloat.cuh): GB300
// issues float64 at 2 FMA per clock per SM against 128 float32/int32 lanes,
// and the classical Gram-Schmidt pass spends two products per element and
// stored vector in each of its two sweeps.  In float64 both sweeps sat on the
// float64 pipe (0.8 element-vector per clock per SM) at every step index; with
// the operands split by integer operations and the products and sums formed
// error-free in float32, no float64 instruction runs per (element, vector)
// pair and the sweeps become HBM-bound.

// q_{k+1} = r_k / b, p_{k+1} = s_k / s_raw.  With vs != nullptr (full
// re-biorthogonalisation) also the double-float splits of the masked new pair
// the projection dots read: vs[e] = split(q mask), vs[ldv + e] = split(p mask).
__global__ void k_normalize(const double *__restrict__ rk, const double *__restrict__ sk,
                            const double *__restrict__ scal, long n, double *__restrict__ qn,
                            double *__restrict__ pn, const double *__restrict__ mask,
                            float2 *__restrict__ vs, long ldv) {
    pdl_enter();
    if (scal[SC_HALT] != 0.0) return;
    // the reciprocals come from k_scal_bc: a float64 division per thread here
    // cost more than the whole pass
    const double ib = scal[SC_IB], is = scal[SC_IS];
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        double q = rk[e] * ib, p = sk[e] * is;
        qn[e] = q;
        pn[e] = p;
        if (vs) {
            if (mask) {
                const double m = mask[e];
                q *= m;
                p *= m;
            }
            vs[e] = split_f64(q);
            vs[ldv + e] = split_f64(p);
        }
    }
}

// Full re-biorthogonalisation of the new pair (q_{k+1}, p_{k+1}) against the
// stored basis: q -= sum_j (p_j.q / p_j.q_j) q_j and p -= sum_j (q_j.p / p_j.q_j) p_j
// (one classical Gram-Schmidt pass; the recurrence scalars are not changed).
// The float64 kernels below serve the q-space recurrence; the real-space one
// uses the double-float forms further down (k_rdots*, k_rscale, k_rapply*).
// The dot products run on a (vectors x chunks) grid of block partials: about
// four blocks per SM over all vectors (a single vector in 24 chunks was
// latency-bound at 14 us), but at least 24 chunks of at least eight elements
// per thread, since every block also pays its float64 tree reductions.
constexpr int kMaxChunks = 256;
inline int dot_chunks(long n, int nvec) {
    int want = ceil_div(4L * 152, std::max(nvec, 1));
    int cap = std::min(kMaxChunks, ceil_div(n, 256L * 8));
    return std::max(std::min(24, cap), std::min(want, cap));
}
// four strides' loads issued before their FMAs (the pass streams the whole
// basis and is bound by loads in flight and the float64 pipe); the
// accumulation order is the plain strided one
template <bool kMasked>
__device__ __forceinline__ void proj_dots_range(const double *__restrict__ pj,
                                                const double *__restrict__ qj,
                                                const double *__restrict__ qn,
                                                const double *__restrict__ pn,
                                                const double *__restrict__ mask, long e0, long e1,
                                                double &a, double &b) {
    const long bd = blockDim.x;
    long e = e0 + threadIdx.x;
    for (; e + 3 * bd < e1; e += 4 * bd) {
        double vp[4], vq[4], vqn[4], vpn[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            long x = e + u * bd;
            vp[u] = pj[x];
            vq[u] = qj[x];
            vqn[u] = masked<kMasked>(qn[x], mask, x);
            vpn[u] = masked<kMasked>(pn[x], mask, x);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a = fma(vp[u], vqn[u], a);
            b = fma(vq[u], vpn[u], b);
        }
    }
    for (; e < e1; e += bd) {
        a = fma(pj[e], masked<kMasked>(qn[e], mask, e), a);
        b = fma(qj[e], masked<kMasked>(pn[e], mask, e), b);
    }
}

__global__ void k_proj_dots(const double *__restrict__ Qb, const double *__restrict__ Pb,
                            const double *__restrict__ qn, const double *__restrict__ pn,
                            const double *__restrict__ mask, long n, long ld,
                            double *__restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    int j = blockIdx.x;
    const long nch = gridDim.y;
    long e0 = n * blockIdx.y / nch, e1 = n * (blockIdx.y + 1) / nch;
    const double *pj = Pb + (long)j * ld, *qj = Qb + (long)j * ld;
    double a = 0, b = 0;
    if (mask)
        proj_dots_range<true>(pj, qj, qn, pn, mask, e0, e1, a, b);
    else
        proj_dots_range<false>(pj, qj, qn, pn, mask, e0, e1, a, b);
    double t = block_sum(a, sh);
    if (threadIdx.x == 0) part[((long)j * nch + blockIdx.y) * 2] = t;
    t = block_sum(b, sh);
    if (threadIdx.x == 0) part[((long)j * nch + blockIdx.y) * 2 + 1] = t;
}

// Sum of the nch chunk partials part[(j * nch + c) * stride + off] by one warp
// (lane-strided, then a fixed shuffle tree): the same order on every run.
__device__ __forceinline__ double warp_chunk_sum(const double *__restrict__ part, long j, int nch,
                                                 int stride, int off) {
    const int lane = threadIdx.x & 31;
    double a = 0;
    for (int c = lane; c < nch; c += 32) a += part[(j * nch + c) * stride + off];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
}

// coef[2j], coef[2j+1] = chunk sums / (p_j . q_j); one warp per j
__global__ void k_proj_scale(const double *__restrict__ part, const double *__restrict__ pqn,
                             int nvec, int nch, double *__restrict__ coef) {
    pdl_enter();
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (j >= nvec) return;   // whole warps
    double a = warp_chunk_sum(part, j, nch, 2, 0);
    double b = warp_chunk_sum(part, j, nch, 2, 1);
    if ((threadIdx.x & 31) == 0) {
        double inv = 1.0 / pqn[j];
        coef[2 * j] = a * inv;
        coef[2 * j + 1] = b * inv;
    }
}

constexpr int kProjMax = 2048;   // coefficients cached in shared memory per pass
// q -= sum_j c_j Q_j, p -= sum_j d_j P_j; with pq_part != nullptr (the last
// pass) also the block partials of p . q (mask) for the new pair's weight.
__global__ void k_proj_apply(const double *__restrict__ Qb, const double *__restrict__ Pb,
                             const double *__restrict__ coef, long n, int j0, int nvec, long ld,
                             double *__restrict__ qn, double *__restrict__ pn,
                             const double *__restrict__ mask, double *__restrict__ pq_part) {
    pdl_enter();
    __shared__ double cs[2 * kProjMax];
    __shared__ double sh[32];
    for (int t = threadIdx.x; t < 2 * nvec; t += blockDim.x) cs[t] = coef[2 * j0 + t];
    __syncthreads();
    double pq = 0;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        double q = qn[e], p = pn[e];
        // eight basis vectors' loads issued before their FMAs (in j order)
        int j = 0;
        for (; j + 8 <= nvec; j += 8) {
            double vq[8], vp[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                vq[u] = Qb[(long)(j0 + j + u) * ld + e];
                vp[u] = Pb[(long)(j0 + j + u) * ld + e];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                q = fma(-cs[2 * (j + u)], vq[u], q);
                p = fma(-cs[2 * (j + u) + 1], vp[u], p);
            }
        }
        for (; j < nvec; ++j) {
            q = fma(-cs[2 * j], Qb[(long)(j0 + j) * ld + e], q);
            p = fma(-cs[2 * j + 1], Pb[(long)(j0 + j) * ld + e], p);
        }
        qn[e] = q;
        pn[e] = p;
        if (pq_part) pq = fma(p, mask ? q * mask[e] : q, pq);
    }
    if (pq_part) {
        double t = block_sum(pq, sh);
        if (threadIdx.x == 0) pq_part[blockIdx.x] = t;
    }
}

// Real-space re-biorthogonalisation in double-float (see split_f64).  The
// same classical Gram-Schmidt pass as k_proj_dots / k_proj_scale /
// k_proj_apply: the dots of every stored vector against the unprojected new
// pair, then one update q -= sum_j c_j q_j, p -= sum_j d_j p_j in ascending j.
//
// Dots: block (j, chunk) sums P_j . split(q mask) and Q_j . split(p mask)
// over a contiguous element range, four strides' loads in flight per thread;
// each thread's double-float sums are folded into float64 once and reduced by
// the float64 block tree.
__global__ void k_rdots(const double *__restrict__ Qb, const double *__restrict__ Pb,
                        const float2 *__restrict__ vs, long n, long ldv, long ld,
                        double *__restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const long nch = gridDim.y;
    const long e0 = n * blockIdx.y / nch, e1 = n * (blockIdx.y + 1) / nch;
    const double *pj = Pb + (long)j * ld, *qj = Qb + (long)j * ld;
    const float2 *qm = vs, *pm = vs + ldv;
    float as = 0.f, ac = 0.f, bs = 0.f, bc = 0.f;
    const long bd = blockDim.x;
    long e = e0 + threadIdx.x;
    for (; e + 3 * bd < e1; e += 4 * bd) {
        double vp[4], vq[4];
        float2 vqm[4], vpm[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long x = e + u * bd;
            vp[u] = pj[x];
            vq[u] = qj[x];
            vqm[u] = qm[x];
            vpm[u] = pm[x];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            df_fma_acc(as, ac, split_f64(vp[u]), vqm[u]);
            df_fma_acc(bs, bc, split_f64(vq[u]), vpm[u]);
        }
    }
    for (; e < e1; e += bd) {
        df_fma_acc(as, ac, split_f64(pj[e]), qm[e]);
        df_fma_acc(bs, bc, split_f64(qj[e]), pm[e]);
    }
    double t = block_sum((double)as + (double)ac, sh);
    if (threadIdx.x == 0) part[((long)j * nch + blockIdx.y) * 2] = t;
    t = block_sum((double)bs + (double)bc, sh);
    if (threadIdx.x == 0) part[((long)j * nch + blockIdx.y) * 2 + 1] = t;
}

// coef[j] = split(c_j), split(d_j) with c_j, d_j = chunk sums / (p_j . q_j)
// (float64 sums and division); one warp per j
__global__ void k_rscale(const double *__restrict__ part, const double *__restrict__ pqn,
                         int nvec, int nch, float4 *__restrict__ coef) {
    pdl_enter();
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (j >= nvec) return;   // whole warps
    double a = warp_chunk_sum(part, j, nch, 2, 0);
    double b = warp_chunk_sum(part, j, nch, 2, 1);
    if ((threadIdx.x & 31) == 0) {
        const double inv = 1.0 / pqn[j];
        const float2 c = split_f64(a * inv), d = split_f64(b * inv);
        coef[j] = make_float4(c.x, c.y, d.x, d.y);
    }
}

constexpr int kRProjMax = 1024;   // coefficients per apply pass (16 KB of shared memory)
// q -= sum_j c_j Q_j, p -= sum_j d_j P_j over j0 <= j < j0 + nvec: the sums
// in double-float (eight vectors' loads in flight, ascending j), subtracted
// from the float64 vectors once per pass.  With pq_part != nullptr (the last
// pass) also the block partials of p . q (mask) for the new pair's weight.
__global__ void __launch_bounds__(256) k_rapply(const double *__restrict__ Qb,
                                                const double *__restrict__ Pb,
                                                const float4 *__restrict__ coef, long n, int j0,
                                                int nvec, long ld, double *__restrict__ qn,
                                                double *__restrict__ pn,
                                                const double *__restrict__ mask,
                                                double *__restrict__ pq_part) {
    pdl_enter();
    __shared__ float4 cs[kRProjMax];
    __shared__ double sh[32];
    for (int t = threadIdx.x; t < nvec; t += blockDim.x) cs[t] = coef[j0 + t];
    __syncthreads();
    const double *Q0 = Qb + (long)j0 * ld, *P0 = Pb + (long)j0 * ld;
    double pq = 0;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        float qs = 0.f, qc = 0.f, ps = 0.f, pc = 0.f;
        int j = 0;
        for (; j + 8 <= nvec; j += 8) {
            double vq[8], vp[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                vq[u] = Q0[(long)(j + u) * ld + e];
                vp[u] = P0[(long)(j + u) * ld + e];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const float4 c = cs[j + u];
                df_fma_acc(qs, qc, make_float2(c.x, c.y), split_f64(vq[u]));
                df_fma_acc(ps, pc, make_float2(c.z, c.w), split_f64(vp[u]));
            }
        }
        for (; j < nvec; ++j) {
            const float4 c = cs[j];
            df_fma_acc(qs, qc, make_float2(c.x, c.y), split_f64(Q0[(long)j * ld + e]));
            df_fma_acc(ps, pc, make_float2(c.z, c.w), split_f64(P0[(long)j * ld + e]));
        }
        const double q = (qn[e] - (double)qs) - (double)qc;
        const double p = (pn[e] - (double)ps) - (double)pc;
        qn[e] = q;
        pn[e] = p;
        if (pq_part) pq = fma(p, mask ? q * mask[e] : q, pq);
    }
    if (pq_part) {
        double t = block_sum(pq, sh);
        if (threadIdx.x == 0) pq_part[blockIdx.x] = t;
    }
}

// Vector forms for 16-byte aligned rows (even row stride, aligned bases): two
// consecutive elements per load.  Measured on the GB300 at 188 stored pairs of
// 329 476 elements: a plain streaming read of the basis 160 us (6.2 TB/s),
// these dots 190 us and this update 189 us, against 240 and 305 us for the
// one-element forms above and 254 and 246 us for the float64 ones.

// split_ld(n): the even stride between the q and p halves of ctx->vsplit
inline long split_ld(long n) { return (n + 1) & ~1L; }

// k_rdots over element pairs: block (j, chunk) takes pairs [i0, i1) of its
// chunk, two pair strides' loads in flight; for odd n the last element is
// added by thread 0 of the last chunk.  vs holds split(q mask) at [0, n) and
// split(p mask) at [ldv, ldv + n), ldv even.
__global__ void k_rdots2(const double *__restrict__ Qb, const double *__restrict__ Pb,
                         const float2 *__restrict__ vs, long n, long ldv, long ld,
                         double *__restrict__ part) {
    pdl_enter();
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const long nch = gridDim.y, npair = n >> 1;
    const long i0 = npair * blockIdx.y / nch, i1 = npair * (blockIdx.y + 1) / nch;
    const double *pj = Pb + (long)j * ld, *qj = Qb + (long)j * ld;
    const double2 *p2 = reinterpret_cast<const double2 *>(pj);
    const double2 *q2 = reinterpret_cast<const double2 *>(qj);
    const float4 *qm = reinterpret_cast<const float4 *>(vs);
    const float4 *pm = reinterpret_cast<const float4 *>(vs + ldv);
    float as = 0.f, ac = 0.f, bs = 0.f, bc = 0.f;
    const long bd = blockDim.x;
    long i = i0 + threadIdx.x;
    for (; i + bd < i1; i += 2 * bd) {
        double2 vp[2], vq[2];
        float4 va[2], vb[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const long x = i + u * bd;
            vp[u] = p2[x];
            vq[u] = q2[x];
            va[u] = qm[x];
            vb[u] = pm[x];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            df_fma_acc(as, ac, split_f64(vp[u].x), make_float2(va[u].x, va[u].y));
            df_fma_acc(as, ac, split_f64(vp[u].y), make_float2(va[u].z, va[u].w));
            df_fma_acc(bs, bc, split_f64(vq[u].x), make_float2(vb[u].x, vb[u].y));
            df_fma_acc(bs, bc, split_f64(vq[u].y), make_float2(vb[u].z, vb[u].w));
        }
    }
    for (; i < i1; i += bd) {
        const double2 vp = p2[i], vq = q2[i];
        const float4 va = qm[i], vb = pm[i];
        df_fma_acc(as, ac, split_f64(vp.x), make_float2(va.x, va.y));
        df_fma_acc(as, ac, split_f64(vp.y), make_float2(va.z, va.w));
        df_fma_acc(bs, bc, split_f64(vq.x), make_float2(vb.x, vb.y));
        df_fma_acc(bs, bc, split_f64(vq.y), make_float2(vb.z, vb.w));
    }
    if ((n & 1) && blockIdx.y == nch - 1 && threadIdx.x == 0) {
        const long e = n - 1;
        df_fma_acc(as, ac, split_f64(pj[e]), vs[e]);
        df_fma_acc(bs, bc, split_f64(qj[e]), vs[ldv + e]);
    }
    double t = block_sum((double)as + (double)ac, sh);
    if (threadIdx.x == 0) part[((long)j * nch + blockIdx.y) * 2] = t;
    t = block_sum((double)bs + (double)bc, sh);
    if (threadIdx.x == 0) part[((long)j * nch + blockIdx.y) * 2 + 1] = t;
}

// k_rapply over tiles of 64 elements, one tile per block: lane l of warp w
// holds the element pair (2l, 2l + 1) of the tile and sums the stored vectors
// j = w, w + 8, ... (ascending) in double-float; the eight warps' sums are
// then added in warp order per element and subtracted from the float64
// vectors.  Odd n: the last pair's second element is the row padding (read,
// never written; ld >= n + 1).  pq_part gets one partial per tile.
constexpr int kTileWarps = 8;
__global__ void __launch_bounds__(32 * kTileWarps) k_rapply2(
    const double *__restrict__ Qb, const double *__restrict__ Pb, const float4 *__restrict__ coef,
    long n, int j0, int nvec, long ld, double *__restrict__ qn, double *__restrict__ pn,
    const double *__restrict__ mask, double *__restrict__ pq_part) {
    pdl_enter();
    __shared__ float4 cs[kRProjMax];
    __shared__ float4 red[kTileWarps][64];
    __shared__ double sh[32];
    for (int t = threadIdx.x; t < nvec; t += blockDim.x) cs[t] = coef[j0 + t];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long ld2 = ld >> 1;
    const double2 *Q2 = reinterpret_cast<const double2 *>(Qb + (long)j0 * ld);
    const double2 *P2 = reinterpret_cast<const double2 *>(Pb + (long)j0 * ld);
    const long npair = (n + 1) >> 1;
    const long i = blockIdx.x * 32L + lane;
    const long ic = i < npair ? i : npair - 1;
    float qs0 = 0.f, qc0 = 0.f, qs1 = 0.f, qc1 = 0.f;
    float ps0 = 0.f, pc0 = 0.f, ps1 = 0.f, pc1 = 0.f;
    int j = w;
    for (; j + kTileWarps < nvec; j += 2 * kTileWarps) {
        double2 vq[2], vp[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            vq[u] = Q2[(long)(j + u * kTileWarps) * ld2 + ic];
            vp[u] = P2[(long)(j + u * kTileWarps) * ld2 + ic];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const float4 c = cs[j + u * kTileWarps];
            const float2 cq = make_float2(c.x, c.y), cp = make_float2(c.z, c.w);
            df_fma_acc(qs0, qc0, cq, split_f64(vq[u].x));
            df_fma_acc(qs1, qc1, cq, split_f64(vq[u].y));
            df_fma_acc(ps0, pc0, cp, split_f64(vp[u].x));
            df_fma_acc(ps1, pc1, cp, split_f64(vp[u].y));
        }
    }
    for (; j < nvec; j += kTileWarps) {
        const double2 vq = Q2[(long)j * ld2 + ic], vp = P2[(long)j * ld2 + ic];
        const float4 c = cs[j];
        const float2 cq = make_float2(c.x, c.y), cp = make_float2(c.z, c.w);
        df_fma_acc(qs0, qc0, cq, split_f64(vq.x));
        df_fma_acc(qs1, qc1, cq, split_f64(vq.y));
        df_fma_acc(ps0, pc0, cp, split_f64(vp.x));
        df_fma_acc(ps1, pc1, cp, split_f64(vp.y));
    }
    const float2 a0 = df_norm(qs0, qc0), a1 = df_norm(qs1, qc1);
    const float2 b0 = df_norm(ps0, pc0), b1 = df_norm(ps1, pc1);
    red[w][2 * lane] = make_float4(a0.x, a0.y, b0.x, b0.y);
    red[w][2 * lane + 1] = make_float4(a1.x, a1.y, b1.x, b1.y);
    __syncthreads();
    double pq = 0;
    if (w < 2) {
        const int x = w * 32 + lane;
        const long e = blockIdx.x * 64L + x;
        if (e < n) {
            float4 r = red[0][x];
            float2 A = make_float2(r.x, r.y), B = make_float2(r.z, r.w);
#pragma unroll
            for (int g = 1; g < kTileWarps; ++g) {
                r = red[g][x];
                A = df_add(A, make_float2(r.x, r.y));
                B = df_add(B, make_float2(r.z, r.w));
            }
            const double q = (qn[e] - (double)A.x) - (double)A.y;
            const double p = (pn[e] - (double)B.x) - (double)B.y;
            qn[e] = q;
            pn[e] = p;
            if (pq_part) pq = p * (mask ? q * mask[e] : q);
        }
    }
    if (pq_part) {
        const double t = block_sum(pq, sh);
        if (threadIdx.x == 0) pq_part[blockIdx.x] = t;
    }
}

// pqn[k] = sum of nblk block partials (one block)
__global__ void k_pq_reduce(const double *__restrict__ part, int nblk, double *__restrict__ pqn,
                            int k) {
    pdl_enter();
    __shared__ double sh[32];
    double s = reduce_parts(part, nblk, sh);
    if (threadIdx.x == 0) pqn[k] = s;
}

// p_j . q_j for j in [j0, j0 + gridDim.x): chunk partials, then one thread per j.
__global__ void k_pq_part(const double *__restrict__ Qb, const double *__restrict__ Pb,
                          const double *__restrict__ mask, long n, long ld, int j0,
                          double *__restrict__ part) {
    __shared__ double sh[32];
    int j = j0 + blockIdx.x;
    const long nch = gridDim.y;
    long e0 = n * blockIdx.y / nch, e1 = n * (blockIdx.y + 1) / nch;
    double a = 0;
    for (long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        double m = mask ? mask[e] : 1.0;
        a = fma(Pb[(long)j * ld + e], Qb[(long)j * ld + e] * m, a);
    }
    double t = block_sum(a, sh);
    if (threadIdx.x == 0) part[(long)blockIdx.x * nch + blockIdx.y] = t;
}

__global__ void k_pq_finish(const double *__restrict__ part, int cnt, int j0, int nch,
                            double *__restrict__ out) {
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (j >= cnt) return;   // whole warps
    double a = warp_chunk_sum(part, j, nch, 1, 0);
    if ((threadIdx.x & 31) == 0) out[j0 + j] = a;
}

// q-space Hermitian re-orthogonalisation tail: q_{k+1} /= |q_{k+1}|, p_{k+1} = q_{k+1}
// and s_norm_{k+1} = c_k (QSpaceLanczos.py:1110-1125).  Every block reduces the
// same partials in the same order, so all blocks scale by the same factor.
__global__ void k_qrenorm(const double *__restrict__ part, int nblk, double *__restrict__ scal,
                          double *__restrict__ hist, int k, long n, double *__restrict__ qn,
                          double *__restrict__ pn) {
    __shared__ double sh[32];
    __shared__ double inv_s;
    if (scal[SC_HALT] != 0.0) return;
    double s = reduce_parts(part, nblk, sh);
    if (threadIdx.x == 0) {
        double nrm = sqrt(s);
        inv_s = 1.0 / nrm;
        if (blockIdx.x == 0) {
            if (nrm < kEps) scal[SC_NEXT] = 1.0;
            hist[4 * (k + 1) + 3] = scal[SC_C];
        }
    }
    __syncthreads();
    const double iv = inv_s;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        double v = qn[e] * iv;
        qn[e] = v;
        pn[e] = v;
    }
}

// Kernel polynomial method (QSpaceKPM.run_KPM, Modules/QSpaceKPM.py:260-454):
// vp = 2 (L v - b v) / a - vm written over vm, and the moment finishers
// moments[idx] = 2 <x, y>_M - moments[ref].
__global__ void k_kpm_combine(const double *__restrict__ Lv, const double *__restrict__ v,
                              double *__restrict__ vm, double a, double b, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        vm[e] = 2 * ((Lv[e] - b * v[e]) / a) - vm[e];
}

__global__ void k_kpm_moment(const double *__restrict__ part, int nblk, double *__restrict__ moments,
                             int idx, int ref) {
    __shared__ double sh[32];
    double s = reduce_parts(part, nblk, sh);
    if (threadIdx.x == 0) moments[idx] = 2 * s - moments[ref];
}

// Copies hist rows / status of steps next..k back to the host and applies the
// stop conditions; returns TDSCHA_OK or an error and sets *stop.
// Lagged read-back for one run on one stream: at a batch boundary the
// history rows and status words of the batch's steps are copied into one of
// two pinned halves of stat_host with an event behind them, and the batch
// before it (whose copies the GPU finished while it ran this batch) is
// processed.  The host never drains the stream at a boundary, so the GPU keeps
// up to one batch of steps queued.  Steps launched after the processed batch
// reports convergence or a NaN are no-ops of the recurrence on the device
// (halt flag) and are not reported.
struct LaggedReadBack {
    double *hist_dev, *stat_dev, *stat_host;
    int capacity;
    cudaStream_t st;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int buf = 0, pend_next = 0, pend_k = -1, pend_buf = 0;
    bool pending = false;

    LaggedReadBack(double *hd, double *sd, double *sh, int cap, cudaStream_t s)
        : hist_dev(hd), stat_dev(sd), stat_host(sh), capacity(cap), st(s) {}
    ~LaggedReadBack() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    double *half(int b) const { return stat_host + (size_t)b * 5 * (capacity + 1); }
    int init() {
        for (auto &e : ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                set_error("lanczos_run: cannot create an event");
                return TDSCHA_ERR_CUDA;
            }
        return TDSCHA_OK;
    }
    // copies of steps next..k behind the launches so far, then the previous batch
    int boundary(int next, int k, double *hist, int start_step, int *steps_done, int *converged,
                 bool *stop) {
        int cnt = k - next + 1;
        double *hh = half(buf), *hs = hh + 4 * (capacity + 1);
        if (cudaMemcpyAsync(hh, hist_dev + 4 * next, sizeof(double) * 4 * (cnt + 1),
                            cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(hs, stat_dev + next, sizeof(double) * cnt, cudaMemcpyDeviceToHost,
                            st) != cudaSuccess ||
            cudaEventRecord(ev[buf], st) != cudaSuccess) {
            set_error("lanczos_run: %s", cudaGetErrorString(cudaGetLastError()));
            return TDSCHA_ERR_CUDA;
        }
        int rc = pending ? process(hist, start_step, steps_done, converged, stop) : TDSCHA_OK;
        pending = true;
        pend_next = next;
        pend_k = k;
        pend_buf = buf;
        buf ^= 1;
        return rc;
    }
    // the last batch enqueued (at the end of the run)
    int finish(double *hist, int start_step, int *steps_done, int *converged, bool *stop) {
        return pending ? process(hist, start_step, steps_done, converged, stop) : TDSCHA_OK;
    }
    int process(double *hist, int start_step, int *steps_done, int *converged, bool *stop) {
        pending = false;
        if (cudaEventSynchronize(ev[pend_buf]) != cudaSuccess) {
            set_error("lanczos_run: %s", cudaGetErrorString(cudaGetLastError()));
            return TDSCHA_ERR_CUDA;
        }
        const double *hh = half(pend_buf), *hs = hh + 4 * (capacity + 1);
        for (int j = 0; j < pend_k - pend_next + 1; ++j) {
            int kj = pend_next + j;
            if (hs[j] == ST_NAN) {
                set_error("Invalid value encountered during the Lanczos (a is NaN at step %d)", kj);
                *stop = true;
                return TDSCHA_ERR_NAN;
            }
            hist[4 * kj + 0] = hh[4 * j + 0];
            *steps_done = kj - start_step + 1;
            if (hs[j] == ST_CONV) {
                *converged = 1;
                *stop = true;
                return TDSCHA_OK;
            }
            hist[4 * kj + 1] = hh[4 * j + 1];
            hist[4 * kj + 2] = hh[4 * j + 2];
            hist[4 * (kj + 1) + 3] = hh[4 * (j + 1) + 3];
        }
        return TDSCHA_OK;
    }
};

static int read_back_steps(double *hist_dev, double *stat_dev, double *stat_host, int capacity,
                           int next, int k, cudaStream_t st, double *hist, int start_step,
                           int *steps_done, int *converged, bool *stop) {
    int cnt = k - next + 1;
    double *hh = stat_host, *hs = stat_host + 4 * (capacity + 1);
    if (cudaMemcpyAsync(hh, hist_dev + 4 * next, sizeof(double) * 4 * (cnt + 1),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(hs, stat_dev + next, sizeof(double) * cnt, cudaMemcpyDeviceToHost,
                        st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("lanczos_run: %s", cudaGetErrorString(cudaGetLastError()));
        return TDSCHA_ERR_CUDA;
    }
    for (int j = 0; j < cnt; ++j) {
        int kj = next + j;
        if (hs[j] == ST_NAN) {
            set_error("Invalid value encountered during the Lanczos (a is NaN at step %d)", kj);
            *stop = true;
            return TDSCHA_ERR_NAN;
        }
        hist[4 * kj + 0] = hh[4 * j + 0];
        *steps_done = kj - start_step + 1;
        if (hs[j] == ST_CONV) {
            *converged = 1;
            *stop = true;
            return TDSCHA_OK;
        }
        hist[4 * kj + 1] = hh[4 * j + 1];
        hist[4 * kj + 2] = hh[4 * j + 2];
        hist[4 * (kj + 1) + 3] = hh[4 * (j + 1) + 3];
    }
    return TDSCHA_OK;
}

}  // namespace tdscha

using namespace tdscha;

extern "C" int tdscha_apply_full_L(tdscha_ctx *ctx, const double *psi_in, double *psi_out,
                                   int transpose, int precision, void *stream) {
    set_error("");
    if (!ctx || !psi_in || !psi_out) { set_error("apply_full_L: null pointer"); return TDSCHA_ERR_ARG; }
    if (psi_in == psi_out) { set_error("apply_full_L: in-place application is not supported"); return TDSCHA_ERR_ARG; }
    return apply_full_L_dev(ctx, psi_in, psi_out, transpose, precision, (cudaStream_t)stream);
}

namespace tdscha {

// Buffers and start-of-run state of one real-space run (everything before the
// first step of tdscha_lanczos_run); stream ordered.
static int lz_begin(tdscha_ctx *ctx, double *basis_Q, double *basis_P, long ld, int capacity,
                    int start_step, int run_simm, int full_reorth, const double *hist,
                    cudaStream_t st) {
    const long P = ctx->P;
    const double *mask = run_simm ? ctx->mask : nullptr;
    if (ctx->hist_cap < capacity + 1) {
        if (ctx->hist_dev) cudaFree(ctx->hist_dev);
        ctx->hist_dev = nullptr;
        TDS_CUDA(cudaMalloc(&ctx->hist_dev, sizeof(double) * 4 * (capacity + 1)));
        ctx->hist_cap = capacity + 1;
    }
    TDS_CUDA(cudaMemcpyAsync(ctx->hist_dev, hist, sizeof(double) * 4 * (start_step + 1),
                             cudaMemcpyHostToDevice, st));
    if (full_reorth) {
        if (ctx->pqn_cap < capacity + 1) {
            if (ctx->pqn) cudaFree(ctx->pqn);
            if (ctx->rcoef) cudaFree(ctx->rcoef);
            ctx->pqn = ctx->rcoef = nullptr;
            TDS_CUDA(cudaMalloc(&ctx->pqn, sizeof(double) * (capacity + 1)));
            TDS_CUDA(cudaMalloc(&ctx->rcoef, sizeof(double) * 2 * (capacity + 1) * (kMaxChunks + 1)));
            ctx->pqn_cap = capacity + 1;
        }
        if (!ctx->vsplit) TDS_CUDA(cudaMalloc(&ctx->vsplit, sizeof(float2) * 2 * split_ld(P)));
        // weights of the vectors already stored
        double *part = ctx->rcoef + 2 * (capacity + 1);
        const int nch = dot_chunks(P, start_step + 1);
        k_pq_part<<<dim3(start_step + 1, nch), 256, 0, st>>>(basis_Q, basis_P, mask, P, ld, 0, part);
        k_pq_finish<<<ceil_div(start_step + 1, 8), 256, 0, st>>>(part, start_step + 1, 0, nch,
                                                                 ctx->pqn);
        TDS_CHECK_LAUNCH();
    }
    if (ctx->stat_cap < capacity + 1) {
        if (ctx->stat_dev) cudaFree(ctx->stat_dev);
        if (ctx->stat_host) cudaFreeHost(ctx->stat_host);
        ctx->stat_dev = ctx->stat_host = nullptr;
        ctx->stat_cap = 0;
        TDS_CUDA(cudaMalloc(&ctx->stat_dev, sizeof(double) * (capacity + 1)));
        // two halves for the lagged read-back
        TDS_CUDA(cudaMallocHost((void **)&ctx->stat_host, sizeof(double) * 10 * (capacity + 1)));
        ctx->stat_cap = capacity + 1;
    }
    TDS_CUDA(cudaMemsetAsync(ctx->scal, 0, sizeof(double) * 64, st));
    return TDSCHA_OK;
}

// The launches of step k (run_FT :6145-6448): operator application(s), the
// recurrence scalars on the device, the new pair and its re-biorthogonalisation.
static int lz_step(tdscha_ctx *ctx, double *basis_Q, double *basis_P, long ld, int capacity,
                   int k, int run_simm, int precision, int full_reorth, cudaStream_t st) {
    const long P = ctx->P;
    const double *mask = run_simm ? ctx->mask : nullptr;
    const int nb = std::max(1, std::min(ceil_div(P, kDotThreads), ctx->nblk_dot));
    // elementwise passes over the vectors and the basis: eight blocks per SM
    const int nbw = std::max(1, std::min(ceil_div(P, kDotThreads), 1216));
    double *q = basis_Q + (long)k * ld, *p = basis_P + (long)k * ld;
    const double *pL = ctx->Lq;
    if (run_simm) {
        TDS_TRY(apply_full_L_dev(ctx, q, ctx->Lq, 0, precision, st));
    } else {
        TDS_TRY(apply_full_L_pair_dev(ctx, q, p, ctx->Lq, ctx->pL, precision, st));
        pL = ctx->pL;
    }
    // the dot products with their scalar tails in one launch each (the last
    // block reduces the partials, counters ctx->ctr[0] and [1])
    launch_pdl(k_dot1_a, nb, kDotThreads, 0, st, p, ctx->Lq, mask, P, ctx->dots, ctx->hist_dev, k,
               ctx->scal, ctx->stat_dev, ctx->ctr);
    const double *qprev = k >= 1 ? basis_Q + (long)(k - 1) * ld : nullptr;
    const double *pprev = k >= 1 ? basis_P + (long)(k - 1) * ld : nullptr;
    launch_pdl(k_resid_bc, nb, kDotThreads, 0, st, ctx->Lq, pL, q, p, qprev, pprev, mask, ctx->scal,
               P, ctx->rk, ctx->sk, ctx->dots, ctx->hist_dev, k, ctx->stat_dev, ctx->ctr + 1);
    double *qn = basis_Q + (long)(k + 1) * ld, *pn = basis_P + (long)(k + 1) * ld;
    const long ldv = split_ld(P);
    launch_pdl(k_normalize, nbw, kDotThreads, 0, st, ctx->rk, ctx->sk, ctx->scal, P, qn, pn, mask,
               full_reorth ? ctx->vsplit : nullptr, ldv);
    if (full_reorth) {
        int nvec = k + 1;
        double *part = ctx->rcoef + 2 * (capacity + 1);
        const int nch = dot_chunks(P, nvec);
        float4 *coef = reinterpret_cast<float4 *>(ctx->rcoef);
        const float2 *vs = ctx->vsplit;
        // two elements per load where every row starts on 16 bytes
        const bool vec = (ld % 2 == 0) && ((uintptr_t)basis_Q % 16 == 0) &&
                         ((uintptr_t)basis_P % 16 == 0);
        {
            ProfScope ps(ctx, 6, st);
            if (vec)
                launch_pdl(k_rdots2, dim3(nvec, nch), 256, 0, st, basis_Q, basis_P, vs, P, ldv, ld,
                           part);
            else
                launch_pdl(k_rdots, dim3(nvec, nch), 256, 0, st, basis_Q, basis_P, vs, P, ldv, ld,
                           part);
            launch_pdl(k_rscale, ceil_div(nvec, 8), 256, 0, st, part, ctx->pqn, nvec, nch, coef);
        }
        ProfScope ps(ctx, 7, st);
        const int ntile = (int)ceil_div(P, 64L);
        const int npq = vec ? ntile : nbw;
        for (int j0 = 0; j0 < nvec; j0 += kRProjMax) {
            bool last = j0 + kRProjMax >= nvec;
            if (vec)
                launch_pdl(k_rapply2, ntile, 32 * kTileWarps, 0, st, basis_Q, basis_P,
                           (const float4 *)coef, P, j0, std::min(kRProjMax, nvec - j0), ld, qn,
                           pn, mask, last ? ctx->dots : nullptr);
            else
                launch_pdl(k_rapply, nbw, 256, 0, st, basis_Q, basis_P, (const float4 *)coef, P,
                           j0, std::min(kRProjMax, nvec - j0), ld, qn, pn, mask,
                           last ? ctx->dots : nullptr);
        }
        // weight p_{k+1} . q_{k+1} of the new pair from the apply pass's partials
        launch_pdl(k_pq_reduce, 1, 512, 0, st, ctx->dots, npq, ctx->pqn, k + 1);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error("lanczos_run launch: %s", cudaGetErrorString(e)); return TDSCHA_ERR_CUDA; }
    return TDSCHA_OK;
}

// the recurrence's stop conditions are evaluated on the device (per-step
// status + a halt flag that turns later steps into no-ops), so steps are
// launched back to back and read back every kSyncEvery steps
constexpr int kSyncEvery = 16;

}  // namespace tdscha

namespace tdscha {

// tdscha_lanczos_run on basis rows of stride ld
static int lz_run(tdscha_ctx *ctx, double *basis_Q, double *basis_P, long ld, int capacity,
                  int start_step, int n_iter, int run_simm, int precision, int full_reorth,
                  double *hist, int *steps_done, int *converged, void *stream) {
    set_error("");
    if (!ctx || !basis_Q || !basis_P || !hist || !steps_done || !converged) {
        set_error("lanczos_run: null pointer");
        return TDSCHA_ERR_ARG;
    }
    if (capacity < 1 || start_step < 0 || n_iter < 0 || start_step + 1 > capacity) {
        set_error("lanczos_run: bad capacity %d / start %d / n_iter %d", capacity, start_step, n_iter);
        return TDSCHA_ERR_ARG;
    }
    if (run_simm && !ctx->use_wigner) {
        set_error("lanczos_run: the symmetric Lanczos works only with Wigner");
        return TDSCHA_ERR_ARG;
    }
    *steps_done = 0;
    *converged = 0;
    cudaStream_t st = (cudaStream_t)stream;
    TDS_TRY(lz_begin(ctx, basis_Q, basis_P, ld, capacity, start_step, run_simm, full_reorth, hist,
                     st));
    LaggedReadBack rb(ctx->hist_dev, ctx->stat_dev, ctx->stat_host, capacity, st);
    TDS_TRY(rb.init());
    int rc = TDSCHA_OK;
    int next = start_step;          // first step not yet copied back
    bool stop = false;
    for (int it = 0; it < n_iter && !stop; ++it) {
        int k = start_step + it;
        if (k + 1 >= capacity) {
            set_error("lanczos_run: basis capacity %d exhausted at step %d", capacity, k);
            rc = TDSCHA_ERR_ARG;
            break;
        }
        if ((rc = lz_step(ctx, basis_Q, basis_P, ld, capacity, k, run_simm, precision, full_reorth,
                          st)) != TDSCHA_OK)
            break;
        if ((it + 1) % kSyncEvery != 0 && it + 1 != n_iter) continue;
        rc = rb.boundary(next, k, hist, start_step, steps_done, converged, &stop);
        // a timed-out tensor-core wait outranks whatever the read-back saw
        int mrc = mixed_check_error(ctx);
        if (mrc != TDSCHA_OK) { rc = mrc; break; }
        if (rc != TDSCHA_OK) break;
        next = k + 1;
    }
    if (rc == TDSCHA_OK && !stop) rc = rb.finish(hist, start_step, steps_done, converged, &stop);
    // every launched step completes before the call returns
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == TDSCHA_OK) {
        set_error("lanczos_run: %s", cudaGetErrorString(cudaGetLastError()));
        rc = TDSCHA_ERR_CUDA;
    }
    int mrc = mixed_check_error(ctx);
    if (mrc != TDSCHA_OK) rc = mrc;
    return rc;
}

inline long basis_stride(const tdscha_ctx *ctx) { return ctx->basis_ld ? ctx->basis_ld : ctx->P; }

}  // namespace tdscha

extern "C" int tdscha_lanczos_run(tdscha_ctx *ctx, double *basis_Q, double *basis_P, int capacity,
                                  int start_step, int n_iter, int run_simm, int precision,
                                  int full_reorth, double *hist, int *steps_done, int *converged,
                                  void *stream) {
    if (!ctx) {
        set_error("lanczos_run: null pointer");
        return TDSCHA_ERR_ARG;
    }
    return lz_run(ctx, basis_Q, basis_P, basis_stride(ctx), capacity, start_step, n_iter, run_simm,
                  precision, full_reorth, hist, steps_done, converged, stream);
}

namespace tdscha {

struct cplx { double x, y; };
__device__ __forceinline__ cplx cmul(cplx a, cplx b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
    // Smith's algorithm
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, d = b.x + b.y * r;
        return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
    }
    double r = b.x / b.y, d = b.y + b.x * r;
    return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
}

__global__ void k_cfrac(const double *__restrict__ a, int n, const double *__restrict__ b,
                        const double *__restrict__ c, int nonsym, const double *__restrict__ w,
                        int n_w, int wigner, double modulus, double sign, double shift,
                        int use_term, int last_average, double smearing, int smooth_ramp,
                        int n_b, double *__restrict__ g) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_w) return;
    double wv = w[t];
    double w2 = wv * wv;
    cplx gf;
    double a_m = 0, b_m = 0, c_m = 0;
    if (use_term) {
        int la = min(last_average, n), lb = min(last_average, n_b);
        double sa = 0, sb = 0, scc = 0;
        for (int i = n - la; i < n; ++i) sa += a[i];
        for (int i = n_b - lb; i < n_b; ++i) { sb += b[i]; scc += c[i]; }
        double a_av = sa / la, b_av = sb / lb, c_av = nonsym ? scc / lb : b_av;
        a_m = a_av * sign - sign * shift;
        b_m = b_av * sign;
        c_m = c_av * sign;
        double d = wigner ? a_m + w2 : a_m - w2;
        double disc = d * d - 4 * b_m * c_m;
        cplx sq = disc >= 0 ? cplx{sqrt(disc), 0.0} : cplx{0.0, sqrt(-disc)};
        double den = 2 * b_m * c_m;
        cplx gp = {(d + sq.x) / den, sq.y / den};
        cplx gm = {(d - sq.x) / den, -sq.y / den};
        gf = (hypot(gp.x, gp.y) < hypot(gm.x, gm.y)) ? gp : gm;
    } else {
        double av = a[n - 1] * sign - sign * shift;
        cplx den = {wigner ? av + w2 : av - w2, 2 * wv * smearing};
        gf = cdiv({1.0, 0.0}, den);
    }
    for (int i = n - 2; i >= 0; --i) {
        double av = a[i] * sign - sign * shift;
        double bv = b[i] * sign;
        double cv = nonsym ? c[i] * sign : bv;
        if (use_term && smooth_ramp > 0 && i >= n - smooth_ramp) {
            double al = (double)(i - n + smooth_ramp + 1) / smooth_ramp;
            av = (1 - al) * av + al * a_m;
            bv = (1 - al) * bv + al * b_m;
            cv = (1 - al) * cv + al * c_m;
        }
        cplx bcg = cmul({bv * cv, 0.0}, gf);
        cplx den = {(wigner ? av + w2 : av - w2) - bcg.x, 2 * wv * smearing - bcg.y};
        gf = cdiv({1.0, 0.0}, den);
    }
    if (wigner) gf = {-gf.x, gf.y};
    g[2 * t] = gf.x * modulus;
    g[2 * t + 1] = gf.y * modulus;
}

}  // namespace tdscha

extern "C" int tdscha_continued_fraction(const double *a, int n, const double *b, int n_b,
                                         const double *c, int n_c, const double *w, int n_w,
                                         int use_wigner, double modulus, int reverse_L,
                                         double shift_value, int use_terminator,
                                         int last_average, double smearing, int smooth_ramp,
                                         double *g_out) {
    set_error("");
    if (n < 1 || n_w < 0 || !a || !w || !g_out || n_b < 0 || (n > 1 && n_b < n - 1) || (n_b > 0 && !b)) {
        set_error("continued_fraction: bad arguments");
        return TDSCHA_ERR_ARG;
    }
    if (use_terminator && (n_b < 1 || last_average < 1)) {
        set_error("continued_fraction: the terminator needs b coefficients and last_average >= 1");
        return TDSCHA_ERR_ARG;
    }
    if (n_w == 0) return TDSCHA_OK;
    int nonsym = (n_c == n_b && c != nullptr) ? 1 : 0;
    double *d_a = nullptr, *d_b = nullptr, *d_c = nullptr, *d_w = nullptr, *d_g = nullptr;
    size_t nbb = std::max(n_b, 1);
    TDS_CUDA(cudaMalloc(&d_a, sizeof(double) * n));
    TDS_CUDA(cudaMalloc(&d_b, sizeof(double) * nbb));
    TDS_CUDA(cudaMalloc(&d_c, sizeof(double) * nbb));
    TDS_CUDA(cudaMalloc(&d_w, sizeof(double) * n_w));
    TDS_CUDA(cudaMalloc(&d_g, sizeof(double) * 2 * n_w));
    cudaMemcpy(d_a, a, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (n_b) cudaMemcpy(d_b, b, sizeof(double) * n_b, cudaMemcpyHostToDevice);
    if (nonsym && n_b) cudaMemcpy(d_c, c, sizeof(double) * n_b, cudaMemcpyHostToDevice);
    cudaMemcpy(d_w, w, sizeof(double) * n_w, cudaMemcpyHostToDevice);
    k_cfrac<<<ceil_div(n_w, 128), 128>>>(d_a, n, d_b, d_c, nonsym, d_w, n_w, use_wigner, modulus,
                                         reverse_L ? -1.0 : 1.0, shift_value, use_terminator,
                                         last_average, smearing, smooth_ramp, n_b, d_g);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(g_out, d_g, sizeof(double) * 2 * n_w, cudaMemcpyDeviceToHost);
    cudaFree(d_a); cudaFree(d_b); cudaFree(d_c); cudaFree(d_w); cudaFree(d_g);
    if (e != cudaSuccess) { set_error("continued_fraction: %s", cudaGetErrorString(e)); return TDSCHA_ERR_CUDA; }
    return TDSCHA_OK;
}

namespace tdscha {

static int qz_begin(tdscha_qctx *ctx, double *basis_Q, int capacity, int start_step,
                    int reorthogonalize, const double *hist, cudaStream_t st) {
    const long n = 2 * ctx->P;           // interleaved (re, im) doubles
    if (ctx->hist_cap < capacity + 1) {
        if (ctx->hist_dev) cudaFree(ctx->hist_dev);
        if (ctx->stat_dev) cudaFree(ctx->stat_dev);
        if (ctx->stat_host) cudaFreeHost(ctx->stat_host);
        if (ctx->pqn) cudaFree(ctx->pqn);
        if (ctx->rcoef) cudaFree(ctx->rcoef);
        ctx->hist_dev = ctx->stat_dev = ctx->stat_host = ctx->pqn = ctx->rcoef = nullptr;
        ctx->hist_cap = 0;
        TDS_CUDA(cudaMalloc(&ctx->hist_dev, sizeof(double) * 4 * (capacity + 1)));
        TDS_CUDA(cudaMalloc(&ctx->stat_dev, sizeof(double) * (capacity + 1)));
        TDS_CUDA(cudaMallocHost((void **)&ctx->stat_host, sizeof(double) * 10 * (capacity + 1)));
        TDS_CUDA(cudaMalloc(&ctx->pqn, sizeof(double) * (capacity + 1)));
        TDS_CUDA(cudaMalloc(&ctx->rcoef, sizeof(double) * 2 * (capacity + 1) * (kMaxChunks + 1)));
        ctx->hist_cap = capacity + 1;
    }
    TDS_CUDA(cudaMemcpyAsync(ctx->hist_dev, hist, sizeof(double) * 4 * (start_step + 1),
                             cudaMemcpyHostToDevice, st));
    double *part = ctx->rcoef + 2 * (capacity + 1);
    if (reorthogonalize) {
        // Q is orthonormal in the mask product; the weights q_j . q_j are kept exact
        const int nch = dot_chunks(n, start_step + 1);
        k_pq_part<<<dim3(start_step + 1, nch), 256, 0, st>>>(basis_Q, basis_Q, ctx->mask, n, n, 0, part);
        k_pq_finish<<<ceil_div(start_step + 1, 8), 256, 0, st>>>(part, start_step + 1, 0, nch,
                                                                 ctx->pqn);
        TDS_CHECK_LAUNCH();
    }
    TDS_CUDA(cudaMemsetAsync(ctx->scal, 0, sizeof(double) * 64, st));
    return TDSCHA_OK;
}

// Step k of the Hermitian q-space Lanczos (QSpaceLanczos.py:1050-1140).
static int qz_step(tdscha_qctx *ctx, double *basis_Q, double *basis_P, int capacity, int k,
                   int reorthogonalize, cudaStream_t st) {
    const long n = 2 * ctx->P;
    const double *mask = ctx->mask;
    const int nb = std::max(1, std::min(ceil_div(n, kDotThreads), 296));
    double *part = ctx->rcoef + 2 * (capacity + 1);
    double *q = basis_Q + (long)k * n, *p = basis_P + (long)k * n;
    // Hermitian operator: p_L = L q (QSpaceLanczos.py:1055-1057)
    TDS_TRY(q_apply_full_L_dev(ctx, q, ctx->Lq, st));
    k_dot1<<<nb, kDotThreads, 0, st>>>(p, ctx->Lq, mask, n, ctx->dots);
    k_scal_a<<<1, 256, 0, st>>>(ctx->dots, nb, ctx->hist_dev, k, ctx->scal, ctx->stat_dev);
    const double *qprev = k >= 1 ? basis_Q + (long)(k - 1) * n : nullptr;
    const double *pprev = k >= 1 ? basis_P + (long)(k - 1) * n : nullptr;
    k_resid<<<nb, kDotThreads, 0, st>>>(ctx->Lq, ctx->Lq, q, p, qprev, pprev, mask, ctx->scal, n,
                                         ctx->rk, ctx->sk, ctx->dots, nb);
    k_scal_bc<<<1, 256, 0, st>>>(ctx->dots, nb, ctx->hist_dev, k, ctx->scal, ctx->stat_dev);
    double *qn = basis_Q + (long)(k + 1) * n, *pn = basis_P + (long)(k + 1) * n;
    k_normalize<<<nb, kDotThreads, 0, st>>>(ctx->rk, ctx->sk, ctx->scal, n, qn, pn, nullptr, nullptr,
                                            0L);
    if (reorthogonalize) {
        // one classical Gram-Schmidt pass of q_{k+1} against q_0..q_k with the
        // real mask product (the p side of the shared kernels runs on the
        // p_{k+1} slot, which the renormalisation then overwrites)
        int nvec = k + 1;
        const int nch = dot_chunks(n, nvec);
        k_proj_dots<<<dim3(nvec, nch), 256, 0, st>>>(basis_Q, basis_Q, qn, pn, mask, n, n, part);
        k_proj_scale<<<ceil_div(nvec, 8), 256, 0, st>>>(part, ctx->pqn, nvec, nch, ctx->rcoef);
        for (int j0 = 0; j0 < nvec; j0 += kProjMax)
            k_proj_apply<<<nb, 256, 0, st>>>(basis_Q, basis_Q, ctx->rcoef, n, j0,
                                             std::min(kProjMax, nvec - j0), n, qn, pn, nullptr,
                                             nullptr);
        k_dot1<<<nb, kDotThreads, 0, st>>>(qn, qn, mask, n, ctx->dots);
        k_qrenorm<<<nb, kDotThreads, 0, st>>>(ctx->dots, nb, ctx->scal, ctx->hist_dev, k, n, qn, pn);
        k_pq_part<<<dim3(1, nch), 256, 0, st>>>(basis_Q, basis_Q, mask, n, n, k + 1, part);
        k_pq_finish<<<1, 32, 0, st>>>(part, 1, k + 1, nch, ctx->pqn);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error("qlanczos_run launch: %s", cudaGetErrorString(e)); return TDSCHA_ERR_CUDA; }
    return TDSCHA_OK;
}

}  // namespace tdscha

extern "C" int tdscha_qlanczos_run(tdscha_qctx *ctx, double *basis_Q, double *basis_P, int capacity,
                                   int start_step, int n_iter, int reorthogonalize, double *hist,
                                   int *steps_done, int *converged, void *stream) {
    set_error("");
    if (!ctx || !basis_Q || !basis_P || !hist || !steps_done || !converged) {
        set_error("qlanczos_run: null pointer");
        return TDSCHA_ERR_ARG;
    }
    if (ctx->n_pairs == 0) { set_error("qlanczos_run: call tdscha_qctx_set_pert first"); return TDSCHA_ERR_STATE; }
    if (capacity < 1 || start_step < 0 || n_iter < 0 || start_step + 1 > capacity) {
        set_error("qlanczos_run: bad capacity %d / start %d / n_iter %d", capacity, start_step, n_iter);
        return TDSCHA_ERR_ARG;
    }
    if (basis_Q == basis_P) { set_error("qlanczos_run: basis_Q and basis_P must be distinct"); return TDSCHA_ERR_ARG; }
    *steps_done = 0;
    *converged = 0;
    cudaStream_t st = (cudaStream_t)stream;
    TDS_TRY(qz_begin(ctx, basis_Q, capacity, start_step, reorthogonalize, hist, st));
    LaggedReadBack rb(ctx->hist_dev, ctx->stat_dev, ctx->stat_host, capacity, st);
    TDS_TRY(rb.init());
    int rc = TDSCHA_OK;
    int next = start_step;
    bool stop = false;
    for (int it = 0; it < n_iter && !stop; ++it) {
        int k = start_step + it;
        if (k + 1 >= capacity) {
            set_error("qlanczos_run: basis capacity %d exhausted at step %d", capacity, k);
            rc = TDSCHA_ERR_ARG;
            break;
        }
        if ((rc = qz_step(ctx, basis_Q, basis_P, capacity, k, reorthogonalize, st)) != TDSCHA_OK) break;
        if ((it + 1) % kSyncEvery != 0 && it + 1 != n_iter) continue;
        rc = rb.boundary(next, k, hist, start_step, steps_done, converged, &stop);
        if (rc != TDSCHA_OK) break;
        next = k + 1;
    }
    if (rc == TDSCHA_OK && !stop) rc = rb.finish(hist, start_step, steps_done, converged, &stop);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == TDSCHA_OK) {
        set_error("qlanczos_run: %s", cudaGetErrorString(cudaGetLastError()));
        rc = TDSCHA_ERR_CUDA;
    }
    return rc;
}

// Many independent runs together (real-space and q-space contexts mixed): each
// run gets its own stream; the driver launches up to kSyncEvery steps of every
// active run before it reads any of them back, so the runs' kernels overlap on
// the device.  Per-run results and status in the descriptors.
extern "C" int tdscha_lanczos_run_batch(tdscha_run *runs, int n_runs) {
    set_error("");
    if (!runs || n_runs < 0) { set_error("lanczos_run_batch: bad arguments"); return TDSCHA_ERR_ARG; }
    for (int i = 0; i < n_runs; ++i) {
        tdscha_run &r = runs[i];
        r.steps_done = 0;
        r.converged = 0;
        r.status = TDSCHA_OK;
        bool ok = r.ctx && r.basis_Q && r.basis_P && r.hist && r.capacity >= 1 && r.start_step >= 0 &&
                  r.n_iter >= 0 && r.start_step + r.n_iter < r.capacity && (r.kind == 0 || r.kind == 1) &&
                  r.basis_Q != r.basis_P;
        if (ok && r.kind == 0) ok = !r.run_simm || ((tdscha_ctx *)r.ctx)->use_wigner;
        if (ok && r.kind == 1) ok = ((tdscha_qctx *)r.ctx)->n_pairs > 0;
        if (!ok) {
            set_error("lanczos_run_batch: run %d has bad arguments", i);
            return TDSCHA_ERR_ARG;
        }
    }
    // a context holds the recurrence state of one run: one context per run
    for (int i = 0; i < n_runs; ++i)
        for (int j = 0; j < i; ++j)
            if (runs[j].ctx == runs[i].ctx) {
                set_error("lanczos_run_batch: runs %d and %d share a context", j, i);
                return TDSCHA_ERR_ARG;
            }
    std::vector<cudaStream_t> own;
    std::vector<cudaStream_t> streams(n_runs, nullptr);
    std::vector<int> next(n_runs), done(n_runs, 0);
    std::vector<bool> active(n_runs, true);
    int rc = TDSCHA_OK;
    auto fail = [&](int i, int code) {
        runs[i].status = code;
        active[i] = false;
        if (rc == TDSCHA_OK) rc = code;
    };
    for (int i = 0; i < n_runs && rc == TDSCHA_OK; ++i) {
        if (cudaStreamCreateWithFlags(&streams[i], cudaStreamNonBlocking) != cudaSuccess) {
            set_error("lanczos_run_batch: cannot create a stream");
            rc = TDSCHA_ERR_CUDA;
            break;
        }
        own.push_back(streams[i]);
        tdscha_run &r = runs[i];
        int b = r.kind == 0
                    ? lz_begin((tdscha_ctx *)r.ctx, r.basis_Q, r.basis_P,
                               basis_stride((tdscha_ctx *)r.ctx), r.capacity, r.start_step,
                               r.run_simm, r.reorth, r.hist, streams[i])
                    : qz_begin((tdscha_qctx *)r.ctx, r.basis_Q, r.capacity, r.start_step, r.reorth,
                               r.hist, streams[i]);
        if (b != TDSCHA_OK) fail(i, b);
        next[i] = r.start_step;
        if (r.n_iter == 0) active[i] = false;
    }
    while (rc == TDSCHA_OK) {
        bool any = false;
        for (int i = 0; i < n_runs; ++i) {
            if (!active[i]) continue;
            any = true;
            tdscha_run &r = runs[i];
            int todo = std::min(kSyncEvery, r.n_iter - done[i]);
            for (int t = 0; t < todo; ++t) {
                int k = r.start_step + done[i] + t;
                int e = r.kind == 0
                            ? lz_step((tdscha_ctx *)r.ctx, r.basis_Q, r.basis_P,
                                      basis_stride((tdscha_ctx *)r.ctx), r.capacity, k,
                                      r.run_simm, r.precision, r.reorth, streams[i])
                            : qz_step((tdscha_qctx *)r.ctx, r.basis_Q, r.basis_P, r.capacity, k,
                                      r.reorth, streams[i]);
                if (e != TDSCHA_OK) { fail(i, e); break; }
            }
            if (active[i]) done[i] += todo;
        }
        if (!any || rc != TDSCHA_OK) break;
        for (int i = 0; i < n_runs; ++i) {
            if (!active[i]) continue;
            tdscha_run &r = runs[i];
            int k = r.start_step + done[i] - 1;
            bool stop = false;
            double *hd = r.kind == 0 ? ((tdscha_ctx *)r.ctx)->hist_dev : ((tdscha_qctx *)r.ctx)->hist_dev;
            double *sd = r.kind == 0 ? ((tdscha_ctx *)r.ctx)->stat_dev : ((tdscha_qctx *)r.ctx)->stat_dev;
            double *sh = r.kind == 0 ? ((tdscha_ctx *)r.ctx)->stat_host : ((tdscha_qctx *)r.ctx)->stat_host;
            int e = read_back_steps(hd, sd, sh, r.capacity, next[i], k, streams[i], r.hist,
                                    r.start_step, &r.steps_done, &r.converged, &stop);
            if (e == TDSCHA_OK && r.kind == 0) e = mixed_check_error((tdscha_ctx *)r.ctx);
            if (e != TDSCHA_OK) { fail(i, e); continue; }
            next[i] = k + 1;
            if (stop || done[i] >= r.n_iter) active[i] = false;
        }
    }
    for (cudaStream_t s : own) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    return rc;
}

extern "C" int tdscha_qkpm_run(tdscha_qctx *ctx, double *vm, double *v, double *work, int n_start,
                               int n_moments, double rescale_a, double rescale_b, double *moments,
                               int *swapped, void *stream) {
    set_error("");
    if (!ctx || !vm || !v || !work || !moments || !swapped) { set_error("qkpm_run: null pointer"); return TDSCHA_ERR_ARG; }
    if (ctx->n_pairs == 0) { set_error("qkpm_run: call tdscha_qctx_set_pert first"); return TDSCHA_ERR_STATE; }
    if (n_start < 1 || n_moments < 2 || !(rescale_a != 0) || !std::isfinite(rescale_a) || !std::isfinite(rescale_b)) {
        set_error("qkpm_run: bad arguments (n_start %d, n_moments %d, a %g)", n_start, n_moments, rescale_a);
        return TDSCHA_ERR_ARG;
    }
    if (vm == v || vm == work || v == work) { set_error("qkpm_run: buffers must be distinct"); return TDSCHA_ERR_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    const long n = 2 * ctx->P;
    const int nb = std::max(1, std::min(ceil_div(n, kDotThreads), 296));
    double *a = vm, *b = v;
    *swapped = 0;
    for (int k = n_start; 2 * k < n_moments; ++k) {
        k_dot1<<<nb, kDotThreads, 0, st>>>(b, b, ctx->mask, n, ctx->dots);
        k_kpm_moment<<<1, 256, 0, st>>>(ctx->dots, nb, moments, 2 * k, 0);
        if (2 * k + 1 >= n_moments) break;
        TDS_TRY(q_apply_full_L_dev(ctx, b, work, st));
        k_kpm_combine<<<nb, kDotThreads, 0, st>>>(work, b, a, rescale_a, rescale_b, n);
        k_dot1<<<nb, kDotThreads, 0, st>>>(a, b, ctx->mask, n, ctx->dots);
        k_kpm_moment<<<1, 256, 0, st>>>(ctx->dots, nb, moments, 2 * k + 1, 1);
        TDS_CHECK_LAUNCH();
        double *t = a;   // (vm, v) <- (v, vp)
        a = b;
        b = t;
        *swapped ^= 1;
    }
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

extern "C" int tdscha_lanczos_run_hostbuf(tdscha_ctx *ctx, double *basis_Q, double *basis_P,
                                          int capacity, int start_step, int n_iter, int run_simm,
                                          int precision, int full_reorth, double *hist,
                                          int *steps_done, int *converged) {
    set_error("");
    if (!ctx || !basis_Q || !basis_P || !hist || !steps_done || !converged) {
        set_error("lanczos_run_hostbuf: null pointer");
        return TDSCHA_ERR_ARG;
    }
    if (capacity < 1 || start_step < 0 || n_iter < 0 || start_step + 1 > capacity) {
        set_error("lanczos_run_hostbuf: bad capacity %d / start %d / n_iter %d", capacity, start_step, n_iter);
        return TDSCHA_ERR_ARG;
    }
    const long P = ctx->P;
    const size_t row = sizeof(double) * P;
    // device rows padded to 32 doubles (256 bytes): the re-biorthogonalisation
    // then reads two elements per load
    const long ld = (P + 31) / 32 * 32;
    const size_t pitch = sizeof(double) * ld;
    double *dQ = nullptr, *dP = nullptr;
    int rc = TDSCHA_OK;
    auto cleanup = [&]() { if (dQ) cudaFree(dQ); if (dP) cudaFree(dP); };
    if (cudaMalloc(&dQ, pitch * capacity) != cudaSuccess || cudaMalloc(&dP, pitch * capacity) != cudaSuccess) {
        cleanup();
        set_error("lanczos_run_hostbuf: cannot allocate %zu bytes for the basis", 2 * pitch * capacity);
        return TDSCHA_ERR_CUDA;
    }
    if (cudaMemcpy2D(dQ, pitch, basis_Q, row, row, start_step + 1, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy2D(dP, pitch, basis_P, row, row, start_step + 1, cudaMemcpyHostToDevice) != cudaSuccess) {
        cleanup();
        set_error("lanczos_run_hostbuf: %s", cudaGetErrorString(cudaGetLastError()));
        return TDSCHA_ERR_CUDA;
    }
    rc = lz_run(ctx, dQ, dP, ld, capacity, start_step, n_iter, run_simm, precision, full_reorth,
                hist, steps_done, converged, 0);
    int nrows = *steps_done - (*converged ? 1 : 0);   // new basis rows written
    if (nrows > 0) {
        const size_t r0 = (size_t)(start_step + 1);
        if (cudaMemcpy2D(basis_Q + r0 * P, row, dQ + r0 * ld, pitch, row, nrows, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy2D(basis_P + r0 * P, row, dP + r0 * ld, pitch, row, nrows, cudaMemcpyDeviceToHost) != cudaSuccess) {
            if (rc == TDSCHA_OK) {
                set_error("lanczos_run_hostbuf: %s", cudaGetErrorString(cudaGetLastError()));
                rc = TDSCHA_ERR_CUDA;
            }
        }
    }
    cleanup();
    return rc;
}
