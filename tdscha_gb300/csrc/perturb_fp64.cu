// Float64 perturbation averages on the CUDA cores.
//
// The three reference loops (get_f_average_from_Y_pert_sym_fast,
// get_d2v_dR2_from_R_pert_sym_fast, get_d2v_dR2_from_Y_pert_sym_fast,
// CModules/LanczosFunctions.c:2082-2754) are rewritten in GEMM form over the
// image rows r = (i, j) with d = S_j X_i, f = S_j Y_i, u = f_Y*d, g = f_psi*f:
//
//   v_r = Y1 d_r            q_r = d_r.v_r     p_r = g_r.v_r       (stage A)
//   s_r = u_r.R1            t_r = f_r.R1
//   alpha_r = rho_i (s_r/3 - [D4] q_r/8)   beta_r = rho_i (t_r/3 - [D4] p_r/4)
//   f_avg   = (1/(S sum rho)) sum_r rho_i (-(q_r/6) f_r - (p_r/3) u_r)
//   G       = sum_r u_r w_r^T,  w_r = alpha_r f_r + (beta_r/2) u_r    (stage B)
//   d2v     = -(G + G^T) / (S sum rho)
//
// which is the reference's sum of rank-2 (u f^T + f u^T) and rank-1 (u u^T)
// updates regrouped into one M x M product with K = N*S.  Work per call:
// 4 N S M^2 flops.  All reductions are split into fixed partial buffers and
// summed in a fixed order, so results are bit-reproducible run to run.
#include "common.cuh"

namespace tdscha {

constexpr int kT = 64;     // output tile (rows x cols)
constexpr int kBK = 16;    // K step

// Stage A: per 64-row x 64-column tile of V = D Y1, partial row dots with d
// and g over the tile's columns.  qp_part[(ct*2 + 0)*R + r] = q partial,
// [(ct*2 + 1)*R + r] = p partial.  blockIdx.z = j selects the perturbation
// image: Y1 the j-th of consecutive M x M matrices, partials at j*nct*2*R.
__global__ void __launch_bounds__(256) k_stageA64(const double *__restrict__ D,
                                                  const double *__restrict__ F,
                                                  const double *__restrict__ Y1,
                                                  const double *__restrict__ fpsi, int M,
                                                  long R, double *__restrict__ qp_part) {
    Y1 += blockIdx.z * (long)M * M;
    qp_part += blockIdx.z * (long)gridDim.y * 2 * R;
    __shared__ double As[kBK][kT + 1];
    __shared__ double Bs[kBK][kT];
    int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    long r0 = (long)blockIdx.x * kT;
    int c0 = blockIdx.y * kT;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < M; k0 += kBK) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int e = tid + 256 * t;
            int rr = e >> 4, kk = e & 15;
            long r = r0 + rr;
            int k = k0 + kk;
            As[kk][rr] = (r < R && k < M) ? D[r * M + k] : 0.0;
            int kb = e >> 6, cc = e & 63;
            int kr = k0 + kb, c = c0 + cc;
            Bs[kb][cc] = (kr < M && c < M) ? Y1[(long)kr * M + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        long r = r0 + ty * 4 + i;
        double pq = 0, pp = 0;
        if (r < R) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int c = c0 + tx * 4 + j;
                if (c < M) {
                    pq = fma(D[r * M + c], acc[i][j], pq);
                    pp = fma(fpsi[c] * F[r * M + c], acc[i][j], pp);
                }
            }
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            pq += __shfl_xor_sync(0xffffffffu, pq, o);
            pp += __shfl_xor_sync(0xffffffffu, pp, o);
        }
        if (tx == 0 && r < R) {
            qp_part[(long)(blockIdx.y * 2 + 0) * R + r] = pq;
            qp_part[(long)(blockIdx.y * 2 + 1) * R + r] = pp;
        }
    }
}

// Row scalars: one warp per image row.
__global__ void k_rows64(const double *__restrict__ D, const double *__restrict__ F,
                         const double *__restrict__ fY, const double *__restrict__ R1,
                         const double *__restrict__ rho, const double *__restrict__ qp_part,
                         int nct, int M, int S, long R, int apply_d4,
                         double *__restrict__ alpha, double *__restrict__ beta,
                         double *__restrict__ c1, double *__restrict__ c2) {
    int lane = threadIdx.x & 31;
    long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= R) return;
    double s = 0, t = 0;
    for (int m = lane; m < M; m += 32) {
        s = fma(fY[m] * R1[m], D[r * M + m], s);
        t = fma(R1[m], F[r * M + m], t);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    if (lane == 0) {
        double q = 0, p = 0;
        for (int ct = 0; ct < nct; ++ct) {
            q += qp_part[(long)(ct * 2 + 0) * R + r];
            p += qp_part[(long)(ct * 2 + 1) * R + r];
        }
        double rw = rho[r / S];
        double d4 = apply_d4 ? 1.0 : 0.0;
        alpha[r] = rw * (s / 3 - d4 * q / 8);
        beta[r] = rw * (t / 3 - d4 * p / 4);
        c1[r] = -rw * q / 6;
        c2[r] = -rw * p / 3;
    }
}

// Row scalars of the pairs (configuration i, perturbation image j), one warp
// per pair r = j*N + i: s = x_i . vs_j, t = y_i . vt_j (vs_j = S_j^T (f_Y R1),
// vt_j = S_j^T R1), q, p from the stage A partials of image j.
__global__ void k_rows64_img(const double *__restrict__ D, const double *__restrict__ F,
                             const double *__restrict__ vs, const double *__restrict__ vt,
                             const double *__restrict__ rho, const double *__restrict__ qp_part,
                             int nct, int M, long N, int J, int apply_d4,
                             double *__restrict__ alpha, double *__restrict__ beta,
                             double *__restrict__ c1, double *__restrict__ c2) {
    int lane = threadIdx.x & 31;
    long r = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= (long)J * N) return;
    long j = r / N, i = r - j * N;
    const double *x = D + i * M, *y = F + i * M, *a = vs + j * M, *b = vt + j * M;
    double s = 0, t = 0;
    for (int m = lane; m < M; m += 32) {
        s = fma(a[m], x[m], s);
        t = fma(b[m], y[m], t);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    if (lane == 0) {
        double q = 0, p = 0;
        const double *qp = qp_part + j * nct * 2 * N;
        for (int ct = 0; ct < nct; ++ct) {
            q += qp[(long)(ct * 2 + 0) * N + i];
            p += qp[(long)(ct * 2 + 1) * N + i];
        }
        double rw = rho[i];
        double d4 = apply_d4 ? 1.0 : 0.0;
        alpha[r] = rw * (s / 3 - d4 * q / 8);
        beta[r] = rw * (t / 3 - d4 * p / 4);
        c1[r] = -rw * q / 6;
        c2[r] = -rw * p / 3;
    }
}

// f partials: fpart[chunk][m] = sum_{r in chunk} c1_r f_r[m] + c2_r u_r[m].
// blockIdx.z = j: row scalars of perturbation image j (at j*R), partials at
// j*nchunk*M.
__global__ void k_favg64(const double *__restrict__ D, const double *__restrict__ F,
                         const double *__restrict__ fY, const double *__restrict__ c1,
                         const double *__restrict__ c2, int M, long R, long chunk,
                         double *__restrict__ fpart) {
    c1 += blockIdx.z * R;
    c2 += blockIdx.z * R;
    fpart += (long)blockIdx.z * gridDim.y * M;
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    long rb = (long)blockIdx.y * chunk, re = min(R, rb + chunk);
    double fy = fY[m], acc = 0;
    for (long r = rb; r < re; ++r) {
        acc = fma(c1[r], F[r * M + m], acc);
        acc = fma(c2[r], fy * D[r * M + m], acc);
    }
    fpart[(long)blockIdx.y * M + m] = acc;
}

// Stage B: split-K partial of G = U^T W over the rows of one chunk.
// blockIdx.z = j: alpha, beta of perturbation image j (at j*R), partial tiles
// at (j*nsplit + split)*M*M.
__global__ void __launch_bounds__(256) k_stageB64(const double *__restrict__ D,
                                                  const double *__restrict__ F,
                                                  const double *__restrict__ fY,
                                                  const double *__restrict__ alpha,
                                                  const double *__restrict__ beta, int M,
                                                  long R, long chunk, int ntile,
                                                  double *__restrict__ gpart) {
    alpha += blockIdx.z * R;
    beta += blockIdx.z * R;
    gpart += (long)blockIdx.z * gridDim.y * M * M;
    __shared__ double As[kBK][kT];
    __shared__ double Bs[kBK][kT];
    int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    int ta = blockIdx.x / ntile, tb = blockIdx.x % ntile;
    int a0 = ta * kT, b0 = tb * kT;
    long rb = (long)blockIdx.y * chunk, re = min(R, rb + chunk);
    double acc[4][4] = {};
    for (long k0 = rb; k0 < re; k0 += kBK) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int e = tid + 256 * t;
            int kk = e >> 6, cc = e & 63;
            long r = k0 + kk;
            int a = a0 + cc, b = b0 + cc;
            double ua = 0, wb = 0;
            if (r < re) {
                if (a < M) ua = fY[a] * D[r * M + a];
                if (b < M) wb = alpha[r] * F[r * M + b] + 0.5 * beta[r] * (fY[b] * D[r * M + b]);
            }
            As[kk][cc] = ua;
            Bs[kk][cc] = wb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    double *g = gpart + (long)blockIdx.y * M * M;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int a = a0 + ty * 4 + i;
        if (a >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int b = b0 + tx * 4 + j;
            if (b < M) g[(long)a * M + b] = acc[i][j];
        }
    }
}

// d2v = -(G + G^T)/(S sum rho) and f = sum fpart / (S sum rho); G given as
// nsplit partials of element type T (double for this path, float for the
// tensor-core path) with leading dimension ld.
template <typename T>
__global__ void k_finalize(const T *__restrict__ gpart, int nsplit, long split_stride, int ld,
                           const double *__restrict__ fpart, int nfchunk, int M, double norm,
                           double *__restrict__ f, double *__restrict__ d2v) {
    long n = (long)M * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e / M), b = (int)(e % M);
        double gab = 0, gba = 0;
        for (int s = 0; s < nsplit; ++s) {
            gab += (double)gpart[s * split_stride + (long)a * ld + b];
            gba += (double)gpart[s * split_stride + (long)b * ld + a];
        }
        d2v[e] = -(gab + gba) / norm;
        if (e < M) {
            double acc = 0;
            for (int ch = 0; ch < nfchunk; ++ch) acc += fpart[(long)ch * M + e];
            f[e] = acc / norm;
        }
    }
}

int alloc_fp64_scratch(tdscha_ctx *c) {
    int M = c->M;
    long R = c->R;          // (configuration, image) pairs
    long Nr = c->Nrows;     // rows of D, F (R, or N with perturbation-side images)
    const int J = c->J;
    c->nct64 = ceil_div(M, kT);
    int ntile = ceil_div(M, kT);
    int tiles = ntile * ntile;
    // split-K: the float64 pipe (about 2 FMA per cycle per SM) bounds stage B,
    // so every SM should get the same share of tiles x splits.  At least two
    // blocks per SM and 64 rows per split as before; above that minimum, up
    // to 64 splits, the count whose blocks fill whole rounds of 152 SMs best
    // (ties: fewer splits, less partial-tile traffic).
    const long n_hi = std::max<long>(1, std::min<long>(64, Nr / 64));
    const long n_lo = std::min<long>(n_hi, ceil_div(2 * 152, (long)tiles * J));
    int ns = (int)n_lo;
    {
        double best = -1;
        for (long n = n_lo; n <= n_hi; ++n) {
            long blocks = (long)tiles * J * n;
            double fill = (double)blocks / (double)(ceil_div(blocks, 152) * 152L);
            if (fill > best + 1e-9) {
                best = fill;
                ns = (int)n;
            }
        }
    }
    c->nsplit64 = ns;
    c->nfchunk = (int)std::min<long>(std::max<long>(1, Nr / 256), 512);
    TDS_CUDA(cached_malloc(&c->qp_part, sizeof(double) * 2 * c->nct64 * R));
    TDS_CUDA(cached_malloc(&c->alpha, sizeof(double) * R));
    TDS_CUDA(cached_malloc(&c->beta, sizeof(double) * R));
    TDS_CUDA(cached_malloc(&c->c1, sizeof(double) * R));
    TDS_CUDA(cached_malloc(&c->c2, sizeof(double) * R));
    TDS_CUDA(cached_malloc(&c->gpart, sizeof(double) * (size_t)J * ns * M * M));
    TDS_CUDA(cached_malloc(&c->fpart, sizeof(double) * (size_t)J * c->nfchunk * M));
    return TDSCHA_OK;
}

// f partials and row scalars shared by both precisions: given q, p partials
// in qp (nct tiles) this fills alpha/beta/c1/c2 and fpart.
int rows_and_favg64(tdscha_ctx *c, int apply_d4, cudaStream_t st) {
    int M = c->M;
    long R = c->R;
    ProfScope ps(c, 1, st);
    k_rows64<<<ceil_div(R, 8), 256, 0, st>>>(c->D, c->F, c->fY, c->R1, c->rho, c->qp_part,
                                              c->nct64, M, c->S, R, apply_d4, c->alpha,
                                              c->beta, c->c1, c->c2);
    TDS_CHECK_LAUNCH();
    long fchunk = (R + c->nfchunk - 1) / c->nfchunk;
    ProfScope ps2(c, 2, st);
    k_favg64<<<dim3(ceil_div(M, 128), c->nfchunk), 128, 0, st>>>(c->D, c->F, c->fY, c->c1,
                                                                 c->c2, M, R, fchunk, c->fpart);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

int finalize_avgs(tdscha_ctx *c, int nsplit, const double *gpart, cudaStream_t st) {
    int M = c->M;
    double norm = c->sum_rho * c->S;
    int blocks = std::max(1, std::min(ceil_div((long)M * M, 256), 2048));
    ProfScope ps(c, 4, st);
    k_finalize<double><<<blocks, 256, 0, st>>>(gpart, nsplit, (long)M * M, M, c->fpart,
                                               c->nfchunk, M, norm, c->f, c->d2v);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

int finalize_avgs_f32(tdscha_ctx *c, int nsplit, const float *gpart, long split_stride, int ld,
                      cudaStream_t st) {
    int M = c->M;
    double norm = c->sum_rho * c->S;
    int blocks = std::max(1, std::min(ceil_div((long)M * M, 256), 2048));
    ProfScope ps(c, 4, st);
    k_finalize<float><<<blocks, 256, 0, st>>>(gpart, nsplit, split_stride, ld, c->fpart,
                                              c->nfchunk, M, norm, c->f, c->d2v);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

// Symmetry images on the perturbation side (symmetry.cu): the same kernels
// over the N configurations with blockIdx.z = image j, then the S_j applied
// to the J partial results.
static int perturb_fp64_img(tdscha_ctx *c, int apply_d4, cudaStream_t st) {
    const int M = c->M, J = c->J, nct = c->nct64, ns = c->nsplit64, nfc = c->nfchunk;
    const long N = c->Nrows;
    TDS_TRY(psi_perturbation64(c, st));
    {
        ProfScope ps(c, 0, st);
        k_stageA64<<<dim3(ceil_div(N, kT), nct, J), 256, 0, st>>>(c->D, c->F, c->Y1all, c->fpsi,
                                                                   M, N, c->qp_part);
        TDS_CHECK_LAUNCH();
    }
    {
        ProfScope ps(c, 1, st);
        k_rows64_img<<<ceil_div((long)J * N, 8), 256, 0, st>>>(
            c->D, c->F, c->vsv, c->vsv + (long)J * M, c->rho, c->qp_part, nct, M, N, J, apply_d4,
            c->alpha, c->beta, c->c1, c->c2);
        TDS_CHECK_LAUNCH();
    }
    {
        ProfScope ps(c, 2, st);
        long fchunk = (N + nfc - 1) / nfc;
        k_favg64<<<dim3(ceil_div(M, 128), nfc, J), 128, 0, st>>>(c->D, c->F, c->fY, c->c1, c->c2,
                                                                 M, N, fchunk, c->fpart);
        TDS_CHECK_LAUNCH();
    }
    const int ntile = ceil_div(M, kT);
    {
        ProfScope ps(c, 3, st);
        long chunk = (N + ns - 1) / ns;
        k_stageB64<<<dim3(ntile * ntile, ns, J), 256, 0, st>>>(c->D, c->F, c->fY, c->alpha,
                                                               c->beta, M, N, chunk, ntile,
                                                               c->gpart);
        TDS_CHECK_LAUNCH();
    }
    const long MM = (long)M * M;
    return psi_finalize64(c, c->gpart, ns, MM, (long)ns * MM, M, c->fpart, nfc, st);
}

int perturb_fp64(tdscha_ctx *c, int apply_d4, cudaStream_t st) {
    if (c->J > 1) return perturb_fp64_img(c, apply_d4, st);
    int M = c->M;
    long R = c->R;
    dim3 gA(ceil_div(R, kT), c->nct64);
    {
        ProfScope ps(c, 0, st);
        k_stageA64<<<gA, 256, 0, st>>>(c->D, c->F, c->Y1, c->fpsi, M, R, c->qp_part);
        TDS_CHECK_LAUNCH();
    }
    TDS_TRY(rows_and_favg64(c, apply_d4, st));
    int ntile = ceil_div(M, kT);
    long chunk = (R + c->nsplit64 - 1) / c->nsplit64;
    {
        ProfScope ps(c, 3, st);
        k_stageB64<<<dim3(ntile * ntile, c->nsplit64), 256, 0, st>>>(c->D, c->F, c->fY, c->alpha,
                                                                     c->beta, M, R, chunk, ntile,
                                                                     c->gpart);
        TDS_CHECK_LAUNCH();
    }
    return finalize_avgs(c, c->nsplit64, c->gpart, st);
}

}  // namespace tdscha
