// Symmetry images on the perturbation side.
//
// The reference forms every image row d = S_j X_i, f = S_j Y_i inside its
// loops (CModules/LanczosFunctions.c:2158-2170, :2360-2372, :2673-2685;
// Modules/tdscha_core.jl:86-87).  The symmetry matrices only mix modes of one
// degenerate block; when each of them maps only between modes of equal f_Y
// and equal f_psi (degenerate modes have equal frequencies), S_j commutes
// with diag(f_Y) and diag(f_psi), and every sum over the image rows becomes a
// sum over the N configurations of the perturbation carried to the image:
//
//   q_ij = x_i . (Y1_j x_i),        Y1_j = S_j^T Y1 S_j
//   p_ij = g_i . (Y1_j x_i),        g_i  = f_psi * y_i
//   s_ij = x_i . S_j^T (f_Y * R1),  t_ij = y_i . S_j^T R1
//   f    =  sum_j S_j [sum_i c1_ij y_i + c2_ij u_i]              / (S sum rho)
//   d2v  = -sum_j S_j (G_j + G_j^T) S_j^T                        / (S sum rho)
//   G_j  =  sum_i u_i (alpha_ij y_i + beta_ij/2 u_i)^T,          u_i = f_Y * x_i
//
// with alpha, beta, c1, c2 the reference's row scalars of image row (i, j).
// No image row is stored: stage A is one GEMM X [Y1_1 ... Y1_S] that reads
// the ensemble once for all images, stage B weights the same rows once per
// image, and the S_j act only on M-vectors and M x M matrices.  Contexts
// whose symmetry tables do not commute with the frequency factors (or with
// TDSCHA_SYMMETRY_IMAGES=rows in the environment) keep the image rows.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "common.cuh"
#include "dfloat.cuh"

namespace tdscha {

// vs[j][m] = (S_j^T (f_Y R1))[m], vt[j][m] = (S_j^T R1)[m]
__global__ void k_psi_vec(const int *__restrict__ sc_idx, const double *__restrict__ sc_val,
                          const double *__restrict__ fY, const double *__restrict__ R1, int J,
                          int M, int md, double *__restrict__ vs, double *__restrict__ vt) {
    long n = (long)J * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int *ix = sc_idx + e * md;
        const double *vv = sc_val + e * md;
        double a = 0, b = 0;
        for (int k = 0; k < md; ++k) {
            int r = ix[k];
            if (r < 0) break;
            a = fma(vv[k], fY[r] * R1[r], a);
            b = fma(vv[k], R1[r], b);
        }
        vs[e] = a;
        vt[e] = b;
    }
}

// Y1all[j][a][b] = sum_{k, l} S_j[k][a] Y1[k][l] S_j[l][b] (Y1 symmetric)
__global__ void k_psi_y1(const int *__restrict__ sc_idx, const double *__restrict__ sc_val,
                         const double *__restrict__ Y1, int J, int M, int md,
                         double *__restrict__ Y1all) {
    long MM = (long)M * M, n = (long)J * MM;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        long j = e / MM;
        int a = (int)((e - j * MM) / M), b = (int)(e % M);
        const int *ia = sc_idx + (j * M + a) * md, *ib = sc_idx + (j * M + b) * md;
        const double *va = sc_val + (j * M + a) * md, *vb = sc_val + (j * M + b) * md;
        double acc = 0;
        for (int p = 0; p < md && ia[p] >= 0; ++p) {
            double inner = 0;
            const double *row = Y1 + (long)ia[p] * M;
            for (int q = 0; q < md && ib[q] >= 0; ++q) inner = fma(vb[q], row[ib[q]], inner);
            acc = fma(va[p], inner, acc);
        }
        Y1all[e] = acc;
    }
}

// sum_s p[s * stride] in float64, in split order, eight loads in flight
// (the sums are load-latency bound)
template <typename T>
__device__ __forceinline__ double split_sum(const T *__restrict__ p, int n, long stride) {
    double acc = 0;
    int s = 0;
    for (; s + 8 <= n; s += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = p[(long)(s + u) * stride];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += (double)v[u];
    }
    for (; s < n; ++s) acc += (double)p[(long)s * stride];
    return acc;
}

// hs[j][k][l] = hs[j][l][k] = sum_s G_js[k][l] + sum_s G_js[l][k], with
// G_js[k][l] = g[s*ss + j*js + k*lda + l], each sum in float64 in split order.
// One block per pair of 32 x 32 tiles (K <= L, upper triangle) and image: the
// tile (K, L) and its mirror (L, K) are each read once, summed over the splits
// into shared memory, and both halves of the symmetric result written along
// rows.  Blocks of the first tile pair row also form
// fs[j][m] = sum_ch fpart[(j*nfc + ch)*M + m] for their columns.
template <typename T>
__global__ void __launch_bounds__(256) k_psi_hsum(const T *__restrict__ g, int nsplit, long ss,
                                                  long js, long lda, const T *__restrict__ fpart,
                                                  int nfc, int M, double *__restrict__ hs,
                                                  double *__restrict__ fs) {
    __shared__ double t1[32][33], t2[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;    // 32 x 8
    const int nt = (M + 31) / 32;
    int K = 0, rem = blockIdx.x;
    while (rem >= nt - K) {
        rem -= nt - K;
        ++K;
    }
    const int L = K + rem;
    const int k0 = K * 32, l0 = L * 32;
    const long j = blockIdx.y;
    const T *base = g + j * js;
    for (int r = ty; r < 32; r += 8) {
        int k = k0 + r, l = l0 + tx;
        t1[r][tx] = (k < M && l < M) ? split_sum(base + (long)k * lda + l, nsplit, ss) : 0.0;
        if (K != L) {
            int l2 = l0 + r, k2 = k0 + tx;
            t2[r][tx] = (l2 < M && k2 < M) ? split_sum(base + (long)l2 * lda + k2, nsplit, ss) : 0.0;
        }
    }
    __syncthreads();
    double(*m2)[33] = K != L ? t2 : t1;     // m2[l - l0][k - k0] = sum_s G[l][k]
    double *H = hs + j * (long)M * M;
    for (int r = ty; r < 32; r += 8) {
        int k = k0 + r, l = l0 + tx;        // rows of tile (K, L)
        if (k < M && l < M) H[(long)k * M + l] = t1[r][tx] + m2[tx][r];
        if (K != L) {
            int l2 = l0 + r, k2 = k0 + tx;  // rows of the mirror tile (L, K)
            if (l2 < M && k2 < M) H[(long)l2 * M + k2] = t1[tx][r] + m2[r][tx];
        }
    }
    if (K == 0 && ty == 0) {
        int m = l0 + tx;
        if (m < M) fs[j * M + m] = split_sum(fpart + j * nfc * M + m, nfc, M);
    }
}

// Per image: tj[j][a][b] = sum_{k, l} S_j[a][k] hs[j][k][l] S_j[b][l] and
// tf[j][a] = sum_k S_j[a][k] fs[j][k].
__global__ void k_psi_sandwich(const int *__restrict__ sr_idx, const double *__restrict__ sr_val,
                               const double *__restrict__ hs, const double *__restrict__ fs,
                               int J, int M, int md, double *__restrict__ tj,
                               double *__restrict__ tf) {
    const long MM = (long)M * M, n = (long)J * MM;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long j = e / MM;
        const int a = (int)((e - j * MM) / M), b = (int)(e % M);
        const int *ia = sr_idx + (j * M + a) * md, *ib = sr_idx + (j * M + b) * md;
        const double *va = sr_val + (j * M + a) * md, *vb = sr_val + (j * M + b) * md;
        const double *H = hs + j * MM;
        double acc = 0, facc = 0;
        for (int p = 0; p < md && ia[p] >= 0; ++p) {
            double inner = 0;
            const double *row = H + (long)ia[p] * M;
            for (int q = 0; q < md && ib[q] >= 0; ++q) inner = fma(vb[q], row[ib[q]], inner);
            acc = fma(va[p], inner, acc);
            if (b == 0) facc = fma(va[p], fs[j * M + ia[p]], facc);
        }
        tj[e] = acc;
        if (b == 0) tf[j * M + a] = facc;
    }
}

// d2v[a][b] = -inv sum_j tj[j][a][b], f[a] = inv sum_j tf[j][a], in image order.
__global__ void k_psi_jsum(const double *__restrict__ tj, const double *__restrict__ tf, int J,
                           int M, double inv, double *__restrict__ f, double *__restrict__ d2v) {
    const long MM = (long)M * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < MM; e += (long)gridDim.x * blockDim.x) {
        d2v[e] = -split_sum(tj + e, J, MM) * inv;
        if (e < M) f[e] = split_sum(tf + e, J, (long)M) * inv;
    }
}

// ---------------------------------------------------------------------------
// The mixed path's finalisation in double-float (dfloat.cuh).  The float64
// forms above spend a float32 -> float64 conversion and a float64 add per
// split partial (J M^2 nsplit of them: 17 M at M = 189, 48 images, 10 splits),
// which kept k_psi_hsum on the float64 pipe at about 0.5 operations per clock
// per SM; here every sum up to d2v itself runs on float32 pairs.

// sum_s p[s * stride] as a normalised double-float pair, split order, eight
// loads in flight
__device__ __forceinline__ float2 split_sum_df(const float *__restrict__ p, int n, long stride) {
    float s = 0.f, c = 0.f;
    int k = 0;
    for (; k + 8 <= n; k += 8) {
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = p[(long)(k + u) * stride];
#pragma unroll
        for (int u = 0; u < 8; ++u) df_two_sum_acc(s, c, v[u]);
    }
    for (; k < n; ++k) df_two_sum_acc(s, c, p[(long)k * stride]);
    return df_norm(s, c);
}

// k_psi_hsum for float partials: the same tile pairs, hs2 and fs2 as
// double-float pairs
__global__ void __launch_bounds__(256) k_psi_hsum_df(const float *__restrict__ g, int nsplit,
                                                     long ss, long js, long lda,
                                                     const float *__restrict__ fpart, int nfc,
                                                     int M, float2 *__restrict__ hs,
                                                     float2 *__restrict__ fs) {
    __shared__ float2 t1[32][33], t2[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;    // 32 x 8
    const int nt = (M + 31) / 32;
    int K = 0, rem = blockIdx.x;
    while (rem >= nt - K) {
        rem -= nt - K;
        ++K;
    }
    const int L = K + rem;
    const int k0 = K * 32, l0 = L * 32;
    const long j = blockIdx.y;
    const float *base = g + j * js;
    const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        int k = k0 + r, l = l0 + tx;
        t1[r][tx] = (k < M && l < M) ? split_sum_df(base + (long)k * lda + l, nsplit, ss) : zero;
        if (K != L) {
            int l2 = l0 + r, k2 = k0 + tx;
            t2[r][tx] = (l2 < M && k2 < M) ? split_sum_df(base + (long)l2 * lda + k2, nsplit, ss) : zero;
        }
    }
    __syncthreads();
    float2(*m2)[33] = K != L ? t2 : t1;     // m2[l - l0][k - k0] = sum_s G[l][k]
    float2 *H = hs + j * (long)M * M;
    for (int r = ty; r < 32; r += 8) {
        int k = k0 + r, l = l0 + tx;        // rows of tile (K, L)
        if (k < M && l < M) H[(long)k * M + l] = df_add(t1[r][tx], m2[tx][r]);
        if (K != L) {
            int l2 = l0 + r, k2 = k0 + tx;  // rows of the mirror tile (L, K)
            if (l2 < M && k2 < M) H[(long)l2 * M + k2] = df_add(t1[tx][r], m2[r][tx]);
        }
    }
    if (K == 0 && ty == 0) {
        int m = l0 + tx;
        if (m < M) fs[j * M + m] = split_sum_df(fpart + j * nfc * M + m, nfc, M);
    }
}

// k_psi_sandwich in double-float: tj[j][a][b] = sum_{k,l} S_j[a][k] hs[j][k][l] S_j[b][l],
// tf[j][a] = sum_k S_j[a][k] fs[j][k]
__global__ void k_psi_sandwich_df(const int *__restrict__ sr_idx, const float2 *__restrict__ sr_val,
                                  const float2 *__restrict__ hs, const float2 *__restrict__ fs,
                                  int J, int M, int md, float2 *__restrict__ tj,
                                  float2 *__restrict__ tf) {
    const long MM = (long)M * M, n = (long)J * MM;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const long j = e / MM;
        const int a = (int)((e - j * MM) / M), b = (int)(e % M);
        const int *ia = sr_idx + (j * M + a) * md, *ib = sr_idx + (j * M + b) * md;
        const float2 *va = sr_val + (j * M + a) * md, *vb = sr_val + (j * M + b) * md;
        const float2 *H = hs + j * MM;
        float as = 0.f, ac = 0.f, fs_ = 0.f, fc = 0.f;
        for (int p = 0; p < md && ia[p] >= 0; ++p) {
            float is = 0.f, ic = 0.f;
            const float2 *row = H + (long)ia[p] * M;
            for (int q = 0; q < md && ib[q] >= 0; ++q) df_fma_acc(is, ic, vb[q], row[ib[q]]);
            df_fma_acc(as, ac, va[p], df_norm(is, ic));
            if (b == 0) df_fma_acc(fs_, fc, va[p], fs[j * M + ia[p]]);
        }
        tj[e] = df_norm(as, ac);
        if (b == 0) tf[j * M + a] = df_norm(fs_, fc);
    }
}

// d2v[a][b] = -inv sum_j tj[j][a][b], f[a] = inv sum_j tf[j][a]: block (64, 4),
// thread (x, y) sums the images j = y, y + 4, ... of element blockIdx.x * 64 + x,
// and the four partial sums are added in y order.
__global__ void __launch_bounds__(256) k_psi_jsum_df(const float2 *__restrict__ tj,
                                                     const float2 *__restrict__ tf, int J, int M,
                                                     double inv, double *__restrict__ f,
                                                     double *__restrict__ d2v) {
    __shared__ float2 red[2][4][64];
    const long MM = (long)M * M;
    const int x = threadIdx.x, y = threadIdx.y;
    const long e = blockIdx.x * 64L + x;
    float s = 0.f, c = 0.f, s2 = 0.f, c2 = 0.f;
    if (e < MM)
        for (int j = y; j < J; j += 4) {
            const float2 v = tj[j * MM + e];
            df_two_sum_acc(s, c, v.x);
            c += v.y;
        }
    if (e < M)
        for (int j = y; j < J; j += 4) {
            const float2 v = tf[(long)j * M + e];
            df_two_sum_acc(s2, c2, v.x);
            c2 += v.y;
        }
    red[0][y][x] = df_norm(s, c);
    red[1][y][x] = df_norm(s2, c2);
    __syncthreads();
    if (y == 0 && e < MM) {
        float2 t = red[0][0][x], u = red[1][0][x];
        for (int k = 1; k < 4; ++k) {
            t = df_add(t, red[0][k][x]);
            u = df_add(u, red[1][k][x]);
        }
        d2v[e] = -df_to_double(t) * inv;
        if (e < M) f[e] = df_to_double(u) * inv;
    }
}

static int grid_for(long n) { return (int)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 16)); }

int psi_setup(tdscha_ctx *c, int n_blocks, const int *n_deg, const int *deg_space,
              const double *sym, const int *blocks_ids, const std::vector<double> &fy,
              const std::vector<double> &fp) {
    const int M = c->M, S = c->S;
    c->J = 1;
    c->maxdeg = 1;
    if (S <= 1) return TDSCHA_OK;
    const char *mode = getenv("TDSCHA_SYMMETRY_IMAGES");
    if (mode && !strcmp(mode, "rows")) return TDSCHA_OK;
    std::vector<int> off(n_blocks);
    std::vector<long> soff(n_blocks);
    int md = 1;
    for (int b = 0, acc = 0; b < n_blocks; ++b) {
        off[b] = acc;
        acc += n_deg[b];
        md = std::max(md, n_deg[b]);
    }
    for (int b = 1; b < n_blocks; ++b) soff[b] = soff[b - 1] + (long)S * n_deg[b - 1] * n_deg[b - 1];
    // row-sparse S_j: row mu from block blocks_ids[mu], mu_id = mu - space[0]
    // (the reference's convention, LanczosFunctions.c:2158-2170)
    const size_t cells = (size_t)S * M * md;
    std::vector<int> ri(cells, -1), ci(cells, -1);
    std::vector<double> rv(cells, 0.0), cv(cells, 0.0);
    std::vector<int> ccount((size_t)S * M, 0);
    for (int j = 0; j < S; ++j)
        for (int mu = 0; mu < M; ++mu) {
            int b = blocks_ids[mu], bd = n_deg[b];
            const int *space = deg_space + off[b];
            int mu_id = mu - space[0];
            const double *row = sym + soff[b] + ((long)j * bd + mu_id) * bd;
            int nr = 0;
            for (int k = 0; k < bd; ++k) {
                if (row[k] == 0.0) continue;
                int nu = space[k];
                // the images must not mix modes of different f_Y or f_psi
                if (fy[mu] != fy[nu] || fp[mu] != fp[nu]) return TDSCHA_OK;
                size_t rs = ((size_t)j * M + mu) * md + nr++;
                ri[rs] = nu;
                rv[rs] = row[k];
                int &cnt = ccount[(size_t)j * M + nu];
                if (cnt >= md) return TDSCHA_OK;   // overlapping blocks: keep image rows
                size_t cs = ((size_t)j * M + nu) * md + cnt++;
                ci[cs] = mu;
                cv[cs] = row[k];
            }
        }
    TDS_CUDA(cached_malloc(&c->sr_idx, sizeof(int) * cells));
    TDS_CUDA(cached_malloc(&c->sc_idx, sizeof(int) * cells));
    TDS_CUDA(cached_malloc(&c->sr_val, sizeof(double) * cells));
    TDS_CUDA(cached_malloc(&c->sc_val, sizeof(double) * cells));
    TDS_CUDA(cudaMemcpy(c->sr_idx, ri.data(), sizeof(int) * cells, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemcpy(c->sc_idx, ci.data(), sizeof(int) * cells, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemcpy(c->sr_val, rv.data(), sizeof(double) * cells, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemcpy(c->sc_val, cv.data(), sizeof(double) * cells, cudaMemcpyHostToDevice));
    // double-float copies of the row- and column-sparse values for the mixed
    // path's finalisation and image preparation
    std::vector<float2> rv2(cells);
    for (size_t i = 0; i < cells; ++i) {
        float hi = (float)rv[i];
        rv2[i] = make_float2(hi, (float)(rv[i] - (double)hi));
    }
    TDS_CUDA(cached_malloc(&c->sr_val2, sizeof(float2) * cells));
    TDS_CUDA(cudaMemcpy(c->sr_val2, rv2.data(), sizeof(float2) * cells, cudaMemcpyHostToDevice));
    for (size_t i = 0; i < cells; ++i) {
        float hi = (float)cv[i];
        rv2[i] = make_float2(hi, (float)(cv[i] - (double)hi));
    }
    TDS_CUDA(cached_malloc(&c->sc_val2, sizeof(float2) * cells));
    TDS_CUDA(cudaMemcpy(c->sc_val2, rv2.data(), sizeof(float2) * cells, cudaMemcpyHostToDevice));
    TDS_CUDA(cached_malloc(&c->vsv, sizeof(double) * 2 * (size_t)S * M));
    // hs and tj (J x M x M each), fs and tf (J x M each)
    TDS_CUDA(cached_malloc(&c->hs, sizeof(double) * 2 * ((size_t)S * M * M + (size_t)S * M)));
    c->J = S;
    c->maxdeg = md;
    return TDSCHA_OK;
}

void psi_free(tdscha_ctx *c) {
    cached_free(c->sr_idx);
    cached_free(c->sc_idx);
    cached_free(c->sr_val);
    cached_free(c->sc_val);
    cached_free(c->sr_val2);
    cached_free(c->sc_val2);
    c->sr_val2 = c->sc_val2 = nullptr;
    cached_free(c->Y1all);
    cached_free(c->vsv);
    cached_free(c->hs);
    c->sr_idx = c->sc_idx = nullptr;
    c->sr_val = c->sc_val = c->Y1all = c->vsv = c->hs = nullptr;
}

int psi_perturbation64(tdscha_ctx *c, cudaStream_t st) {
    const int M = c->M, J = c->J, md = c->maxdeg;
    k_psi_vec<<<grid_for((long)J * M), 256, 0, st>>>(c->sc_idx, c->sc_val, c->fY, c->R1, J, M, md,
                                                     c->vsv, c->vsv + (long)J * M);
    TDS_CHECK_LAUNCH();
    if (!c->Y1all) TDS_CUDA(cached_malloc(&c->Y1all, sizeof(double) * (size_t)J * M * M));
    k_psi_y1<<<grid_for((long)J * M * M), 256, 0, st>>>(c->sc_idx, c->sc_val, c->Y1, J, M, md,
                                                        c->Y1all);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

template <typename T>
static int psi_finalize(tdscha_ctx *c, const T *gpart, int nsplit, long sstride, long jstride,
                        long lda, const T *fpart, int nfchunk, cudaStream_t st) {
    const int M = c->M, J = c->J;
    const size_t JMM = (size_t)J * M * M, JM = (size_t)J * M;
    double *hs = c->hs, *tj = hs + JMM, *fs = tj + JMM, *tf = fs + JM;
    ProfScope ps(c, 4, st);
    const int nt = ceil_div(M, 32);
    dim3 gt(nt * (nt + 1) / 2, J);
    k_psi_hsum<T><<<gt, 256, 0, st>>>(gpart, nsplit, sstride, jstride, lda, fpart, nfchunk, M, hs,
                                      fs);
    TDS_CHECK_LAUNCH();
    k_psi_sandwich<<<grid_for((long)JMM), 256, 0, st>>>(c->sr_idx, c->sr_val, hs, fs, J, M,
                                                        c->maxdeg, tj, tf);
    TDS_CHECK_LAUNCH();
    k_psi_jsum<<<std::max(1, ceil_div((long)M * M, 64)), 64, 0, st>>>(
        tj, tf, J, M, 1.0 / (c->sum_rho * c->S), c->f, c->d2v);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

int psi_finalize64(tdscha_ctx *c, const double *gpart, int nsplit, long sstride, long jstride,
                   long lda, const double *fpart, int nfchunk, cudaStream_t st) {
    return psi_finalize<double>(c, gpart, nsplit, sstride, jstride, lda, fpart, nfchunk, st);
}

int psi_finalize32(tdscha_ctx *c, const float *gpart, int nsplit, long sstride, long jstride,
                   long lda, const float *fpart, int nfchunk, double *f_out, double *d2v_out,
                   cudaStream_t st) {
    const int M = c->M, J = c->J;
    const size_t JMM = (size_t)J * M * M, JM = (size_t)J * M;
    // the float64 layout of hs, tj, fs, tf holds the double-float pairs
    float2 *hs = reinterpret_cast<float2 *>(c->hs), *tj = hs + JMM, *fs = tj + JMM, *tf = fs + JM;
    ProfScope ps(c, 4, st);
    const int nt = ceil_div(M, 32);
    dim3 gt(nt * (nt + 1) / 2, J);
    k_psi_hsum_df<<<gt, 256, 0, st>>>(gpart, nsplit, sstride, jstride, lda, fpart, nfchunk, M, hs,
                                      fs);
    TDS_CHECK_LAUNCH();
    k_psi_sandwich_df<<<grid_for((long)JMM), 256, 0, st>>>(c->sr_idx, c->sr_val2, hs, fs, J, M,
                                                           c->maxdeg, tj, tf);
    TDS_CHECK_LAUNCH();
    k_psi_jsum_df<<<std::max(1, ceil_div((long)M * M, 64)), dim3(64, 4), 0, st>>>(
        tj, tf, J, M, 1.0 / (c->sum_rho * c->S), f_out, d2v_out);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

}  // namespace tdscha
