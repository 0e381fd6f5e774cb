// Ensemble preprocessing and the gamma-only translation projection.
//
// * Mode projection (Modules/DynamicalLanczos.py:392-452): with u the
//   displacements and f the forces minus the SSCHA forces, both N x n_cart,
//     X = (u * u_scale * sqrt(m)) . pols,   Y = ((f * f_scale - f_mean) / sqrt(m)) . pols
// * Bloch projection (Modules/QSpaceLanczos.py:221-296): per q-point,
//     X_q = (u_q * u_scale * sqrt(m)) . conj(pols_q),
//     Y_q = ((f_q - f_mean_q) * f_scale / sqrt(m)) . conj(pols_q)
//   with f_mean_q non-zero at Gamma only.
// * gamma_only projection of the averages (DynamicalLanczos.py:3173-3191):
//     f   <- P_t f,  P_t = mean_R pols^T P_R pols
//     d2v <- pols^T [ mean_R Perm_R(pols d2v pols^T) ] pols
//   Perm_R(D)[r][s] = D[perm_R[r]][perm_R[s]] (Cartesian index permutations).
// All float64 (complex double2 for the Bloch projection) on the CUDA cores:
// one-off or O(M^3) per application, no tensor-core variant.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace tdscha {

struct RealOps {
    using T = double;
    __device__ static T zero() { return 0.0; }
    __device__ static T fma_(T a, T b, T c) { return fma(a, b, c); }
};
struct CplxConjBOps {   // acc + a conj(b)
    using T = double2;
    __device__ static T zero() { return make_double2(0, 0); }
    __device__ static T fma_(T a, T b, T c) {
        c.x = fma(a.x, b.x, c.x);
        c.x = fma(a.y, b.y, c.x);
        c.y = fma(a.y, b.x, c.y);
        c.y = fma(-a.x, b.y, c.y);
        return c;
    }
};

// C (rows x cols) = A . B, A(i, k) = A[i*sai + k*sak], B(k, j) = B[k*sbk + j*sbj],
// C row-major with leading dimension ldc.  64 x 64 tiles, 16-deep k slices,
// 256 threads, 4 x 4 outputs per thread; batched over blockIdx.z with the
// given per-batch strides.
template <class Ops>
__global__ void __launch_bounds__(256) k_gemm64(const typename Ops::T *__restrict__ A,
                                                const typename Ops::T *__restrict__ B,
                                                typename Ops::T *__restrict__ C, int rows,
                                                int cols, int K, long sai, long sak, long sbk,
                                                long sbj, long ldc, long bsA, long bsB,
                                                long bsC) {
    using T = typename Ops::T;
    __shared__ T As[16][64 + 1];
    __shared__ T Bs[16][64 + 1];
    A += blockIdx.z * bsA;
    B += blockIdx.z * bsB;
    C += blockIdx.z * bsC;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = Ops::zero();
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            int kk = t % 16, ii = t / 16;
            int i = i0 + ii, k = k0 + kk;
            As[kk][ii] = (i < rows && k < K) ? A[i * sai + k * sak] : Ops::zero();
            int jj = t % 64, kb = t / 64;
            int j = j0 + jj, k2 = k0 + kb;
            Bs[kb][jj] = (j < cols && k2 < K) ? B[k2 * sbk + j * sbj] : Ops::zero();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] = Ops::fma_(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
            if (i < rows && j < cols) C[i * ldc + j] = acc[p][q];
        }
}

template <class Ops>
static int gemm(const typename Ops::T *A, const typename Ops::T *B, typename Ops::T *C, int rows,
                int cols, int K, long sai, long sak, long sbk, long sbj, long ldc,
                cudaStream_t st, int batch = 1, long bsA = 0, long bsB = 0, long bsC = 0) {
    dim3 grid(ceil_div(cols, 64), ceil_div(rows, 64), batch);
    k_gemm64<Ops><<<grid, 256, 0, st>>>(A, B, C, rows, cols, K, sai, sak, sbk, sbj, ldc, bsA, bsB,
                                        bsC);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

// a'[i][k] = (a[i][k] * s - sub[k]) * mul[k] on row-major n x K data (T = double or double2)
__global__ void k_prologue(const double *__restrict__ a, long n, int K, int width, double s,
                           const double *__restrict__ sub, const double *__restrict__ mul,
                           double *__restrict__ out) {
    // width = 1 (real) or 2 (interleaved complex); sub has width entries per k
    long total = n * K * width;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        int k = (int)((e / width) % K), c = (int)(e % width);
        double v = a[e] * s;
        if (sub) v -= sub[k * width + c];
        out[e] = v * mul[k];
    }
}

// Perm-average: out[r][s] = mean_R D[perm_R[r]][perm_R[s]]
__global__ void k_perm_average(const double *__restrict__ D, const int *__restrict__ perms,
                               int n_trans, int n, double *__restrict__ out) {
    long total = (long)n * n;
    const double inv = 1.0 / n_trans;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        int r = (int)(e / n), s = (int)(e % n);
        double acc = 0;
        for (int t = 0; t < n_trans; ++t) {
            const int *p = perms + (long)t * n;
            acc += D[(long)p[r] * n + p[s]];
        }
        out[e] = acc * inv;
    }
}

// Q[r][mu] = mean_R pols[perm_R[r]][mu]
__global__ void k_perm_rows(const double *__restrict__ pols, const int *__restrict__ perms,
                            int n_trans, int n, int M, double *__restrict__ Q) {
    long total = (long)n * M;
    const double inv = 1.0 / n_trans;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        int r = (int)(e / M), mu = (int)(e % M);
        double acc = 0;
        for (int t = 0; t < n_trans; ++t) acc += pols[(long)perms[(long)t * n + r] * M + mu];
        Q[e] = acc * inv;
    }
}

// y = P x (M x M, row-major)
__global__ void k_matvec(const double *__restrict__ P, const double *__restrict__ x, int M,
                         double *__restrict__ y) {
    int i = blockIdx.x;
    __shared__ double sh[32];
    double acc = 0;
    for (int k = threadIdx.x; k < M; k += blockDim.x) acc = fma(P[(long)i * M + k], x[k], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
        y[i] = s;
    }
}

// gamma_only projection of ctx->f and ctx->d2v in place (device, stream ordered)
int apply_translation_projection(tdscha_ctx *c, cudaStream_t st) {
    const int M = c->M, n = c->tr_ncart;
    // f <- P_t f
    k_matvec<<<M, 128, 0, st>>>(c->tr_proj, c->f, M, c->tr_f);
    TDS_CHECK_LAUNCH();
    TDS_CUDA(cudaMemcpyAsync(c->f, c->tr_f, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
    // T1 = pols . d2v (n x M); D = T1 . pols^T (n x n)
    TDS_TRY(gemm<RealOps>(c->tr_pols, c->d2v, c->tr_w1, n, M, M, M, 1, M, 1, M, st));
    TDS_TRY(gemm<RealOps>(c->tr_w1, c->tr_pols, c->tr_w2, n, n, M, M, 1, 1, M, n, st));
    int nb = std::max(1, std::min(ceil_div((long)n * n, 256), 152 * 8));
    k_perm_average<<<nb, 256, 0, st>>>(c->tr_w2, c->tr_perms, c->tr_ntrans, n, c->tr_w3);
    TDS_CHECK_LAUNCH();
    // T2 = pols^T . Davg (M x n); d2v = T2 . pols (M x M)
    TDS_TRY(gemm<RealOps>(c->tr_pols, c->tr_w3, c->tr_w1, M, n, n, 1, M, n, 1, n, st));
    TDS_TRY(gemm<RealOps>(c->tr_w1, c->tr_pols, c->d2v, M, M, n, n, 1, M, 1, M, st));
    return TDSCHA_OK;
}

void free_translations(tdscha_ctx *c) {
    double *bufs[] = {c->tr_pols, c->tr_proj, c->tr_w1, c->tr_w2, c->tr_w3, c->tr_f};
    for (double *b : bufs)
        if (b) cudaFree(b);
    if (c->tr_perms) cudaFree(c->tr_perms);
    c->tr_pols = c->tr_proj = c->tr_w1 = c->tr_w2 = c->tr_w3 = c->tr_f = nullptr;
    c->tr_perms = nullptr;
    c->tr_ntrans = 0;
    c->tr_ncart = 0;
}

}  // namespace tdscha

using namespace tdscha;

extern "C" int tdscha_project_modes(int N, int n_cart, int M, const double *u, const double *f,
                                    const double *f_mean, const double *masses,
                                    const double *pols, double u_scale, double f_scale,
                                    double *X_out, double *Y_out) {
    set_error("");
    if (N <= 0 || n_cart <= 0 || M <= 0 || !u || !f || !masses || !pols || !X_out || !Y_out) {
        set_error("project_modes: bad arguments");
        return TDSCHA_ERR_ARG;
    }
    std::vector<double> sq(n_cart), isq(n_cart), sub;
    for (int k = 0; k < n_cart; ++k) {
        if (!(masses[k] > 0)) { set_error("project_modes: masses must be positive"); return TDSCHA_ERR_ARG; }
        sq[k] = std::sqrt(masses[k]);
        isq[k] = 1.0 / sq[k];
    }
    if (f_mean) {
        sub.resize(n_cart);
        for (int k = 0; k < n_cart; ++k) sub[k] = f_mean[k] * f_scale;
    }
    size_t nu = (size_t)N * n_cart, nx = (size_t)N * M;
    double *d_in = nullptr, *d_tmp = nullptr, *d_pols = nullptr, *d_out = nullptr, *d_vec = nullptr;
    auto done = [&](int rc) {
        double *b[] = {d_in, d_tmp, d_pols, d_out, d_vec};
        for (double *p : b) if (p) cudaFree(p);
        return rc;
    };
#define PCU(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { set_error("%s: %s", #x, cudaGetErrorString(_e)); return done(TDSCHA_ERR_CUDA); } } while (0)
    PCU(cudaMalloc(&d_in, sizeof(double) * nu));
    PCU(cudaMalloc(&d_tmp, sizeof(double) * nu));
    PCU(cudaMalloc(&d_pols, sizeof(double) * (size_t)n_cart * M));
    PCU(cudaMalloc(&d_out, sizeof(double) * nx));
    PCU(cudaMalloc(&d_vec, sizeof(double) * 3 * n_cart));
    PCU(cudaMemcpy(d_pols, pols, sizeof(double) * (size_t)n_cart * M, cudaMemcpyHostToDevice));
    PCU(cudaMemcpy(d_vec, sq.data(), sizeof(double) * n_cart, cudaMemcpyHostToDevice));
    PCU(cudaMemcpy(d_vec + n_cart, isq.data(), sizeof(double) * n_cart, cudaMemcpyHostToDevice));
    if (f_mean) PCU(cudaMemcpy(d_vec + 2 * n_cart, sub.data(), sizeof(double) * n_cart, cudaMemcpyHostToDevice));
    int nb = std::max(1, std::min(ceil_div((long)nu, 256), 152 * 8));
    for (int pass = 0; pass < 2; ++pass) {
        PCU(cudaMemcpy(d_in, pass == 0 ? u : f, sizeof(double) * nu, cudaMemcpyHostToDevice));
        if (pass == 0)
            k_prologue<<<nb, 256>>>(d_in, N, n_cart, 1, u_scale, nullptr, d_vec, d_tmp);
        else
            k_prologue<<<nb, 256>>>(d_in, N, n_cart, 1, f_scale, f_mean ? d_vec + 2 * n_cart : nullptr,
                                    d_vec + n_cart, d_tmp);
        PCU(cudaGetLastError());
        int rc = gemm<RealOps>(d_tmp, d_pols, d_out, N, M, n_cart, n_cart, 1, M, 1, M, 0);
        if (rc != TDSCHA_OK) return done(rc);
        PCU(cudaMemcpy(pass == 0 ? X_out : Y_out, d_out, sizeof(double) * nx, cudaMemcpyDeviceToHost));
    }
#undef PCU
    return done(TDSCHA_OK);
}

extern "C" int tdscha_project_bloch(int n_q, int N, int n_cart, int nb, const double *u_q,
                                    const double *f_q, const double *f_mean_gamma,
                                    const double *masses, const double *pols_q, double u_scale,
                                    double f_scale, double *X_q, double *Y_q) {
    set_error("");
    if (n_q <= 0 || N <= 0 || n_cart <= 0 || nb <= 0 || !u_q || !f_q || !masses || !pols_q || !X_q || !Y_q) {
        set_error("project_bloch: bad arguments");
        return TDSCHA_ERR_ARG;
    }
    // layouts: u_q, f_q (n_q, N, n_cart) complex; pols_q (n_q, n_cart, nb) complex;
    // X_q, Y_q (n_q, N, nb) complex; f_mean_gamma (n_cart) complex or NULL
    std::vector<double> sq(n_cart), isq(n_cart);
    for (int k = 0; k < n_cart; ++k) {
        if (!(masses[k] > 0)) { set_error("project_bloch: masses must be positive"); return TDSCHA_ERR_ARG; }
        sq[k] = std::sqrt(masses[k]);
        isq[k] = 1.0 / sq[k];
    }
    size_t nu = (size_t)n_q * N * n_cart, nx = (size_t)n_q * N * nb, npol = (size_t)n_q * n_cart * nb;
    double2 *d_in = nullptr, *d_tmp = nullptr, *d_pols = nullptr, *d_out = nullptr;
    double *d_vec = nullptr;
    auto done = [&](int rc) {
        void *b[] = {d_in, d_tmp, d_pols, d_out, d_vec};
        for (void *p : b) if (p) cudaFree(p);
        return rc;
    };
#define PCU(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { set_error("%s: %s", #x, cudaGetErrorString(_e)); return done(TDSCHA_ERR_CUDA); } } while (0)
    PCU(cudaMalloc(&d_in, sizeof(double2) * nu));
    PCU(cudaMalloc(&d_tmp, sizeof(double2) * nu));
    PCU(cudaMalloc(&d_pols, sizeof(double2) * npol));
    PCU(cudaMalloc(&d_out, sizeof(double2) * nx));
    PCU(cudaMalloc(&d_vec, sizeof(double) * 4 * n_cart));
    PCU(cudaMemcpy(d_pols, pols_q, sizeof(double2) * npol, cudaMemcpyHostToDevice));
    PCU(cudaMemcpy(d_vec, sq.data(), sizeof(double) * n_cart, cudaMemcpyHostToDevice));
    PCU(cudaMemcpy(d_vec + n_cart, isq.data(), sizeof(double) * n_cart, cudaMemcpyHostToDevice));
    if (f_mean_gamma) PCU(cudaMemcpy(d_vec + 2 * n_cart, f_mean_gamma, sizeof(double) * 2 * n_cart, cudaMemcpyHostToDevice));
    int nbk = std::max(1, std::min(ceil_div((long)nu * 2, 256), 152 * 8));
    for (int pass = 0; pass < 2; ++pass) {
        PCU(cudaMemcpy(d_in, pass == 0 ? u_q : f_q, sizeof(double2) * nu, cudaMemcpyHostToDevice));
        if (pass == 0) {
            k_prologue<<<nbk, 256>>>((const double *)d_in, (long)n_q * N, n_cart, 2, u_scale, nullptr,
                                     d_vec, (double *)d_tmp);
        } else {
            // (f - f_mean) * f_scale / sqrt(m): the mean is subtracted at Gamma (q index 0) only
            k_prologue<<<nbk, 256>>>((const double *)d_in, (long)n_q * N, n_cart, 2, 1.0, nullptr,
                                     d_vec + n_cart, (double *)d_tmp);
            if (f_mean_gamma) {
                // Gamma rows: redo with the mean subtracted, scale folded as (f - g) / sqrt(m)
                k_prologue<<<nbk, 256>>>((const double *)d_in, (long)N, n_cart, 2, 1.0, d_vec + 2 * n_cart,
                                         d_vec + n_cart, (double *)d_tmp);
            }
        }
        PCU(cudaGetLastError());
        int rc = gemm<CplxConjBOps>(d_tmp, d_pols, d_out, N, nb, n_cart, n_cart, 1, nb, 1, nb, 0, n_q,
                                    (long)N * n_cart, (long)n_cart * nb, (long)N * nb);
        if (rc != TDSCHA_OK) return done(rc);
        PCU(cudaMemcpy(pass == 0 ? X_q : Y_q, d_out, sizeof(double2) * nx, cudaMemcpyDeviceToHost));
        if (pass == 1 && f_scale != 1.0) {
            for (size_t e = 0; e < 2 * nx; ++e) Y_q[e] *= f_scale;
        }
    }
#undef PCU
    return done(TDSCHA_OK);
}

extern "C" int tdscha_ctx_set_translations(tdscha_ctx *ctx, int n_cart, const double *pols,
                                           int n_trans, const int *perms) {
    set_error("");
    if (!ctx) { set_error("ctx_set_translations: null context"); return TDSCHA_ERR_ARG; }
    cudaDeviceSynchronize();
    free_translations(ctx);
    if (n_trans == 0) return TDSCHA_OK;
    const int M = ctx->M;
    if (n_cart < M || n_trans < 0 || !pols || !perms) { set_error("ctx_set_translations: bad arguments"); return TDSCHA_ERR_ARG; }
    for (long e = 0; e < (long)n_trans * n_cart; ++e)
        if (perms[e] < 0 || perms[e] >= n_cart) { set_error("ctx_set_translations: permutation index out of range"); return TDSCHA_ERR_ARG; }
    const int n = n_cart;
    ctx->tr_ncart = n;
    ctx->tr_ntrans = n_trans;
    TDS_CUDA(cudaMalloc(&ctx->tr_pols, sizeof(double) * (size_t)n * M));
    TDS_CUDA(cudaMalloc(&ctx->tr_perms, sizeof(int) * (size_t)n_trans * n));
    TDS_CUDA(cudaMalloc(&ctx->tr_proj, sizeof(double) * (size_t)M * M));
    TDS_CUDA(cudaMalloc(&ctx->tr_w1, sizeof(double) * (size_t)n * std::max(n, M)));
    TDS_CUDA(cudaMalloc(&ctx->tr_w2, sizeof(double) * (size_t)n * n));
    TDS_CUDA(cudaMalloc(&ctx->tr_w3, sizeof(double) * (size_t)n * n));
    TDS_CUDA(cudaMalloc(&ctx->tr_f, sizeof(double) * M));
    TDS_CUDA(cudaMemcpy(ctx->tr_pols, pols, sizeof(double) * (size_t)n * M, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemcpy(ctx->tr_perms, perms, sizeof(int) * (size_t)n_trans * n, cudaMemcpyHostToDevice));
    // P_t = pols^T (mean_R P_R pols) (the reference's trans_projector, :764-785)
    int nb = std::max(1, std::min(ceil_div((long)n * M, 256), 152 * 8));
    k_perm_rows<<<nb, 256>>>(ctx->tr_pols, ctx->tr_perms, n_trans, n, M, ctx->tr_w2);
    TDS_CUDA(cudaGetLastError());
    TDS_TRY(gemm<RealOps>(ctx->tr_pols, ctx->tr_w2, ctx->tr_proj, M, M, n, 1, M, M, 1, M, 0));
    TDS_CUDA(cudaDeviceSynchronize());
    return TDSCHA_OK;
}
