// Static (free-energy Hessian) operator on the resident ensemble.
//
// The static response solves L_static x = b with
//   L_static psi = apply_L1_static(psi) + apply_anharmonic_static(psi)
// (Modules/DynamicalLanczos.py:2562-2624 and :3369-3430), psi = [R (M) | W (M(M+1)/2,
// upper-triangle rows)].  The anharmonic part is the same ensemble average as
// the dynamical operator, called with R1 = psi_R and
// Y1_ab = -2 psi_W(ab) Upsilon_a Upsilon_b (Upsilon = 2w/(2n+1)); its output is
// [-f | d2v upper triangle].  The harmonic part is diagonal: psi_R w^(2p) and
// psi_W / Lambda^p with the pair factor Lambda of apply_L1_static.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace tdscha {

int run_perturb(tdscha_ctx *c, int apply_d4, int precision, cudaStream_t st);

// Lambda per upper-triangle pair (row i, column j), as apply_L1_static builds it
// (:2588-2622): i_a = column, i_b = row; both population masks are taken from
// w_a (:2603-2604); on the w_a == w_b diagonal the derivative term is
// -beta exp(w beta) n_equal^2 with n_equal read before the occupations are
// set (:2607-2619), i.e. a zero (NaN where exp overflows).
static int build_static_lambda(tdscha_ctx *c) {
    const int M = c->M;
    const long H = c->H;
    std::vector<double> w(M), lam(H);
    TDS_CUDA(cudaMemcpy(w.data(), c->w, sizeof(double) * M, cudaMemcpyDeviceToHost));
    const double T = c->T;
    long k = 0;
    for (int i = 0; i < M; ++i)
        for (int j = i; j < M; ++j, ++k) {
            double wa = w[j], wb = w[i];
            double na = 0, nb = 0, diff = 0;
            bool unpopulated = 0.01 * wa * kRyToK > T;
            bool equal = fabs(wa - wb) < 1e-8;
            if (T > 0) {
                double beta = kRyToK / T;
                na = 1 / (exp(wa * beta) - 1);
                nb = 1 / (exp(wb * beta) - 1);
                if (unpopulated) { na = 0; nb = 0; }
                diff = equal ? (-beta * exp(wa * beta)) * 0.0 : (na - nb) / (wa - wb);
            }
            double l = (na + nb + 1) / (wa + wb) - diff;
            lam[k] = l / (4 * wa * wb);
        }
    if (!c->lam_static) TDS_CUDA(cudaMalloc(&c->lam_static, sizeof(double) * H));
    TDS_CUDA(cudaMemcpy(c->lam_static, lam.data(), sizeof(double) * H, cudaMemcpyHostToDevice));
    return TDSCHA_OK;
}

__device__ __forceinline__ long tri_index_s(int i, int j, int M) {
    return (long)i * M - (long)i * (i - 1) / 2 + (j - i);
}

// R1 = psi_R; Y1_ab = -2 (psi_W(ab) Upsilon_a) Upsilon_b
__global__ void k_unpack_static(const double *__restrict__ psi, const double *__restrict__ Yw,
                                int M, double *__restrict__ R1, double *__restrict__ Y1) {
    long n = (long)M * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e / M), b = (int)(e % M);
        long k = tri_index_s(min(a, b), max(a, b), M);
        Y1[e] = -2 * ((psi[M + k] * Yw[a]) * Yw[b]);
        if (e < M) R1[e] = psi[e];
    }
}

// x^p for the exponents numpy evaluates exactly (square, identity, square root,
// reciprocal), pow otherwise
__device__ __forceinline__ double pow_np(double x, double p) {
    if (p == 2.0) return x * x;
    if (p == 1.0) return x;
    if (p == 0.0) return 1.0;
    if (p == 0.5) return sqrt(x);
    if (p == -1.0) return 1.0 / x;
    return pow(x, p);
}

__global__ void k_assemble_static(const double *__restrict__ psi, const double *__restrict__ f,
                                  const double *__restrict__ d2v, const double *__restrict__ w,
                                  const double *__restrict__ lam, const int *__restrict__ tri,
                                  int M, long H, int harm, int anh, double power,
                                  double *__restrict__ out) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < M + H; e += (long)gridDim.x * blockDim.x) {
        double o = 0;
        if (e < M) {
            if (harm) o = psi[e] * pow_np(w[e], 2 * power);
            if (anh) o += -f[e];
        } else {
            long k = e - M;
            if (harm) o = psi[e] / pow_np(lam[k], power);
            if (anh) o += d2v[(long)tri[2 * k] * M + tri[2 * k + 1]];
        }
        out[e] = o;
    }
}

// StaticHessian vector <-> M static psi rows (Modules/StaticHessian.py:561-691).
// The vector is [G upper triangle rows (M(M+1)/2) | W, i <= j <= k (M(M+1)(M+2)/6)];
// row i of the batch is [G_i: (M) | W_i upper triangle rows (M(M+1)/2)].
__device__ __forceinline__ long sh_s3(long n) { return n * (n + 1) * (n + 2) / 6; }
__device__ __forceinline__ long sh_w_index(int a, int b, int c, int M) {   // a <= b <= c
    return sh_s3(M) - sh_s3(M - a) + (long)(b - a) * M - (long)(b - 1 + a) * (b - a) / 2 + (c - b);
}

__global__ void k_sh_expand(const double *__restrict__ vec, const int *__restrict__ tri, int M,
                            long H, double *__restrict__ X) {
    const long Ps = M + H, n_g = H;
    const long total = (long)M * Ps;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int i = (int)(t / Ps);
        long e = t % Ps;
        double v;
        if (e < M) {
            int j = (int)e;
            v = vec[tri_index_s(min(i, j), max(i, j), M)];
        } else {
            long k = e - M;
            int j = tri[2 * k], l = tri[2 * k + 1];        // j <= l
            int a = i, b = j, c = l;                        // sort (i, j, l)
            if (a > b) { int s = a; a = b; b = s; }
            if (b > c) { int s = b; b = c; c = s; }
            if (a > b) { int s = a; a = b; b = s; }
            v = vec[n_g + sh_w_index(a, b, c, M)];
        }
        X[t] = v;
    }
}

__global__ void k_sh_collect(const double *__restrict__ Y, const int *__restrict__ tri, int M,
                             long H, double *__restrict__ vec) {
    const long Ps = M + H, n_g = H;
    const long total = (long)M * Ps;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        int i = (int)(t / Ps);
        long e = t % Ps;
        if (e < M) {
            if ((int)e >= i) vec[tri_index_s(i, (int)e, M)] = Y[t];
        } else {
            long k = e - M;
            int j = tri[2 * k], l = tri[2 * k + 1];
            if (i <= j) vec[n_g + sh_w_index(i, j, l, M)] = Y[t];
        }
    }
}

}  // namespace tdscha

using namespace tdscha;

extern "C" int tdscha_static_hessian_expand(tdscha_ctx *ctx, const double *vec, double *X,
                                            void *stream) {
    set_error("");
    if (!ctx || !vec || !X) { set_error("static_hessian_expand: null pointer"); return TDSCHA_ERR_ARG; }
    long total = (long)ctx->M * (ctx->M + ctx->H);
    int nb = std::max(1, std::min(ceil_div(total, 256), 152 * 16));
    k_sh_expand<<<nb, 256, 0, (cudaStream_t)stream>>>(vec, ctx->tri, ctx->M, ctx->H, X);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

extern "C" int tdscha_static_hessian_collect(tdscha_ctx *ctx, const double *Y, double *vec,
                                             void *stream) {
    set_error("");
    if (!ctx || !vec || !Y) { set_error("static_hessian_collect: null pointer"); return TDSCHA_ERR_ARG; }
    long total = (long)ctx->M * (ctx->M + ctx->H);
    int nb = std::max(1, std::min(ceil_div(total, 256), 152 * 16));
    k_sh_collect<<<nb, 256, 0, (cudaStream_t)stream>>>(Y, ctx->tri, ctx->M, ctx->H, vec);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

extern "C" int tdscha_static_L(tdscha_ctx *ctx, int nvec, const double *psi_in, double *psi_out,
                               int what, double power, int precision, void *stream) {
    set_error("");
    if (!ctx || !psi_in || !psi_out || nvec < 0) { set_error("static_L: bad arguments"); return TDSCHA_ERR_ARG; }
    if (psi_in == psi_out) { set_error("static_L: in-place application is not supported"); return TDSCHA_ERR_ARG; }
    if (what < 1 || what > 3) { set_error("static_L: what must be 1 (harmonic), 2 (anharmonic) or 3 (both)"); return TDSCHA_ERR_ARG; }
    if (precision != TDSCHA_PREC_FP64 && precision != TDSCHA_PREC_MIXED) { set_error("static_L: bad precision"); return TDSCHA_ERR_ARG; }
    if (precision == TDSCHA_PREC_MIXED && !ctx->with_mixed) {
        set_error("static_L: context created without the mixed-precision operands");
        return TDSCHA_ERR_STATE;
    }
    if (!std::isfinite(power)) { set_error("static_L: power must be finite"); return TDSCHA_ERR_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    const int M = ctx->M;
    const long H = ctx->H, Ps = M + H;
    if (!ctx->lam_static) TDS_TRY(build_static_lambda(ctx));
    const int harm = what & 1, anh = (what >> 1) & 1;
    const int nbu = std::max(1, std::min(ceil_div((long)M * M, 256), 4096));
    const int nba = std::max(1, std::min(ceil_div(Ps, 256), 4096));
    for (int v = 0; v < nvec; ++v) {
        const double *in = psi_in + (long)v * Ps;
        double *out = psi_out + (long)v * Ps;
        if (anh) {
            k_unpack_static<<<nbu, 256, 0, st>>>(in, ctx->Yw, M, ctx->R1, ctx->Y1);
            TDS_CHECK_LAUNCH();
            TDS_TRY(run_perturb(ctx, ctx->ignore_v4 ? 0 : 1, precision, st));
        }
        k_assemble_static<<<nba, 256, 0, st>>>(in, ctx->f, ctx->d2v, ctx->w, ctx->lam_static,
                                               ctx->tri, M, H, harm, anh, power, out);
        TDS_CHECK_LAUNCH();
    }
    return TDSCHA_OK;
}
