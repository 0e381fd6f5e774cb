// Float64 perturbation averages that allocate no device memory.
//
// Who needs this: host programs that hand this library a fixed device-memory
// budget and do not let it take more -- for example a simulation code that
// reserves all of the GPU's memory for its own pool at start-up and manages
// every allocation itself -- and latency-critical callers that cannot accept
// the device-wide synchronisation that cudaMalloc / cudaFree may perform.
// Such callers pass their own device buffers for every input and output; the
// intermediate arrays of the computation (row partials, split-K tiles, the
// symmetrised Y1, ...) live in one statically sized __device__ array that
// exists in every process that loads the library, on every GPU it uses,
// until the process exits.
//
// This variant runs the float64 pipeline of perturb_fp64.cu (same kernels)
// for ensembles without symmetry images (one identity image per
// configuration).
#include <cmath>
#include <mutex>

#include "common.cuh"

namespace tdscha {

// kernels of the float64 path (perturb_fp64.cu)
__global__ void k_stageA64(const double *__restrict__ D, const double *__restrict__ F,
                           const double *__restrict__ Y1, const double *__restrict__ fpsi, int M,
                           long R, double *__restrict__ qp_part);
__global__ void k_rows64(const double *__restrict__ D, const double *__restrict__ F,
                         const double *__restrict__ fY, const double *__restrict__ R1,
                         const double *__restrict__ rho, const double *__restrict__ qp_part,
                         int nct, int M, int S, long R, int apply_d4, double *__restrict__ alpha,
                         double *__restrict__ beta, double *__restrict__ c1,
                         double *__restrict__ c2);
__global__ void k_favg64(const double *__restrict__ D, const double *__restrict__ F,
                         const double *__restrict__ fY, const double *__restrict__ c1,
                         const double *__restrict__ c2, int M, long R, long chunk,
                         double *__restrict__ fpart);
__global__ void k_stageB64(const double *__restrict__ D, const double *__restrict__ F,
                           const double *__restrict__ fY, const double *__restrict__ alpha,
                           const double *__restrict__ beta, int M, long R, long chunk, int ntile,
                           double *__restrict__ gpart);

// The static scratch area: 32 MiB of float64 words.
constexpr size_t kNoAllocWords = (size_t)4 << 20;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocWords];

// Device address of g_noalloc_scratch, looked up once per device.
static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(double **out) {
    int dev = 0;
    TDS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("perturb_averages_noalloc: device ordinal %d out of range", dev);
        return TDSCHA_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("perturb_averages_noalloc: cudaGetSymbolAddress failed: %s",
                      cudaGetErrorString(e));
            return TDSCHA_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return TDSCHA_OK;
}

// f_Y, f_psi per mode, the symmetrised Y1, and sum(rho) (block 0).
__global__ void k_na_setup(const double *__restrict__ w, const double *__restrict__ rho,
                           const double *__restrict__ Y1, double T, int M, long N,
                           double *__restrict__ fY, double *__restrict__ fpsi,
                           double *__restrict__ Y1s, double *__restrict__ sum_rho) {
    long n = (long)M * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e / M), b = (int)(e % M);
        Y1s[e] = 0.5 * (Y1[(long)a * M + b] + Y1[(long)b * M + a]);
        if (e < M) {
            double nw = 0;
            if (T > 0) nw = 1 / (exp(w[e] * kRyToK / T) - 1);
            fY[e] = 2 * w[e] / (1 + 2 * nw);
            fpsi[e] = (1 + 2 * nw) / (2 * w[e]);
        }
    }
    if (blockIdx.x == 0) {
        __shared__ double sh[32];
        double s = 0;
        for (long i = threadIdx.x; i < N; i += blockDim.x) s += rho[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
            *sum_rho = t;
        }
    }
}

__global__ void k_na_finalize(const double *__restrict__ gpart, int nsplit, const double *__restrict__ fpart,
                              int nfchunk, int M, const double *__restrict__ sum_rho,
                              double *__restrict__ f, double *__restrict__ d2v) {
    long n = (long)M * M;
    double norm = *sum_rho;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e / M), b = (int)(e % M);
        double gab = 0, gba = 0;
        for (int s = 0; s < nsplit; ++s) {
            gab += gpart[(long)s * n + (long)a * M + b];
            gba += gpart[(long)s * n + (long)b * M + a];
        }
        d2v[e] = -(gab + gba) / norm;
        if (e < M) {
            double acc = 0;
            for (int ch = 0; ch < nfchunk; ++ch) acc += fpart[(long)ch * M + e];
            f[e] = acc / norm;
        }
    }
}

}  // namespace tdscha

using namespace tdscha;

extern "C" int tdscha_perturb_averages_noalloc(int M, int N, const double *X, const double *Y,
                                               const double *w, const double *rho,
                                               const double *R1, const double *Y1, double T,
                                               int apply_D4, double *f_out, double *d2v_out,
                                               void *stream) {
    set_error("");
    if (M <= 0 || N <= 0) {
        set_error("perturb_averages_noalloc: bad sizes M=%d N=%d", M, N);
        return TDSCHA_ERR_ARG;
    }
    if (!X || !Y || !w || !rho || !R1 || !Y1 || !f_out || !d2v_out) {
        set_error("perturb_averages_noalloc: null pointer");
        return TDSCHA_ERR_ARG;
    }
    if (apply_D4 != 0 && apply_D4 != 1) {
        set_error("perturb_averages_noalloc: apply_D4 must be 0 or 1, got %d", apply_D4);
        return TDSCHA_ERR_ARG;
    }
    if (!(T >= 0) || !std::isfinite(T)) {
        set_error("perturb_averages_noalloc: bad temperature %g", T);
        return TDSCHA_ERR_ARG;
    }
    // scratch layout (float64 words), the same partitioning as the context path
    constexpr int kT = 64;
    const long R = N;
    const int nct = ceil_div(M, kT);
    const int ntile = nct;
    int nsplit = std::max(1, ceil_div(2 * 152, ntile * ntile));
    nsplit = (int)std::min<long>(nsplit, std::max<long>(1, R / 64));
    const int nfchunk = (int)std::min<long>(std::max<long>(1, R / 256), 512);
    const size_t MM = (size_t)M * M;
    const size_t need = 2 * (size_t)M + MM + 2 * (size_t)nct * R + 4 * (size_t)R +
                        (size_t)nsplit * MM + (size_t)nfchunk * M + 1;
    if (need > kNoAllocWords) {
        set_error("perturb_averages_noalloc: M=%d, N=%d needs %zu bytes of scratch; the static "
                  "area holds %zu bytes (use the context API for larger ensembles)",
                  M, N, need * sizeof(double), kNoAllocWords * sizeof(double));
        return TDSCHA_ERR_ARG;
    }
    double *base = nullptr;
    TDS_TRY(noalloc_scratch(&base));
    double *fY = base, *fpsi = fY + M, *Y1s = fpsi + M, *qp = Y1s + MM;
    double *alpha = qp + 2 * (size_t)nct * R, *beta = alpha + R, *c1 = beta + R, *c2 = c1 + R;
    double *gpart = c2 + R, *fpart = gpart + (size_t)nsplit * MM;
    double *sum_rho = fpart + (size_t)nfchunk * M;
    // every scratch word below is written before it is read; nothing needs clearing
    cudaStream_t st = (cudaStream_t)stream;
    int nb = std::max(1, std::min(ceil_div((long)MM, 256), 2048));
    k_na_setup<<<nb, 256, 0, st>>>(w, rho, Y1, T, M, R, fY, fpsi, Y1s, sum_rho);
    TDS_CHECK_LAUNCH();
    k_stageA64<<<dim3(ceil_div(R, kT), nct), 256, 0, st>>>(X, Y, Y1s, fpsi, M, R, qp);
    TDS_CHECK_LAUNCH();
    k_rows64<<<ceil_div(R, 8), 256, 0, st>>>(X, Y, fY, R1, rho, qp, nct, M, 1, R, apply_D4,
                                              alpha, beta, c1, c2);
    TDS_CHECK_LAUNCH();
    long fchunk = (R + nfchunk - 1) / nfchunk;
    k_favg64<<<dim3(ceil_div(M, 128), nfchunk), 128, 0, st>>>(X, Y, fY, c1, c2, M, R, fchunk,
                                                                fpart);
    TDS_CHECK_LAUNCH();
    long chunk = (R + nsplit - 1) / nsplit;
    k_stageB64<<<dim3(ntile * ntile, nsplit), 256, 0, st>>>(X, Y, fY, alpha, beta, M, R, chunk,
                                                            ntile, gpart);
    TDS_CHECK_LAUNCH();
    k_na_finalize<<<nb, 256, 0, st>>>(gpart, nsplit, fpart, nfchunk, M, sum_rho, f_out, d2v_out);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}
