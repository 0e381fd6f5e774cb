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

// Device address of g_noalloc_scratch.  The array lives in the module the
// runtime loads into each CUDA context, so its address belongs to a context,
// not to a device: a caller running its own driver-API context, or a
// cudaDeviceReset, gives the same device another module at another address.
// So every call made outside a stream capture looks the address up again
// (a host-side table lookup) and records it under the current context; a
// call made while its stream is being captured uses the address recorded for
// the current context and fails if there is none.
typedef int (*ctx_get_current_fn)(void **);
static std::mutex g_noalloc_mu;
struct NoallocSlot {
    void *ctx;
    double *ptr;
};
static NoallocSlot g_noalloc_slots[32];
static int g_noalloc_next = 0;

static void *current_context() {
    static ctx_get_current_fn fn = nullptr;
    static bool looked = false;
    if (!looked) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<ctx_get_current_fn>(p);
        looked = true;
    }
    void *ctx = nullptr;
    if (fn && fn(&ctx) != 0) ctx = nullptr;
    return ctx;
}

static int noalloc_scratch(cudaStream_t st, double **out) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        (void)cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;      // unknown: do not touch the module table
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    void *ctx = current_context();
    NoallocSlot *slot = nullptr;
    for (auto &s : g_noalloc_slots)
        if (s.ptr && s.ctx == ctx) slot = &s;
    if (cap != cudaStreamCaptureStatusNone) {
        if (!slot) {
            set_error("perturb_averages_noalloc: first call in this CUDA context made during a "
                      "stream capture; make one call outside the capture first");
            return TDSCHA_ERR_STATE;
        }
        *out = slot->ptr;
        return TDSCHA_OK;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        set_error("perturb_averages_noalloc: cudaGetSymbolAddress failed: %s",
                  cudaGetErrorString(e));
        return TDSCHA_ERR_CUDA;
    }
    if (!slot) {
        slot = &g_noalloc_slots[g_noalloc_next];
        g_noalloc_next = (g_noalloc_next + 1) % 32;
    }
    slot->ctx = ctx;
    slot->ptr = static_cast<double *>(p);
    *out = slot->ptr;
    return TDSCHA_OK;
}

// f_Y, f_psi per mode, the symmetrised Y1, sum(rho) (block 0), and the input
// check: block k writes bad[k] = 1 if any entry it scanned is invalid
// (non-finite X, Y, R1, Y1 or w; w <= 0; rho negative or non-finite), else 0,
// so no word has to be cleared between calls.
__global__ void k_na_setup(const double *__restrict__ w, const double *__restrict__ rho,
                           const double *__restrict__ Y1, const double *__restrict__ R1,
                           const double *__restrict__ X, const double *__restrict__ Y, double T,
                           int M, long N, double *__restrict__ fY, double *__restrict__ fpsi,
                           double *__restrict__ Y1s, double *__restrict__ sum_rho,
                           double *__restrict__ bad) {
    const long n = (long)M * M;
    const long stride = (long)gridDim.x * blockDim.x;
    const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
    int invalid = 0;
    for (long e = t0; e < n; e += stride) {
        int a = (int)(e / M), b = (int)(e % M);
        double yab = Y1[(long)a * M + b];
        Y1s[e] = 0.5 * (yab + Y1[(long)b * M + a]);
        invalid |= !isfinite(yab);
        if (e < M) {
            double we = w[e];
            invalid |= !(isfinite(we) && we > 0) || !isfinite(R1[e]);
            double nw = 0;
            if (T > 0) nw = 1 / (exp(we * kRyToK / T) - 1);
            fY[e] = 2 * we / (1 + 2 * nw);
            fpsi[e] = (1 + 2 * nw) / (2 * we);
        }
    }
    const long nx = (long)M * N;
    for (long e = t0; e < nx; e += stride) invalid |= !isfinite(X[e]) || !isfinite(Y[e]);
    for (long e = t0; e < N; e += stride) invalid |= !(isfinite(rho[e]) && rho[e] >= 0);
    invalid = __syncthreads_or(invalid);
    if (threadIdx.x == 0) bad[blockIdx.x] = invalid ? 1.0 : 0.0;
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

// d2v = -(G + G^T) / sum(rho), f = sum of the force partials / sum(rho); every
// output entry NaN when the input check failed or sum(rho) is not positive.
__global__ void k_na_finalize(const double *__restrict__ gpart, int nsplit,
                              const double *__restrict__ fpart, int nfchunk, int M,
                              const double *__restrict__ sum_rho, const double *__restrict__ bad,
                              int nbad, double *__restrict__ f, double *__restrict__ d2v) {
    int any = 0;
    for (int k = threadIdx.x; k < nbad; k += blockDim.x) any |= bad[k] != 0.0;
    const double norm = *sum_rho;
    any = __syncthreads_or(any | !(norm > 0));
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    long n = (long)M * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e / M), b = (int)(e % M);
        double gab = 0, gba = 0;
        for (int s = 0; s < nsplit; ++s) {
            gab += gpart[(long)s * n + (long)a * M + b];
            gba += gpart[(long)s * n + (long)b * M + a];
        }
        d2v[e] = any ? nan : -(gab + gba) / norm;
        if (e < M) {
            double acc = 0;
            for (int ch = 0; ch < nfchunk; ++ch) acc += fpart[(long)ch * M + e];
            f[e] = any ? nan : acc / norm;
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
    // scratch layout (float64 words).  The split-K count of stage B is the
    // smallest that gives two blocks per SM; the context path searches further
    // (up to 64 splits, for whole rounds of 152 SMs), which here would need up
    // to 64 partial M x M tiles.  So results agree with tdscha_perturb_averages
    // to rounding, not bit for bit.
    constexpr int kT = 64;
    const long R = N;
    const int nct = ceil_div(M, kT);
    const int ntile = nct;
    int nsplit = std::max(1, ceil_div(2 * 152, ntile * ntile));
    nsplit = (int)std::min<long>(nsplit, std::max<long>(1, R / 64));
    const int nfchunk = (int)std::min<long>(std::max<long>(1, R / 256), 512);
    const size_t MM = (size_t)M * M;
    // blocks of the set-up pass: enough for the M x M and N x M scans
    const int nset = (int)std::max<long>(1, std::min<long>(2048, std::max(ceil_div((long)MM, 256),
                                                                          ceil_div((long)M * R, 2048))));
    const size_t need = 2 * (size_t)M + MM + 2 * (size_t)nct * R + 4 * (size_t)R +
                        (size_t)nsplit * MM + (size_t)nfchunk * M + 1 + (size_t)nset;
    if (need > kNoAllocWords) {
        set_error("perturb_averages_noalloc: M=%d, N=%d needs %zu bytes of scratch; the static "
                  "area holds %zu bytes (use the context API for larger ensembles)",
                  M, N, need * sizeof(double), kNoAllocWords * sizeof(double));
        return TDSCHA_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    double *base = nullptr;
    TDS_TRY(noalloc_scratch(st, &base));
    double *fY = base, *fpsi = fY + M, *Y1s = fpsi + M, *qp = Y1s + MM;
    double *alpha = qp + 2 * (size_t)nct * R, *beta = alpha + R, *c1 = beta + R, *c2 = c1 + R;
    double *gpart = c2 + R, *fpart = gpart + (size_t)nsplit * MM;
    double *sum_rho = fpart + (size_t)nfchunk * M, *bad = sum_rho + 1;
    // every scratch word below is written before it is read; nothing needs clearing
    int nb = std::max(1, std::min(ceil_div((long)MM, 256), 2048));
    k_na_setup<<<nset, 256, 0, st>>>(w, rho, Y1, R1, X, Y, T, M, R, fY, fpsi, Y1s, sum_rho, bad);
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
    k_na_finalize<<<nb, 256, 0, st>>>(gpart, nsplit, fpart, nfchunk, M, sum_rho, bad, nset, f_out,
                                      d2v_out);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}
