// Context lifecycle, error reporting and the perturbation-average entry
// points of the C ABI (include/tdscha_gb300.h).
#include <cmath>
#include <cstdarg>
#include <cstring>

#include <list>
#include <map>
#include <mutex>
#include <unordered_map>

#include "common.cuh"

namespace tdscha {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

// f_ups / f_psi of the reference (CModules/LanczosFunctions.c:14-30), in the
// same expression order.
static double h_f_ups(double w, double T) {
    double n_w = 0;
    if (T > 0) n_w = 1 / (exp(w * kRyToK / T) - 1);
    return 2 * w / (1 + 2 * n_w);
}
static double h_f_psi(double w, double T) {
    double n_w = 0;
    if (T > 0) n_w = 1 / (exp(w * kRyToK / T) - 1);
    return (1 + 2 * n_w) / (2 * w);
}

// d = S_j X_i and f = S_j Y_i for every image row r = i*S + j, block by block
// with the reference's row convention mu_id = mu - deg_space[b][0]
// (LanczosFunctions.c:2158-2170).
__global__ void k_expand_images(const double *__restrict__ X, const double *__restrict__ Y,
                                int N, int M, int S, const int *__restrict__ n_deg,
                                const int *__restrict__ deg_off, const long *__restrict__ sym_off,
                                const int *__restrict__ deg_space,
                                const int *__restrict__ blocks_ids,
                                const double *__restrict__ sym, double *__restrict__ D,
                                double *__restrict__ F,
                                unsigned long long *__restrict__ first_bad) {
    long total = (long)N * S * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total;
         e += (long)gridDim.x * blockDim.x) {
        int mu = (int)(e % M);
        long r = e / M;
        int i = (int)(r / S), j = (int)(r % S);
        // every input entry once (first image): the smallest non-finite index
        if (j == 0) {
            long x = (long)i * M + mu;
            if (!isfinite(X[x]) || !isfinite(Y[x])) atomicMin(first_bad, (unsigned long long)x);
        }
        int b = blocks_ids[mu];
        const int *space = deg_space + deg_off[b];
        int bd = n_deg[b];
        int mu_id = mu - space[0];
        const double *s = sym + sym_off[b] + (long)j * bd * bd + (long)mu_id * bd;
        double fo = 0, di = 0;
        for (int k = 0; k < bd; ++k) {
            int nu = space[k];
            fo += Y[(long)i * M + nu] * s[k];
            di += X[(long)i * M + nu] * s[k];
        }
        D[e] = di;
        F[e] = fo;
    }
}

// The smallest index of a non-finite entry of X or Y (N x M, already copied).
__global__ void k_first_nonfinite(const double *__restrict__ X, const double *__restrict__ Y,
                                  long n, unsigned long long *__restrict__ first_bad) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        if (!isfinite(X[e]) || !isfinite(Y[e])) atomicMin(first_bad, (unsigned long long)e);
}

}  // namespace tdscha

using namespace tdscha;

extern "C" const char *tdscha_last_error(void) { return g_err; }

extern "C" const char *tdscha_version(void) { return "tdscha_gb300 0.1 sm_103a"; }

static void prof_clear(tdscha_ctx *c) {
    for (auto &v : c->prof_ev) {
        for (auto &e : v) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        v.clear();
    }
}

namespace {
// Freed blocks are kept for reuse by exact size; past the cap the blocks freed
// longest ago are released first (the block just freed is the one a repeated
// context of the same shape asks for next).
struct BlockCache {
    struct Idle {
        int dev;
        size_t bytes;
        void *p;
    };
    std::mutex mu;
    std::unordered_map<void *, std::pair<int, size_t>> live;   // block -> (device, bytes)
    std::list<Idle> order;                                     // idle blocks, oldest first
    std::multimap<std::pair<int, size_t>, std::list<Idle>::iterator> idle;
    size_t idle_bytes = 0;
};
void free_on_device(int dev, void *p) {
    int cur = 0;
    cudaGetDevice(&cur);
    if (dev != cur) cudaSetDevice(dev);
    cudaFree(p);
    if (dev != cur) cudaSetDevice(cur);
}
BlockCache &block_cache() {
    static BlockCache *bc = new BlockCache();   // never destroyed: no cudaFree at exit
    return *bc;
}
// cap on the cached bytes: TDSCHA_BLOCK_CACHE_GIB (GiB; 0 turns caching off),
// default 16
size_t cache_cap() {
    static const size_t cap = [] {
        const char *e = getenv("TDSCHA_BLOCK_CACHE_GIB");
        double gib = e ? atof(e) : 16.0;
        return gib > 0 ? (size_t)(gib * (double)(size_t(1) << 30)) : size_t(0);
    }();
    return cap;
}
}  // namespace

cudaError_t tdscha::cached_malloc(void **p, size_t bytes) {
    if (bytes == 0) bytes = 1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lock(bc.mu);
    auto it = bc.idle.find({dev, bytes});
    if (it != bc.idle.end()) {
        *p = it->second->p;
        bc.order.erase(it->second);
        bc.idle.erase(it);
        bc.idle_bytes -= bytes;
        bc.live[*p] = {dev, bytes};
        return cudaSuccess;
    }
    e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation && !bc.idle.empty()) {
        cudaGetLastError();
        for (auto &b : bc.order) free_on_device(b.dev, b.p);
        bc.order.clear();
        bc.idle.clear();
        bc.idle_bytes = 0;
        e = cudaMalloc(p, bytes);
    }
    if (e == cudaSuccess) bc.live[*p] = {dev, bytes};
    return e;
}

void tdscha::cached_free(void *p) {
    if (!p) return;
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lock(bc.mu);
    auto it = bc.live.find(p);
    if (it == bc.live.end()) {
        cudaFree(p);
        return;
    }
    auto key = it->second;
    bc.live.erase(it);
    const size_t cap = cache_cap();
    if (key.second > cap) {
        free_on_device(key.first, p);
        return;
    }
    // release the blocks freed longest ago until this one fits
    while (!bc.order.empty() && bc.idle_bytes + key.second > cap) {
        BlockCache::Idle &old = bc.order.front();
        auto range = bc.idle.equal_range({old.dev, old.bytes});
        for (auto r = range.first; r != range.second; ++r)
            if (r->second == bc.order.begin()) {
                bc.idle.erase(r);
                break;
            }
        bc.idle_bytes -= old.bytes;
        free_on_device(old.dev, old.p);
        bc.order.pop_front();
    }
    bc.order.push_back({key.first, key.second, p});
    bc.idle.insert({key, std::prev(bc.order.end())});
    bc.idle_bytes += key.second;
}

// returns a block to the device at once, bypassing the idle cache
void tdscha::release_block(void *p) {
    if (!p) return;
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lock(bc.mu);
    auto it = bc.live.find(p);
    if (it == bc.live.end()) {
        cudaFree(p);
        return;
    }
    const int dev = it->second.first;
    bc.live.erase(it);
    free_on_device(dev, p);
}

extern "C" int tdscha_release_cached_memory(unsigned long long *bytes) {
    set_error("");
    cudaDeviceSynchronize();
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lock(bc.mu);
    unsigned long long freed = 0;
    for (auto &b : bc.order) {
        free_on_device(b.dev, b.p);   // on the device it was allocated on
        freed += b.bytes;
    }
    bc.order.clear();
    bc.idle.clear();
    bc.idle_bytes = 0;
    if (bytes) *bytes = freed;
    return TDSCHA_OK;
}

static void ctx_free(tdscha_ctx *c) {
    if (!c) return;
    prof_clear(c);
    mixed_release(c);
    double *bufs[] = {c->w, c->fY, c->fpsi, c->rho, c->Yw, c->ReAw, c->D, c->F, c->pc,
                      c->R1, c->Y1, c->f, c->d2v, c->qp_part, c->alpha, c->beta, c->c1,
                      c->c2, c->gpart, c->fpart, c->Lq, c->pL, c->rk, c->sk, c->mask,
                      c->dots, c->scal, c->hist_dev, c->pqn, c->rcoef, c->Ywinv,
                      c->stat_dev};
    for (double *p : bufs) cached_free(p);
    cached_free(c->tri);
    cached_free(c->lam_static);
    cached_free(c->vsplit);
    cached_free(c->ctr);
    cached_free(c->f2);
    cached_free(c->d2v2);
    free_translations(c);
    psi_free(c);
    if (c->host_pinned) cudaFreeHost(c->host_pinned);
    if (c->stat_host) cudaFreeHost(c->stat_host);
    delete c;
}

template <typename T>
static int dev_alloc(T **p, size_t count) {
    TDS_CUDA(cached_malloc(p, sizeof(T) * (count ? count : 1)));
    return TDSCHA_OK;
}

extern "C" int tdscha_ctx_create(tdscha_ctx **out, int M, int N, const double *X,
                                 const double *Y, const double *w, const double *rho,
                                 double T, int N_syms, int n_blocks, const int *n_deg,
                                 const int *deg_space, const double *sym,
                                 const int *blocks_ids, int with_mixed) {
    set_error("");
    if (!out) { set_error("ctx_create: null output pointer"); return TDSCHA_ERR_ARG; }
    *out = nullptr;
    if (M <= 0 || N <= 0 || N_syms <= 0 || n_blocks <= 0 || n_blocks > M) {
        set_error("ctx_create: bad sizes M=%d N=%d N_syms=%d n_blocks=%d", M, N, N_syms, n_blocks);
        return TDSCHA_ERR_ARG;
    }
    if (!X || !Y || !w || !rho || !n_deg || !deg_space || !sym || !blocks_ids) {
        set_error("ctx_create: null input pointer");
        return TDSCHA_ERR_ARG;
    }
    if (!(T >= 0) || !std::isfinite(T)) { set_error("ctx_create: bad temperature %g", T); return TDSCHA_ERR_ARG; }
    if (with_mixed < 0 || with_mixed > 2) { set_error("ctx_create: with_mixed=%d (0, 1 or 2)", with_mixed); return TDSCHA_ERR_ARG; }
    // validate the symmetry tables so that no device access can leave them
    std::vector<int> deg_off(n_blocks);
    std::vector<long> sym_off(n_blocks);
    long acc_d = 0, acc_s = 0;
    for (int b = 0; b < n_blocks; ++b) {
        if (n_deg[b] <= 0 || n_deg[b] > M) { set_error("ctx_create: n_deg[%d]=%d", b, n_deg[b]); return TDSCHA_ERR_ARG; }
        deg_off[b] = (int)acc_d;
        sym_off[b] = acc_s;
        acc_d += n_deg[b];
        acc_s += (long)N_syms * n_deg[b] * n_deg[b];
    }
    if (acc_d != M) { set_error("ctx_create: blocks cover %ld modes, expected %d", acc_d, M); return TDSCHA_ERR_ARG; }
    for (long k = 0; k < acc_d; ++k)
        if (deg_space[k] < 0 || deg_space[k] >= M) { set_error("ctx_create: deg_space[%ld]=%d out of range", k, deg_space[k]); return TDSCHA_ERR_ARG; }
    for (int mu = 0; mu < M; ++mu) {
        int b = blocks_ids[mu];
        if (b < 0 || b >= n_blocks) { set_error("ctx_create: blocks_ids[%d]=%d out of range", mu, b); return TDSCHA_ERR_ARG; }
        int mu_id = mu - deg_space[deg_off[b]];
        if (mu_id < 0 || mu_id >= n_deg[b]) {
            set_error("ctx_create: mode %d is not inside block %d starting at %d", mu, b, deg_space[deg_off[b]]);
            return TDSCHA_ERR_ARG;
        }
    }
    for (long k = 0; k < acc_s; ++k)
        if (!std::isfinite(sym[k])) { set_error("ctx_create: non-finite symmetry entry"); return TDSCHA_ERR_NAN; }
    // X and Y are checked for non-finite entries on the device (k_expand_images)
    for (int mu = 0; mu < M; ++mu)
        if (!(w[mu] > 0) || !std::isfinite(w[mu])) { set_error("ctx_create: frequency w[%d]=%g must be positive", mu, w[mu]); return TDSCHA_ERR_ARG; }
    double sum_rho = 0;
    for (int i = 0; i < N; ++i) {
        if (!std::isfinite(rho[i])) { set_error("ctx_create: non-finite rho[%d]", i); return TDSCHA_ERR_NAN; }
        sum_rho += rho[i];
    }
    if (sum_rho == 0) { set_error("ctx_create: sum of weights is zero"); return TDSCHA_ERR_ARG; }

    tdscha_ctx *c = new tdscha_ctx();
    cudaGetDevice(&c->device);
    c->M = M; c->N = N; c->S = N_syms; c->R = (long)N * N_syms;
    c->H = (long)M * (M + 1) / 2;
    c->P = M + 2 * c->H;
    c->T = T; c->sum_rho = sum_rho;
    c->with_mixed = with_mixed;

    int rc = TDSCHA_OK;
    std::vector<double> fy(M), fp(M), yw(M), reaw(M);
    for (int mu = 0; mu < M; ++mu) {
        fy[mu] = h_f_ups(w[mu], T);
        fp[mu] = h_f_psi(w[mu], T);
        // Y_w, ReA_w of apply_anharmonic_FT (DynamicalLanczos.py:3024-3031)
        double n_mu = 0;
        if (T > kEps) n_mu = 1.0 / (exp(w[mu] * 157887.32400374097 / T) - 1.0);
        yw[mu] = 2 * w[mu] / (2 * n_mu + 1);
        reaw[mu] = 2 * w[mu] * n_mu * (n_mu + 1) / (2 * n_mu + 1);
    }
    int *d_ndeg = nullptr, *d_degoff = nullptr, *d_space = nullptr, *d_bid = nullptr;
    long *d_symoff = nullptr;
    double *d_sym = nullptr, *d_X = nullptr, *d_Y = nullptr;
    unsigned long long *d_bad = nullptr, h_bad = ~0ULL;
#define TRYC(x) do { rc = (x); if (rc != TDSCHA_OK) goto fail; } while (0)
#define CUC(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { set_error("%s: %s", #x, cudaGetErrorString(_e)); rc = TDSCHA_ERR_CUDA; goto fail; } } while (0)
    TRYC(dev_alloc(&c->w, M)); TRYC(dev_alloc(&c->fY, M)); TRYC(dev_alloc(&c->fpsi, M));
    TRYC(dev_alloc(&c->Yw, M)); TRYC(dev_alloc(&c->ReAw, M)); TRYC(dev_alloc(&c->rho, N));
    CUC(cudaMemcpy(c->w, w, sizeof(double) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(c->fY, fy.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(c->fpsi, fp.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(c->Yw, yw.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(c->ReAw, reaw.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(c->rho, rho, sizeof(double) * N, cudaMemcpyHostToDevice));
    // symmetry images on the perturbation side when the tables allow it
    TRYC(psi_setup(c, n_blocks, n_deg, deg_space, sym, blocks_ids, fy, fp));
    c->Nrows = c->J > 1 ? (long)N : c->R;
    c->rho_div = c->J > 1 ? 1 : N_syms;
    if (c->J > 1) {
        // the N configurations once; no image rows
        TRYC(dev_alloc(&c->D, (size_t)N * M)); TRYC(dev_alloc(&c->F, (size_t)N * M));
        TRYC(dev_alloc(&d_bad, 1));
        CUC(cudaMemcpy(d_bad, &h_bad, sizeof(h_bad), cudaMemcpyHostToDevice));
        CUC(cudaMemcpy(c->D, X, sizeof(double) * N * M, cudaMemcpyHostToDevice));
        CUC(cudaMemcpy(c->F, Y, sizeof(double) * N * M, cudaMemcpyHostToDevice));
        long total = (long)N * M;
        int blocks = (int)std::min<long>((total + 255) / 256, 152L * 16);
        k_first_nonfinite<<<blocks, 256>>>(c->D, c->F, total, d_bad);
        CUC(cudaGetLastError());
        CUC(cudaMemcpy(&h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost));
        if (h_bad != ~0ULL) {
            set_error("ctx_create: non-finite X/Y at %ld", (long)h_bad);
            rc = TDSCHA_ERR_NAN;
            goto fail;
        }
        cached_free(d_bad);
        d_bad = nullptr;
        goto images_done;
    }

    TRYC(dev_alloc(&c->D, (size_t)c->R * M)); TRYC(dev_alloc(&c->F, (size_t)c->R * M));
    TRYC(dev_alloc(&d_X, (size_t)N * M)); TRYC(dev_alloc(&d_Y, (size_t)N * M));
    TRYC(dev_alloc(&d_ndeg, n_blocks)); TRYC(dev_alloc(&d_degoff, n_blocks));
    TRYC(dev_alloc(&d_symoff, n_blocks)); TRYC(dev_alloc(&d_space, M));
    TRYC(dev_alloc(&d_bid, M)); TRYC(dev_alloc(&d_sym, acc_s));
    TRYC(dev_alloc(&d_bad, 1));
    CUC(cudaMemcpy(d_bad, &h_bad, sizeof(h_bad), cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_X, X, sizeof(double) * N * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_Y, Y, sizeof(double) * N * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_ndeg, n_deg, sizeof(int) * n_blocks, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_degoff, deg_off.data(), sizeof(int) * n_blocks, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_symoff, sym_off.data(), sizeof(long) * n_blocks, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_space, deg_space, sizeof(int) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_bid, blocks_ids, sizeof(int) * M, cudaMemcpyHostToDevice));
    CUC(cudaMemcpy(d_sym, sym, sizeof(double) * acc_s, cudaMemcpyHostToDevice));
    {
        long total = c->R * M;
        int blocks = (int)std::min<long>((total + 255) / 256, 152L * 16);
        k_expand_images<<<blocks, 256>>>(d_X, d_Y, N, M, N_syms, d_ndeg, d_degoff, d_symoff,
                                         d_space, d_bid, d_sym, c->D, c->F, d_bad);
        CUC(cudaGetLastError());
        CUC(cudaMemcpy(&h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost));
        if (h_bad != ~0ULL) {
            set_error("ctx_create: non-finite X/Y at %ld", (long)h_bad);
            rc = TDSCHA_ERR_NAN;
            goto fail;
        }
    }
    cached_free(d_X); cached_free(d_Y); cached_free(d_ndeg); cached_free(d_degoff);
    cached_free(d_symoff); cached_free(d_space); cached_free(d_bid); cached_free(d_sym);
    cached_free(d_bad);
    d_X = d_Y = nullptr; d_ndeg = d_degoff = d_space = d_bid = nullptr; d_symoff = nullptr; d_sym = nullptr;
    d_bad = nullptr;
images_done:

    TRYC(dev_alloc(&c->R1, M)); TRYC(dev_alloc(&c->Y1, (size_t)M * M));
    TRYC(dev_alloc(&c->f, M)); TRYC(dev_alloc(&c->d2v, (size_t)M * M));
    TRYC(alloc_fp64_scratch(c));
    TRYC(dev_alloc(&c->Lq, c->P)); TRYC(dev_alloc(&c->pL, c->P));
    TRYC(dev_alloc(&c->rk, c->P)); TRYC(dev_alloc(&c->sk, c->P));
    TRYC(dev_alloc(&c->mask, c->P)); TRYC(dev_alloc(&c->pc, 12 * c->H + 4 * (size_t)M));
    c->nblk_dot = 296;    // block partials of the fused dot kernels (two blocks per SM)
    // block partials: the fused dot kernels (up to 1216 blocks, three sums) and
    // the tiled re-biorthogonalisation update (one per 64 elements)
    TRYC(dev_alloc(&c->dots, std::max<size_t>(4 * (size_t)std::max(c->nblk_dot, 1216),
                                              (size_t)(c->P + 63) / 64)));
    TRYC(dev_alloc(&c->scal, 64));
    TRYC(dev_alloc(&c->ctr, 4));
    CUC(cudaMemset(c->ctr, 0, sizeof(unsigned) * 4));
    CUC(cudaMemset(c->scal, 0, sizeof(double) * 64));
    CUC(cudaMallocHost((void **)&c->host_pinned, sizeof(double) * 64));
    TRYC(build_pair_coeffs(c));
    if (with_mixed) TRYC(mixed_prepare(c));
    CUC(cudaDeviceSynchronize());
    if (with_mixed == 2) {
        // 4-byte storage only: the float64 image rows served the preparation of
        // the fp32 rows and fp16 limbs above and are not read again
        release_block(c->D); c->D = nullptr;
        release_block(c->F); c->F = nullptr;
    }
    *out = c;
    return TDSCHA_OK;
fail:
    cudaDeviceSynchronize();
    cached_free(d_X); cached_free(d_Y); cached_free(d_ndeg); cached_free(d_degoff);
    cached_free(d_symoff); cached_free(d_space); cached_free(d_bid); cached_free(d_sym);
    cached_free(d_bad);
    ctx_free(c);
    return rc;
#undef TRYC
#undef CUC
}

extern "C" int tdscha_ctx_destroy(tdscha_ctx *ctx) {
    if (!ctx) return TDSCHA_OK;
    cudaDeviceSynchronize();
    ctx_free(ctx);
    return TDSCHA_OK;
}

extern "C" int tdscha_ctx_set_options(tdscha_ctx *ctx, int use_wigner, int ignore_harmonic,
                                      int ignore_v3, int ignore_v4, int reverse_L,
                                      double shift_value) {
    set_error("");
    if (!ctx) { set_error("set_options: null context"); return TDSCHA_ERR_ARG; }
    if (!std::isfinite(shift_value)) { set_error("set_options: non-finite shift"); return TDSCHA_ERR_ARG; }
    ctx->use_wigner = use_wigner != 0;
    ctx->ignore_harmonic = ignore_harmonic != 0;
    ctx->ignore_v3 = ignore_v3 != 0;
    ctx->ignore_v4 = ignore_v4 != 0;
    ctx->reverse_L = reverse_L != 0;
    ctx->shift = shift_value;
    // the pair coefficients depend only on the representation (and the
    // context's frequencies and temperature)
    return ctx->pc_wigner == ctx->use_wigner ? TDSCHA_OK : build_pair_coeffs(ctx);
}

namespace tdscha {

// Y1 <- (Y1 + Y1^T) / 2: the quadratic forms of the reference only see the
// symmetric part of Y1 (LanczosFunctions.c:2199-2220 sums both orderings).
__global__ void k_symmetrize(double *Y1, int M) {
    long n = (long)M * M;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        int a = (int)(e / M), b = (int)(e % M);
        if (a < b) {
            double s = 0.5 * (Y1[(long)a * M + b] + Y1[(long)b * M + a]);
            Y1[(long)a * M + b] = s;
            Y1[(long)b * M + a] = s;
        }
    }
}

// Perturbation averages for a Y1 already symmetric in ctx->Y1.
int run_perturb_sym(tdscha_ctx *c, int apply_d4, int precision, cudaStream_t st) {
    if (precision == TDSCHA_PREC_FP64) {
        if (!c->D) {
            set_error("float64 averages requested but the context keeps the ensemble in 4-byte storage only (with_mixed=2)");
            return TDSCHA_ERR_STATE;
        }
        return perturb_fp64(c, apply_d4, st);
    }
    if (precision == TDSCHA_PREC_MIXED) {
        if (!c->with_mixed) { set_error("mixed precision requested but the context was created without it"); return TDSCHA_ERR_STATE; }
        return perturb_mixed(c, apply_d4, st);
    }
    set_error("unknown precision %d", precision);
    return TDSCHA_ERR_ARG;
}

int run_perturb(tdscha_ctx *c, int apply_d4, int precision, cudaStream_t st) {
    k_symmetrize<<<std::max(1, std::min(ceil_div((long)c->M * c->M, 256), 1024)), 256, 0, st>>>(c->Y1, c->M);
    TDS_CHECK_LAUNCH();
    return run_perturb_sym(c, apply_d4, precision, st);
}

}  // namespace tdscha

extern "C" int tdscha_perturb_averages(tdscha_ctx *ctx, const double *R1, const double *Y1,
                                       int apply_D4, int precision, double *f_out,
                                       double *d2v_out, int device_ptrs, void *stream) {
    set_error("");
    if (!ctx || !R1 || !Y1 || !f_out || !d2v_out) { set_error("perturb_averages: null pointer"); return TDSCHA_ERR_ARG; }
    if (apply_D4 != 0 && apply_D4 != 1) {
        set_error("perturb_averages: apply_D4 must be 0 or 1, got %d", apply_D4);
        return TDSCHA_ERR_ARG;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int M = ctx->M;
    cudaMemcpyKind in = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaMemcpyKind outk = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (!device_ptrs) {
        for (int k = 0; k < M; ++k)
            if (!std::isfinite(R1[k])) { set_error("perturb_averages: non-finite R1"); return TDSCHA_ERR_NAN; }
        for (long k = 0; k < (long)M * M; ++k)
            if (!std::isfinite(Y1[k])) { set_error("perturb_averages: non-finite Y1"); return TDSCHA_ERR_NAN; }
    }
    TDS_CUDA(cudaMemcpyAsync(ctx->R1, R1, sizeof(double) * M, in, st));
    TDS_CUDA(cudaMemcpyAsync(ctx->Y1, Y1, sizeof(double) * M * M, in, st));
    TDS_TRY(run_perturb(ctx, apply_D4, precision, st));
    TDS_CUDA(cudaMemcpyAsync(f_out, ctx->f, sizeof(double) * M, outk, st));
    TDS_CUDA(cudaMemcpyAsync(d2v_out, ctx->d2v, sizeof(double) * M * M, outk, st));
    if (!device_ptrs) {
        TDS_CUDA(cudaStreamSynchronize(st));
        TDS_TRY(mixed_check_error(ctx));
    }
    return TDSCHA_OK;
}

extern "C" int tdscha_get_perturb_average_sym(int M, int N, const double *X, const double *Y,
                                              const double *w, const double *rho,
                                              const double *R1, const double *Y1, double T,
                                              int apply_D4, int N_syms, int n_blocks,
                                              const int *n_deg, const int *deg_space,
                                              const double *sym, const int *blocks_ids,
                                              double *f_out, double *d2v_out) {
    if (apply_D4 != 0 && apply_D4 != 1) {
        set_error("GetPerturbAverageSym: apply_D4 must be 0 or 1, got %d", apply_D4);
        return TDSCHA_ERR_ARG;
    }
    tdscha_ctx *c = nullptr;
    TDS_TRY(tdscha_ctx_create(&c, M, N, X, Y, w, rho, T, N_syms, n_blocks, n_deg, deg_space,
                              sym, blocks_ids, 0));
    int rc = tdscha_perturb_averages(c, R1, Y1, apply_D4, TDSCHA_PREC_FP64, f_out, d2v_out, 0, 0);
    std::string keep = tdscha_last_error();
    tdscha_ctx_destroy(c);
    if (rc != TDSCHA_OK) set_error("%s", keep.c_str());
    return rc;
}

extern "C" int tdscha_ctx_set_basis_ld(tdscha_ctx *ctx, long long ld) {
    set_error("");
    if (!ctx) { set_error("set_basis_ld: null context"); return TDSCHA_ERR_ARG; }
    if (ld != 0 && ld < ctx->P) {
        set_error("set_basis_ld: row stride %lld below the vector length %ld", ld, ctx->P);
        return TDSCHA_ERR_ARG;
    }
    ctx->basis_ld = (long)ld;
    return TDSCHA_OK;
}

extern "C" int tdscha_ctx_profile(tdscha_ctx *ctx, int enable) {
    if (!ctx) { set_error("profile: null context"); return TDSCHA_ERR_ARG; }
    if (enable) {
        TDS_CUDA(cudaDeviceSynchronize());
        prof_clear(ctx);
    }
    ctx->prof = enable != 0;
    return TDSCHA_OK;
}

extern "C" int tdscha_ctx_profile_read(tdscha_ctx *ctx, int kernel_id, double *total_ms,
                                       int *launches) {
    if (!ctx || !total_ms || !launches || kernel_id < 0 || kernel_id >= 8) {
        set_error("profile_read: bad arguments");
        return TDSCHA_ERR_ARG;
    }
    TDS_CUDA(cudaDeviceSynchronize());
    double tot = 0;
    for (auto &e : ctx->prof_ev[kernel_id]) {
        float ms = 0;
        TDS_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
        tot += ms;
    }
    *total_ms = tot;
    *launches = (int)ctx->prof_ev[kernel_id].size();
    return TDSCHA_OK;
}

extern "C" int tdscha_ctx_layout(tdscha_ctx *ctx, int *images_on_perturbation,
                                 long long *ensemble_rows) {
    set_error("");
    if (!ctx || !images_on_perturbation || !ensemble_rows) {
        set_error("ctx_layout: null pointer");
        return TDSCHA_ERR_ARG;
    }
    *images_on_perturbation = ctx->J;
    *ensemble_rows = ctx->Nrows;
    return TDSCHA_OK;
}

extern "C" int tdscha_ctx_tuning(tdscha_ctx *ctx, int *stage_a_one_accumulator, int *stage_b_splits,
                                 double *application_ms) {
    set_error("");
    if (!ctx || !stage_a_one_accumulator || !stage_b_splits || !application_ms) {
        set_error("ctx_tuning: null pointer");
        return TDSCHA_ERR_ARG;
    }
    return mixed_tuning(ctx, stage_a_one_accumulator, stage_b_splits, application_ms);
}

extern "C" int tdscha_ctx_sync(tdscha_ctx *ctx, void *stream) {
    set_error("");
    if (!ctx) { set_error("ctx_sync: null context"); return TDSCHA_ERR_ARG; }
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) { set_error("ctx_sync: %s", cudaGetErrorString(e)); return TDSCHA_ERR_CUDA; }
    return mixed_check_error(ctx);
}
