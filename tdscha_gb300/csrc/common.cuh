// Internal declarations shared by the translation units of libtdscha_gb300.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "../../include/tdscha_gb300.h"

namespace tdscha {

constexpr double kRyToK = 157887.32400374097;   // LanczosFunctions.h:9
constexpr double kEps = 1e-12;                   // DynamicalLanczos.py:121

void set_error(const char *fmt, ...);

#define TDS_CUDA(call)                                                               \
    do {                                                                             \
        cudaError_t _e = (call);                                                     \
        if (_e != cudaSuccess) {                                                     \
            ::tdscha::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,           \
                                cudaGetErrorString(_e));                             \
            return TDSCHA_ERR_CUDA;                                                  \
        }                                                                            \
    } while (0)

#define TDS_CHECK_LAUNCH()                                                           \
    do {                                                                             \
        cudaError_t _e = cudaGetLastError();                                         \
        if (_e != cudaSuccess) {                                                     \
            ::tdscha::set_error("%s:%d launch: %s", __FILE__, __LINE__,              \
                                cudaGetErrorString(_e));                             \
            return TDSCHA_ERR_CUDA;                                                  \
        }                                                                            \
    } while (0)

#define TDS_TRY(expr)                                                                \
    do {                                                                             \
        int _rc = (expr);                                                            \
        if (_rc != TDSCHA_OK) return _rc;                                            \
    } while (0)

// Two-limb fp16 copies of the ensemble used by the tensor-core path.  Rows are
// image rows r = i*S + j (configuration-major, like the reference's bigindex,
// tdscha_core.jl:212-238).  Mp is M padded to the tile width; Rp is R padded
// to the K block of the second GEMM.
struct MixedStore {
    int Mp = 0;
    long Rp = 0;
    // row layout (R x Mp): A operand of V = D Y1, and the epilogue's rows
    __half *d_hi = nullptr, *d_lo = nullptr;
    float *g32 = nullptr;    // g = f_psi * f rows (fp32)      R x Mp
    // transposed layout (Mp x Rp): operands of G = U^T W
    __half *ut_hi = nullptr, *ut_lo = nullptr;          // U^T, U = f_Y * D
    float *ft32 = nullptr;                               // F^T (fp32)
    float *ut32 = nullptr;                               // U^T (fp32)
    __half *wt_hi = nullptr, *wt_lo = nullptr;          // W^T, rebuilt per call
    __half *y1_hi = nullptr, *y1_lo = nullptr;          // Y1 (Mp x Mp), per call
    float *qp = nullptr;          // per-column-tile partial q, p, s, t  (ntile x 4 x R)
    float *gpart = nullptr;       // split-K partial G            (nsplit x Mp x Mp)
    int nsplit = 0;
    int nctile = 0;
    void *tmaps = nullptr;        // device copy of the TMA descriptors
    std::vector<uint8_t> tmaps_host;
    int *err_flag = nullptr;      // bounded-wait failure flag (device)
};

}  // namespace tdscha

struct tdscha_ctx {
    int device = 0;
    int M = 0, N = 0, S = 0;
    long R = 0;                 // image rows N*S
    long P = 0;                 // psi length M + M(M+1)
    long H = 0;                 // M(M+1)/2
    double T = 0, sum_rho = 0;  // sum_rho accumulated in config order
    int with_mixed = 0;     // 0 float64 only, 1 float64 + mixed, 2 mixed with 4-byte storage only
    // operator options
    int use_wigner = 1, ignore_harmonic = 0, ignore_v3 = 0, ignore_v4 = 0, reverse_L = 0;
    int pc_wigner = -1;          // representation the pair coefficients were built for
    double shift = 0;
    // per-mode (device)
    double *w = nullptr, *fY = nullptr, *fpsi = nullptr, *rho = nullptr;
    double *Yw = nullptr, *ReAw = nullptr;     // equilibrium Upsilon / ReA eigenvalues
    double *Ywinv = nullptr;                    // 1 / Yw
    int *tri = nullptr;                         // (row, column) of each upper-triangle pair
    double *lam_static = nullptr;               // static pair factor Lambda (H), on first use
    // gamma-only translation projection (tdscha_ctx_set_translations)
    int tr_ncart = 0, tr_ntrans = 0;
    double *tr_pols = nullptr, *tr_proj = nullptr, *tr_w1 = nullptr, *tr_w2 = nullptr,
           *tr_w3 = nullptr, *tr_f = nullptr;
    int *tr_perms = nullptr;
    // rows of the ensemble (device), Nrows x M: the N configurations when the
    // symmetry images act on the perturbation (J > 1, symmetry.cu), else the
    // R = N*S image rows r = i*S + j
    double *D = nullptr, *F = nullptr;
    long Nrows = 0;
    int rho_div = 1;            // row r of D belongs to configuration r / rho_div
    // perturbation-side images: J = S when the images are applied to the
    // perturbation, 1 when they are materialised (or S = 1).  S_j as sparse
    // tables of maxdeg entries per mode: column-sparse (rows k with
    // S_j[k][m] != 0) and row-sparse (columns k with S_j[m][k] != 0), index -1
    // for unused slots.  [J][M][maxdeg] each.
    int J = 1, maxdeg = 1;
    int *sc_idx = nullptr, *sr_idx = nullptr;
    double *sc_val = nullptr, *sr_val = nullptr;
    float2 *sr_val2 = nullptr;  // sr_val as double-float pairs (mixed path)
    float2 *sc_val2 = nullptr;  // sc_val as double-float pairs (mixed path)
    double *Y1all = nullptr;    // float64 path, J x M x M: S_j^T Y1 S_j
    double *vsv = nullptr;      // J x M: S_j^T (f_Y R1), then J x M: S_j^T R1
    double *hs = nullptr;       // J x M x M: G_j + G_j^T summed over the splits
    // per-pair coefficients (device), length H, rebuilt by set_options
    double *pc = nullptr;       // 10 arrays of H: see lanczos.cu
    // per-application scratch (device)
    double *R1 = nullptr, *Y1 = nullptr, *f = nullptr, *d2v = nullptr;
    double *f2 = nullptr, *d2v2 = nullptr;   // second output of a two-perturbation call
    double *qp_part = nullptr;  // fp64 path: nct x 2 x R
    double *alpha = nullptr, *beta = nullptr, *c1 = nullptr, *c2 = nullptr;   // R each
    double *gpart = nullptr;    // fp64 path: nsplit x M x M
    double *fpart = nullptr;    // nfchunk x M
    int nct64 = 0, nsplit64 = 0, nfchunk = 0;
    // Lanczos work vectors (device), P each
    double *Lq = nullptr, *pL = nullptr, *rk = nullptr, *sk = nullptr;
    double *mask = nullptr;     // Wigner double-counting mask (P)
    double *dots = nullptr;     // block partials of the fused dot kernels
    unsigned *ctr = nullptr;    // last-block counters of the fused dot kernels (zero between launches)
    double *scal = nullptr;     // device scalars of the recurrence
    double *hist_dev = nullptr; // device copy of the coefficient history
    int hist_cap = 0;
    double *stat_dev = nullptr; // per-step recurrence status (device)
    double *stat_host = nullptr;// pinned read-back area (history rows + status)
    int stat_cap = 0;
    double *pqn = nullptr;      // p_j . q_j of the stored basis (full reorthogonalisation)
    double *rcoef = nullptr;    // projection coefficients (2 per basis vector)
    int pqn_cap = 0;
    float2 *vsplit = nullptr;   // 2 x ldv: double-float splits of the masked new pair
    long basis_ld = 0;          // row stride of the Lanczos basis buffers (0: P)
    double *host_pinned = nullptr;
    int nblk_dot = 0;
    tdscha::MixedStore mx;
    // diagnostics: CUDA-event pairs per kernel id while profiling is on
    int prof = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[8];
};

// q-space (Bloch basis) context, see qspace.cu
struct tdscha_qctx {
    int n_q = 0, nb = 0, N = 0, S = 1;
    long R = 0;          // image rows N * S
    int L = 0;           // n_q * nb (length of one image row)
    double T = 0, sum_rho = 0;
    double2 *Xr = nullptr, *Yr = nullptr;      // R x L image rows
    double *fY = nullptr, *fpsi = nullptr;     // [q][nu] (0 for masked modes)
    double *rho = nullptr;
    std::vector<double> w_q;                   // [nu][q] host copy
    std::vector<int> valid;                    // [nu][q]
    // perturbation layout (tdscha_qctx_set_pert)
    int iq_pert = -1, n_pairs = 0;
    long P = 0;                                // complex psi length
    int ignore_harmonic = 0, ignore_v3 = 0, ignore_v4 = 0;
    int *qpair = nullptr, *qrole = nullptr, *qpartner = nullptr;   // per q
    int *pair_q = nullptr;                     // 2 per pair
    int *elem = nullptr;                       // per psi element: sector | pair | nu1 | nu2
    double *pcoef = nullptr;                   // per pair block element: 6 coefficients
    double *mask = nullptr;                    // 2P (per real component)
    long *q_off = nullptr;                     // block offsets: a' (n_pairs), b' (n_pairs)
    double *wpert = nullptr;                   // -(w^2) at q_pert (0 for masked modes)
    // per-call scratch
    double2 *R1 = nullptr, *alpha = nullptr, *f = nullptr, *d2v = nullptr;
    double2 *rowc = nullptr;                   // 4 per image row
    double2 *fpart = nullptr, *dpart = nullptr;
    // mixed precision (tdscha_qctx_set_precision): float copies of the image
    // rows and frequency factors, per-call float perturbation and row weights
    int precision = 0;
    float2 *Xr32 = nullptr, *Yr32 = nullptr;
    float *fY32 = nullptr, *fpsi32 = nullptr;
    float2 *R1_32 = nullptr, *alpha32 = nullptr, *rowc32 = nullptr;
    int nfchunk = 0, nbchunk = 0;
    // Lanczos scratch (2P doubles each)
    double *Lq = nullptr, *rk = nullptr, *sk = nullptr;
    double *dots = nullptr, *scal = nullptr, *hist_dev = nullptr, *stat_dev = nullptr;
    double *stat_host = nullptr, *pqn = nullptr, *rcoef = nullptr;
    int hist_cap = 0;
};

namespace tdscha {

// perturb_fp64.cu
int perturb_fp64(tdscha_ctx *c, int apply_d4, cudaStream_t st);
int alloc_fp64_scratch(tdscha_ctx *c);
// perturb_mixed.cu
int mixed_prepare(tdscha_ctx *c);
int mixed_release(tdscha_ctx *c);
int perturb_mixed(tdscha_ctx *c, int apply_d4, cudaStream_t st);
// the same with Y1 and R1 unpacked from psi inside the operand preparation
// (plain layout, or the transposed one with its per-pair factors cty / ctra)
int perturb_mixed_psi(tdscha_ctx *c, int apply_d4, const double *psi, const double *cty,
                      const double *ctra, cudaStream_t st);
// The two applications of a bi-Lanczos step in one call: perturbation a from
// psi_a in the plain layout, b from psi_b in the transposed one (per-pair
// factors cty, ctra); results in (f, d2v) and (f2, d2v2).
int perturb_mixed_pair(tdscha_ctx *c, int apply_d4, const double *psi_a, const double *psi_b,
                       const double *cty, const double *ctra, cudaStream_t st);
int mixed_check_error(tdscha_ctx *c);
// the autotuner's choice: stage A kernel (1: one accumulator per 128 x 192
// tile), stage B split count, and the timed application (ms; 0: not tuned)
int mixed_tuning(tdscha_ctx *c, int *one_acc, int *nsplit, double *ms);
// lanczos.cu
int build_pair_coeffs(tdscha_ctx *c);
int apply_full_L_dev(tdscha_ctx *c, const double *psi_in, double *psi_out, int transpose,
                     int precision, cudaStream_t st);
// qspace.cu
int q_apply_full_L_dev(tdscha_qctx *c, const double *psi_in, double *psi_out, cudaStream_t st);
// preprocess.cu
int apply_translation_projection(tdscha_ctx *c, cudaStream_t st);
void free_translations(tdscha_ctx *c);
// shared: f / d2v finalisation from the row scalars and G partials
int finalize_avgs(tdscha_ctx *c, int nsplit, const double *gpart, cudaStream_t st);
// symmetry.cu: perturbation-side symmetry images
int psi_setup(tdscha_ctx *c, int n_blocks, const int *n_deg, const int *deg_space,
              const double *sym, const int *blocks_ids, const std::vector<double> &fy,
              const std::vector<double> &fp);
void psi_free(tdscha_ctx *c);
// J x M vectors S_j^T (f_Y R1) and S_j^T R1 into c->vsv, and (float64 path) the
// J matrices S_j^T Y1 S_j into c->Y1all
int psi_perturbation64(tdscha_ctx *c, cudaStream_t st);
// d2v = -(1 / (S sum rho)) sum_j S_j (G_j + G_j^T) S_j^T and f = (1 / (S sum
// rho)) sum_j S_j fsum_j from split-K partials G_js[a][b] = gpart[s*sstride +
// j*jstride + a*lda + b] and force partials fpart[(j*nfchunk + chunk)*M + m]
int psi_finalize64(tdscha_ctx *c, const double *gpart, int nsplit, long sstride, long jstride,
                   long lda, const double *fpart, int nfchunk, cudaStream_t st);
int psi_finalize32(tdscha_ctx *c, const float *gpart, int nsplit, long sstride, long jstride,
                   long lda, const float *fpart, int nfchunk, double *f_out, double *d2v_out,
                   cudaStream_t st);

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// Device buffers of contexts come from a process-wide cache of freed blocks,
// reused by exact size: applications create and destroy contexts of the same
// shapes over and over (one per ensemble, perturbation or q-point), and
// cudaMalloc / cudaFree of a context's buffers cost about 4 ms of a 22 ms
// 20-step run at M=573, N=50 000.  At most TDSCHA_BLOCK_CACHE_GIB GiB (default
// 16, 0 turns caching off) stay cached, larger surpluses are released with
// cudaFree, an allocation that fails empties the cache and retries once, and
// tdscha_release_cached_memory empties it on request.  cached_free of a pointer that did not come from
// cached_malloc calls cudaFree.  A block is cached only after its last use:
// callers free after synchronising.
cudaError_t cached_malloc(void **p, size_t bytes);
void cached_free(void *p);
// frees a block at once (cudaFree), whether it came from cached_malloc or not
void release_block(void *p);
template <typename T>
inline cudaError_t cached_malloc(T **p, size_t bytes) {
    return cached_malloc(reinterpret_cast<void **>(p), bytes);
}

// Programmatic dependent launch.  A kernel started by launch_pdl is scheduled
// as the blocks of the kernel before it in the stream exit, so its launch and
// block set-up (and the barrier / TMEM set-up of the persistent kernels) hide
// behind that kernel's tail.  Its threads call pdl_enter() before touching
// global memory: it returns once the earlier kernels have completed and their
// writes are visible.  No kernel triggers its dependents early: blocks of the
// next kernel resident during a whole kernel took SM slots from its last wave
// and made the Lanczos step slower (1365 steps/s against 1413 without
// dependent launch and about 1500 with the launch at block exit, M=573,
// N=50 000).  Launched the usual way, pdl_enter() is a no-op.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args &&...args) {
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Bracket a launch with CUDA events when profiling is on.
struct ProfScope {
    tdscha_ctx *c;
    int id;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    ProfScope(tdscha_ctx *c_, int id_, cudaStream_t st_) : c(c_), id(id_), st(st_) {
        if (c->prof) {
            cudaEventCreate(&a);
            cudaEventRecord(a, st);
        }
    }
    ~ProfScope() {
        if (c->prof && a) {
            cudaEvent_t b;
            cudaEventCreate(&b);
            cudaEventRecord(b, st);
            c->prof_ev[id].push_back({a, b});
        }
    }
};

}  // namespace tdscha
