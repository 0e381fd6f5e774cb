/*
 * tdscha_gb300 -- C ABI of the GB300 (sm_103a) Lanczos linear-response engine.
 *
 * Plain pointers and sizes only.  Every entry point returns 0 on success or a
 * negative TDSCHA_ERR_* code (never exits the process); the message of the
 * last failure on the calling thread is available from tdscha_last_error().
 *
 * Layouts follow the reference:
 *   X, Y      : double[N][M] row-major (configuration-major), the ensemble's
 *               displacements / forces in the mass-scaled polarisation basis
 *               (Modules/DynamicalLanczos.py:446-452)
 *   Y1, d2v   : double[M][M] row-major
 *   psi       : double[M + M*(M+1)], sectors R | upper triangle | upper
 *               triangle, triangles stored row by row from the diagonal
 *               (Modules/DynamicalLanczos.py:3326-3345)
 *   symmetry  : n_blocks degenerate blocks; block b has n_deg[b] modes listed
 *               at deg_space[sum_{b'<b} n_deg[b']...]; its N_syms matrices
 *               (N_syms, n_deg[b], n_deg[b]) are stored back to back in `sym`
 *               in block order (the flattened form of the lists passed to
 *               GetPerturbAverageSym, CModules/odd_corr_module.c:491-634);
 *               blocks_ids[M] maps each mode to its block.
 */
#ifndef TDSCHA_GB300_H
#define TDSCHA_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define TDSCHA_OK 0
#define TDSCHA_ERR_ARG (-1)      /* bad argument (size, flag, pointer)          */
#define TDSCHA_ERR_CUDA (-2)     /* CUDA runtime / driver failure               */
#define TDSCHA_ERR_NAN (-3)      /* NaN met in the recurrence or input          */
#define TDSCHA_ERR_STATE (-4)    /* call not valid in the context's state       */
#define TDSCHA_ERR_TIMEOUT (-5)  /* a bounded device wait gave up               */

/* precision of the perturbation averages */
#define TDSCHA_PREC_FP64 0       /* float64 on the CUDA cores                   */
#define TDSCHA_PREC_MIXED 1      /* two-limb fp16 operands, three tensor-core products per K step, fp32 accumulate */

typedef struct tdscha_ctx tdscha_ctx;
typedef struct tdscha_qctx tdscha_qctx;

/* Text of the last error on this thread ("" if none). */
const char *tdscha_last_error(void);

/* Library version string. */
const char *tdscha_version(void);

/*
 * One-shot drop-in for sscha_HP_odd.GetPerturbAverageSym
 * (CModules/odd_corr_module.c:491-634, called from
 * Modules/DynamicalLanczos.py:3114-3116): host buffers in, host buffers out.
 * f_out[M] is overwritten; d2v_out[M*M] is overwritten with the D3 term and
 * the D4 term is added when apply_D4 == 1 (LanczosFunctions.c:2741-2745).
 * Uploads the ensemble, runs in float64 on the GPU, copies back.
 */
int tdscha_get_perturb_average_sym(int M, int N, const double *X, const double *Y,
                                   const double *w, const double *rho,
                                   const double *R1, const double *Y1, double T,
                                   int apply_D4, int N_syms, int n_blocks,
                                   const int *n_deg, const int *deg_space,
                                   const double *sym, const int *blocks_ids,
                                   double *f_out, double *d2v_out);

/*
 * Context: the ensemble uploaded once and kept resident in HBM, with the
 * symmetry images, the per-mode Bose factors and (with_mixed != 0) the fp32
 * rows and two-limb fp16 operands used by TDSCHA_PREC_MIXED.  with_mixed = 0:
 * float64 storage only; 1: both; 2: the mixed operands only (4-byte storage),
 * the float64 image rows released once the operands are built, so that
 * TDSCHA_PREC_FP64 calls on this context return TDSCHA_ERR_STATE.  Replaces
 * the state the reference keeps in `Lanczos`
 * (Modules/DynamicalLanczos.py:183-505, :694-871) and re-sends to the C
 * module on every call.  Host pointers.
 */
int tdscha_ctx_create(tdscha_ctx **out, int M, int N, const double *X, const double *Y,
                      const double *w, const double *rho, double T, int N_syms,
                      int n_blocks, const int *n_deg, const int *deg_space,
                      const double *sym, const int *blocks_ids, int with_mixed);
int tdscha_ctx_destroy(tdscha_ctx *ctx);

/*
 * Flags of the operator (Modules/DynamicalLanczos.py:242-245, :2227-2253):
 * use_wigner, ignore_harmonic, ignore_v3, ignore_v4, reverse_L, shift_value.
 */
int tdscha_ctx_set_options(tdscha_ctx *ctx, int use_wigner, int ignore_harmonic,
                           int ignore_v3, int ignore_v4, int reverse_L, double shift_value);

/*
 * Perturbation averages on the resident ensemble: the context form of
 * GetPerturbAverageSym.  R1[M], Y1[M*M] in; f_out[M], d2v_out[M*M] out, with
 * the same overwrite/add convention as above.  device_ptrs != 0: all four
 * pointers are device memory and the call is asynchronous on `stream`
 * (a cudaStream_t, 0 = legacy default); otherwise host memory, synchronous.
 */
int tdscha_perturb_averages(tdscha_ctx *ctx, const double *R1, const double *Y1,
                            int apply_D4, int precision, double *f_out, double *d2v_out,
                            int device_ptrs, void *stream);

/*
 * psi_out = L psi_in (or L^T psi_in with transpose != 0): the harmonic part
 * (apply_L1_FT, Modules/DynamicalLanczos.py:2287-2445), the anharmonic part
 * (apply_anharmonic_FT, :2951-3363) and the reverse/shift (:3639-3641), as
 * apply_full_L (:3549-3651) computes them.  Device pointers of length
 * M + M*(M+1); asynchronous on `stream`.
 */
int tdscha_apply_full_L(tdscha_ctx *ctx, const double *psi_in, double *psi_out,
                        int transpose, int precision, void *stream);

/*
 * Lanczos iterations (run_FT, Modules/DynamicalLanczos.py:5958-6497) with the
 * reference's default n_rep_orth = 0 (no Gram-Schmidt), bi-Lanczos when
 * run_simm == 0 and the symmetric Wigner Lanczos with the double-counting mask
 * (mask_dot_wigner, :5905-5954) when run_simm != 0.
 *
 * basis_Q, basis_P: device buffers of (capacity) rows of P doubles, row stride
 *   P or the one set by tdscha_ctx_set_basis_ld; rows 0 .. start_step hold
 *   the Krylov vectors already computed (row 0 is the normalised start
 *   vector, which the caller writes before the first call).
 * hist: host double[4 * capacity] holding a_k, b_k, c_k, s_norm_k in rows of 4
 *   for k < start_step (a, b, c) and k <= start_step (s_norm); the call
 *   appends the new rows.  n_iter steps are attempted; *steps_done receives
 *   the number of a_k appended and *converged 1 when |b| or |c| < 1e-12
 *   stopped the run (the last step then appends only a_k, like the reference).
 * full_reorth != 0 adds a full re-biorthogonalisation of each new pair of
 *   vectors against the stored basis (not in the reference's default path).
 */
int tdscha_lanczos_run(tdscha_ctx *ctx, double *basis_Q, double *basis_P, int capacity,
                       int start_step, int n_iter, int run_simm, int precision,
                       int full_reorth, double *hist, int *steps_done, int *converged,
                       void *stream);

/*
 * Row stride (in doubles) of the basis buffers that tdscha_lanczos_run and
 * tdscha_lanczos_run_batch receive for this context: row k of basis_Q starts
 * at basis_Q + k * ld.  0 (the default) means ld = P; otherwise ld >= P.  No
 * counterpart in the reference, whose basis is a list of vectors.  With an even
 * ld and 16-byte aligned basis pointers the re-biorthogonalisation reads two
 * elements per load (the Python layer pads rows to 32 doubles); other layouts
 * take one element per load.
 */
int tdscha_ctx_set_basis_ld(tdscha_ctx *ctx, long long ld);

/*
 * tdscha_lanczos_run with host-memory basis arrays (capacity x P doubles each):
 * rows 0 .. start_step are uploaded, the new rows are copied back; device
 * buffers are allocated and freed inside the call.  For host programs without
 * a CUDA runtime of their own (the input-file executable).  Synchronous.
 */
int tdscha_lanczos_run_hostbuf(tdscha_ctx *ctx, double *basis_Q, double *basis_P, int capacity,
                               int start_step, int n_iter, int run_simm, int precision,
                               int full_reorth, double *hist, int *steps_done, int *converged);

/*
 * Independent Lanczos runs advanced together (the batched workload of
 * independent perturbations, polarisations and q-points): one descriptor per
 * run, real-space (kind 0, ctx a tdscha_ctx, the arguments of
 * tdscha_lanczos_run) or q-space (kind 1, ctx a tdscha_qctx, those of
 * tdscha_qlanczos_run; run_simm and precision ignored).  A context carries
 * the recurrence state of one run, so runs need distinct contexts (several
 * perturbations of one ensemble: one context each).  Every run gets its own
 * stream; up to 16 steps of every active run are launched before any is read
 * back, so the runs' kernels overlap on the GPU.  Fills steps_done, converged
 * and status (0 or a TDSCHA_ERR_*) per run; returns the first error.
 */
typedef struct tdscha_run {
    int kind;
    void *ctx;
    double *basis_Q, *basis_P;
    int capacity, start_step, n_iter;
    int run_simm, precision, reorth;
    double *hist;
    int steps_done, converged, status;
} tdscha_run;
int tdscha_lanczos_run_batch(tdscha_run *runs, int n_runs);

/*
 * Continued-fraction Green function on the GPU, one thread per frequency
 * (get_green_function_continued_fraction, Modules/DynamicalLanczos.py:
 * 5032-5162).  a[n], b[n_b], c[n_c] host arrays; c is used when n_c == n_b,
 * otherwise c = b.  w[n_w] in Ry (host); g_out: host interleaved complex
 * (re, im) of length 2*n_w.
 */
int tdscha_continued_fraction(const double *a, int n, const double *b, int n_b,
                              const double *c, int n_c, const double *w, int n_w,
                              int use_wigner, double modulus, int reverse_L,
                              double shift_value, int use_terminator, int last_average,
                              double smearing, int smooth_ramp, double *g_out);

/*
 * Diagnostics (no counterpart in the reference): per-kernel CUDA-event timing
 * of the perturbation averages.  enable != 0 clears and starts recording,
 * 0 stops.  tdscha_ctx_profile_read returns the total device milliseconds and
 * the launch count recorded for kernel_id: 0 stage A (quadratic forms),
 * 1 row scalars, 2 force average, 3 stage B (weighted outer products),
 * 4 finalisation, 5 operand preparation, 6 re-biorthogonalisation dots and
 * coefficients, 7 re-biorthogonalisation update; it synchronises the device.
 */
int tdscha_ctx_profile(tdscha_ctx *ctx, int enable);
int tdscha_ctx_profile_read(tdscha_ctx *ctx, int kernel_id, double *total_ms, int *launches);

/*
 * How the context holds the symmetry images (no counterpart in the reference,
 * which forms every image row inside its loops, CModules/LanczosFunctions.c:
 * 2158-2170).  *images_on_perturbation = S when the images are applied to the
 * perturbation (Y1 -> S_j^T Y1 S_j, R1 -> S_j^T R1, results carried back by
 * S_j): the ensemble is resident once, *ensemble_rows = N.  This is the case
 * whenever every symmetry matrix maps only between modes of equal frequency
 * factors f_Y and f_psi (degenerate modes).  Otherwise, or with
 * TDSCHA_SYMMETRY_IMAGES=rows in the environment at creation, the N*S image
 * rows are stored: *images_on_perturbation = 1, *ensemble_rows = N*S.
 */
int tdscha_ctx_layout(tdscha_ctx *ctx, int *images_on_perturbation, long long *ensemble_rows);

/*
 * The tensor-core shapes the autotuner chose for a context created with the
 * mixed path (no counterpart in the reference).  At creation the context
 * times one mixed application for each candidate -- stage A with two
 * accumulators on 128 x 128 tiles or one accumulator on 128 x 192 tiles,
 * stage B split counts whose fp32 accumulations stay within about 1.1 x 1024
 * rows -- and keeps the fastest, cached per (modes, rows, images) shape for
 * the process.  TDSCHA_AUTOTUNE=0 keeps the rule-based shape (two
 * accumulators, best wave fill); TDSCHA_STAGEA_ACC=0/1 fixes the stage A
 * kernel.  *application_ms = the timed application (0 when not tuned).
 */
int tdscha_ctx_tuning(tdscha_ctx *ctx, int *stage_a_one_accumulator, int *stage_b_splits,
                      double *application_ms);

/*
 * Float64 perturbation averages that allocate no device memory (no
 * counterpart in the reference).  For callers that cannot let a library call
 * cudaMalloc: host programs that reserve the GPU's memory for their own pool
 * and hand out fixed budgets, and latency-critical loops that cannot accept
 * the device-wide synchronisation cudaMalloc / cudaFree may cause.
 *
 * All pointers are device memory owned by the caller: X, Y (N x M), w (M),
 * rho (N), R1 (M), Y1 (M x M) in; f_out (M), d2v_out (M x M) out, written
 * with the same convention as tdscha_perturb_averages (no symmetry images:
 * one identity image per configuration).  Asynchronous on `stream`.  The
 * results agree with tdscha_perturb_averages (float64) to rounding, not bit
 * for bit: stage B here uses the smallest split-K count.
 *
 * Inputs are checked on the device, not on the host: a non-finite entry of
 * X, Y, R1, Y1 or w, a frequency w <= 0, a negative or non-finite weight in
 * rho, or sum(rho) = 0 makes every entry of f_out and d2v_out NaN (the call
 * itself still returns TDSCHA_OK, since it does not wait for the device).
 *
 * Intermediate arrays live in one static 32 MiB device array that every
 * process loading this library holds on each GPU it uses until exit.  Sizes
 * whose scratch exceeds it (at M=573, N above about 100 000) are rejected
 * with TDSCHA_ERR_ARG and a message giving the bytes needed.  Every call
 * uses the same array (each call writes every word it reads, so nothing
 * carries over), so calls that overlap on the GPU -- on different streams or
 * from different host threads -- race and must be serialised by the caller.
 * The array's device address belongs to a CUDA context (each context that
 * loads the library gets its own copy).  Every call made outside a stream
 * capture looks the address up in the current context; a call made while
 * its stream is being captured reuses the address recorded for the current
 * context, so make a first call in each context before any stream capture
 * (otherwise the call returns TDSCHA_ERR_STATE).
 */
int tdscha_perturb_averages_noalloc(int M, int N, const double *X, const double *Y,
                                    const double *w, const double *rho, const double *R1,
                                    const double *Y1, double T, int apply_D4, double *f_out,
                                    double *d2v_out, void *stream);

/*
 * Static (free-energy Hessian) operator, batched: psi_out[v] = L_static psi_in[v]
 * for v < nvec, device buffers of nvec x (M + M(M+1)/2) doubles (psi = [R | upper-
 * triangle rows of W]).  what = 1: harmonic part apply_L1_static(psi, power)
 * (Modules/DynamicalLanczos.py:2562-2624; power < 0 is its inverse=True form);
 * 2: anharmonic part apply_anharmonic_static (:3369-3430), R1 = psi_R,
 * Y1 = -2 Upsilon psi_W Upsilon, output [-f | d2v upper]; 3: both (the matvec of
 * run_hessian_calculation, :4129-4138, and StaticHessian.apply_L,
 * Modules/StaticHessian.py:561-620).  Asynchronous on stream; ignore_v4 from
 * tdscha_ctx_set_options selects apply_d4.
 */
int tdscha_static_L(tdscha_ctx *ctx, int nvec, const double *psi_in, double *psi_out, int what,
                    double power, int precision, void *stream);

/*
 * StaticHessian vector <-> batch of M static psi rows (StaticHessian.apply_L,
 * Modules/StaticHessian.py:561-691): vec = [G upper-triangle rows (M(M+1)/2) |
 * W_ijk for i <= j <= k (M(M+1)(M+2)/6)], X / Y = M rows of M + M(M+1)/2
 * doubles, row i = [G_i | upper-triangle rows of W_i].  expand fills every
 * row from the symmetric G and W; collect writes G_ij (j >= i) from Y[i][j] and
 * W_ijk (i <= j <= k) from row i.  Device buffers, asynchronous on stream.
 */
int tdscha_static_hessian_expand(tdscha_ctx *ctx, const double *vec, double *X, void *stream);
int tdscha_static_hessian_collect(tdscha_ctx *ctx, const double *Y, double *vec, void *stream);

/* Synchronise stream and report asynchronous failures (CUDA errors, an expired
 * bounded wait of the tensor-core path). */
int tdscha_ctx_sync(tdscha_ctx *ctx, void *stream);

/*
 * Device memory of destroyed contexts (no counterpart in the reference).  The
 * device buffers of a context come from a process-wide cache of freed blocks,
 * reused by exact size by later contexts (creating and destroying contexts
 * of one shape costs no cudaMalloc / cudaFree after the first).  At most
 * TDSCHA_BLOCK_CACHE_GIB GiB (environment, read once; default 16, 0 turns the
 * cache off) stay cached, and an allocation that fails empties the cache and
 * retries.  tdscha_release_cached_memory frees every cached block now (blocks
 * of live contexts are untouched) and writes the bytes released to *bytes
 * (may be null).  It synchronises the device.
 */
int tdscha_release_cached_memory(unsigned long long *bytes);

/*
 * q-space (Bloch basis) operator, float64 complex, Wigner only
 * (QSpaceLanczos, Modules/QSpaceLanczos.py; perturbation averages
 * get_perturb_averages_qspace_fused, Modules/tdscha_qspace.jl:455-712).
 * Complex numbers are interleaved (re, im) doubles everywhere.
 *
 * tdscha_qctx_create: X_q, Y_q host (n_q, N, nb) complex, the Bloch-transformed
 *   mass-scaled displacements and anharmonic forces projected on the q
 *   polarisation vectors (_bloch_transform_ensemble, :221-296); w_q host
 *   (nb, n_q) frequencies in Ry; valid (nb, n_q) 0/1 or NULL (all valid;
 *   valid_modes_q, :181-191); rho (N); n_syms == 0 means the identity only,
 *   otherwise n_syms sparse complex (n_q nb)^2 matrices in CSR form acting on
 *   vectors indexed iq * nb + nu (the q-space symmetry matrices of
 *   prepare_symmetrization, :1472-1657): sym_rowptr (n_syms x (n_q nb + 1)),
 *   each row pointer array indexing sym_col / sym_val (complex) from 0.
 *   nb is limited to 32.  Replaces the Julia-side ensemble cache of
 *   _call_julia_qspace (:775-830).
 */
int tdscha_qctx_create(tdscha_qctx **ctx, int n_q, int nb, int N, const double *X_q,
                       const double *Y_q, const double *w_q, const int *valid,
                       const double *rho, double T, int n_syms, const int *sym_rowptr,
                       const int *sym_col, const double *sym_val);
int tdscha_qctx_destroy(tdscha_qctx *ctx);

/*
 * Perturbation q-point and pairing (build_q_pair_map, :298-333, with the
 * pairing given as q_pair_map[n_q], an involution; pairs (iq1 <= iq2) and the
 * psi layout [R (nb) | a' blocks | b' blocks] follow _compute_block_layout,
 * :335-364).  Writes the complex psi length and the number of pairs.
 */
int tdscha_qctx_set_pert(tdscha_qctx *ctx, int iq_pert, const int *q_pair_map,
                         int ignore_harmonic, int ignore_v3, int ignore_v4, long *psi_size,
                         int *n_pairs);

/*
 * get_perturb_averages_qspace (tdscha_qspace.jl:639-712): R1 (nb complex),
 * alpha1 (n_pairs blocks of nb x nb complex, row-major) in; f_out (nb) and
 * d2v_out (n_pairs x nb x nb) out.  device_ptrs selects device or host
 * buffers; host calls synchronise.
 */
int tdscha_qperturb_averages(tdscha_qctx *ctx, const double *R1, const double *alpha1,
                             int apply_d4, double *f_out, double *d2v_out, int device_ptrs,
                             void *stream);

/* apply_full_L (QSpaceLanczos.py:941-961): device psi_in / psi_out of psi_size complex. */
int tdscha_qapply_full_L(tdscha_qctx *ctx, const double *psi_in, double *psi_out, void *stream);

/*
 * Precision of the q-space averages (no counterpart in the reference, whose
 * Julia kernel is float64): TDSCHA_PREC_FP64 (default) or TDSCHA_PREC_MIXED,
 * where the row, force and d2v kernels run in fp32 on the CUDA cores over
 * float copies of the image rows (made on the first switch; 24-bit operands,
 * partial sums and finalisation in float64).  Applies to every later
 * tdscha_qperturb_averages, tdscha_qapply_full_L, tdscha_qlanczos_run and
 * tdscha_qkpm_run of the context.
 */
int tdscha_qctx_set_precision(tdscha_qctx *ctx, int precision);

/*
 * Hermitian Lanczos (run_FT, QSpaceLanczos.py:967-1182): basis_Q, basis_P
 * distinct device buffers of capacity x (2 psi_size) doubles, rows 0..start_step
 * filled (row 0 the start vector normalised in the mask product, P = Q).
 * reorthogonalize != 0 is the reference's default Gram-Schmidt against all Q
 * vectors with P = Q and s_norm = c (:1110-1125); 0 is its plain recurrence
 * (n_rep_orth = 0).  hist / steps_done / converged as tdscha_lanczos_run.
 */
int tdscha_qlanczos_run(tdscha_qctx *ctx, double *basis_Q, double *basis_P, int capacity,
                        int start_step, int n_iter, int reorthogonalize, double *hist,
                        int *steps_done, int *converged, void *stream);

/*
 * Ensemble preprocessing on the GPU (one call per run; host buffers in and out).
 * tdscha_project_modes (Modules/DynamicalLanczos.py:392-452): u, f (N x n_cart)
 * displacements and forces minus SSCHA forces, f_mean (n_cart, may be NULL),
 * masses (n_cart), pols (n_cart x M) ->
 *   X = (u u_scale sqrt(m)) . pols,  Y = ((f f_scale - f_mean f_scale) / sqrt(m)) . pols
 * tdscha_project_bloch (Modules/QSpaceLanczos.py:221-296): complex interleaved
 * u_q, f_q (n_q x N x n_cart), pols_q (n_q x n_cart x nb), f_mean_gamma (n_cart,
 * subtracted at q index 0, may be NULL) ->
 *   X_q = (u_q u_scale sqrt(m)) . conj(pols_q),  Y_q = ((f_q - f_mean) f_scale / sqrt(m)) . conj(pols_q)
 */
int tdscha_project_modes(int N, int n_cart, int M, const double *u, const double *f,
                         const double *f_mean, const double *masses, const double *pols,
                         double u_scale, double f_scale, double *X_out, double *Y_out);
int tdscha_project_bloch(int n_q, int N, int n_cart, int nb, const double *u_q, const double *f_q,
                         const double *f_mean_gamma, const double *masses, const double *pols_q,
                         double u_scale, double f_scale, double *X_q, double *Y_q);

/*
 * gamma_only (DynamicalLanczos.py:746-786, :3173-3191): the supercell's lattice
 * translations as Cartesian index permutations perms (n_trans x n_cart, the
 * reference's trans_cart_perms) and pols (n_cart x M).  Every later operator
 * application (tdscha_apply_full_L, tdscha_lanczos_run) projects the averages:
 * f <- P_t f, d2v <- pols^T mean_R Perm_R(pols d2v pols^T) pols.  n_trans = 0
 * removes it.
 */
int tdscha_ctx_set_translations(tdscha_ctx *ctx, int n_cart, const double *pols, int n_trans,
                                const int *perms);

/*
 * Chebyshev moments of the q-space operator (QSpaceKPM.run_KPM,
 * Modules/QSpaceKPM.py:260-454, main loop :413-440): for k = n_start, ... while
 * 2k < n_moments: moments[2k] = 2 <v, v>_M - moments[0]; then
 * vp = 2 (L v - b v)/a - vm, moments[2k+1] = 2 <vp, v>_M - moments[1] and
 * (vm, v) <- (v, vp).  vm, v, work: distinct device buffers of 2 psi_size
 * doubles (T_{k-1}, T_k applied to the start vector); moments: device, with
 * moments[0], moments[1] set.  On return the final (vm, v) pair is in (vm, v)
 * when *swapped == 0, in (v, vm) otherwise.  <x, y>_M is the Wigner metric
 * Re(x^H (mask y)).
 */
int tdscha_qkpm_run(tdscha_qctx *ctx, double *vm, double *v, double *work, int n_start,
                    int n_moments, double rescale_a, double rescale_b, double *moments,
                    int *swapped, void *stream);

/*
 * Learned continued-fraction terminator (no counterpart in the reference): a
 * 3-layer perceptron h1 = tanh(x W1 + b1), h2 = tanh(h1 W2 + b2), y = h2 W3 + b3,
 * trained on the GPU (float32 forward / backward, mean-squared error, Adam).
 * Parameters flat: W1 (n_in x n_hidden), b1, W2 (n_hidden x n_hidden), b2,
 * W3 (n_hidden x n_out), b3, weights row-major.  forward / loss_grad take host
 * buffers; train_step takes device buffers (x: rows x n_in, t: rows x n_out).
 * bf16 != 0 in forward rounds weights and layer inputs to bfloat16 (float32
 * accumulation).
 */
typedef struct tdscha_mlp tdscha_mlp;
int tdscha_mlp_create(tdscha_mlp **mlp, int n_in, int n_hidden, int n_out);
int tdscha_mlp_destroy(tdscha_mlp *mlp);
long tdscha_mlp_num_params(const tdscha_mlp *mlp);
int tdscha_mlp_set_params(tdscha_mlp *mlp, const float *params);
int tdscha_mlp_get_params(tdscha_mlp *mlp, float *params);
int tdscha_mlp_forward(tdscha_mlp *mlp, const float *x, int rows, int bf16, float *y);
int tdscha_mlp_loss_grad(tdscha_mlp *mlp, const float *x, const float *t, int rows, float *loss,
                         float *grad);
int tdscha_mlp_train_step(tdscha_mlp *mlp, const float *x, const float *t, int rows, float lr,
                          float beta1, float beta2, float eps, int step, float *loss,
                          void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TDSCHA_GB300_H */
