/*
 * ORACLE -- test infrastructure only.  CPU restatement of the reference's
 * symmetrised perturbation averages, used by tests/, by smoke() and by the
 * CPU-baseline leg of bench.py as the checker.  The product (the CUDA
 * library under tdscha_gb300/csrc) never links or calls this file.
 *
 * Follows, operation by operation (same loop nests, same evaluation order,
 * so a single-threaded run is bit-identical to the reference's C module):
 *   get_f_average_from_Y_pert_sym_fast   CModules/LanczosFunctions.c:2082-2254
 *   get_d2v_dR2_from_R_pert_sym_fast     CModules/LanczosFunctions.c:2257-2438
 *   get_d2v_dR2_from_Y_pert_sym_fast     CModules/LanczosFunctions.c:2615-2754
 *   driver GetPerturbAverageSym          CModules/odd_corr_module.c:491-634
 * The only change: f_psi / f_ups (LanczosFunctions.c:14-30) are evaluated
 * once per mode instead of inside the M^2 loops (same function, same inputs,
 * same bits).  Multi-threading (n_threads > 1) splits the configurations in
 * contiguous slices like the reference's MPI split (LanczosFunctions.c:
 * 2124-2137) and sums the slices in rank order.
 *
 * Symmetry tables are flattened: block b owns n_deg[b] modes listed at
 * deg_space[deg_off[b] ...], and its S matrices (S, deg, deg) start at
 * sym[sym_off[b]]; offsets are prefix sums over the blocks.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define ORACLE_RY_TO_K 157887.32400374097

static double o_f_ups(double w, double T) {
    double n_w = 0;
    if (T > 0) n_w = 1 / (exp(w * ORACLE_RY_TO_K / T) - 1);
    return 2 * w / (1 + 2 * n_w);
}

static double o_f_psi(double w, double T) {
    double n_w = 0;
    if (T > 0) n_w = 1 / (exp(w * ORACLE_RY_TO_K / T) - 1);
    return (1 + 2 * n_w) / (2 * w);
}

typedef struct {
    const double *X, *Y, *w, *rho, *R1, *Y1;
    double T;
    int apply_d4, M, N, S;
    const int *n_deg, *deg_space, *blocks_ids;
    const int *deg_off;
    const long *sym_off;
    const double *sym;
    const double *fps, *fus;
    int start, stop;
    double *f_acc;      /* M   */
    double *d3_acc;     /* M*M */
    double *d4_acc;     /* M*M */
} oracle_job;

/* d = S_j X_i, f = S_j Y_i, block by block (LanczosFunctions.c:2158-2170). */
static void sym_image(const oracle_job *J, int i, int j, double *force, double *disp) {
    int M = J->M;
    for (int mu = 0; mu < M; ++mu) {
        force[mu] = 0;
        disp[mu] = 0;
        int b = J->blocks_ids[mu];
        const int *space = J->deg_space + J->deg_off[b];
        int mu_id = mu - space[0];
        int bd = J->n_deg[b];
        const double *s = J->sym + J->sym_off[b] + (long)j * bd * bd + (long)mu_id * bd;
        for (int k = 0; k < bd; ++k) {
            int nu = space[k];
            force[mu] += J->Y[(long)i * M + nu] * s[k];
            disp[mu] += J->X[(long)i * M + nu] * s[k];
        }
    }
}

static void *oracle_worker(void *arg) {
    oracle_job *J = (oracle_job *)arg;
    int M = J->M;
    double *force = (double *)calloc(M, sizeof(double));
    double *disp = (double *)calloc(M, sizeof(double));
    const double *Y1 = J->Y1, *R1 = J->R1, *fps = J->fps, *fus = J->fus;
    for (int i = J->start; i < J->stop; ++i) {
        double wi = J->rho[i];
        for (int j = 0; j < J->S; ++j) {
            sym_image(J, i, j, force, disp);
            double weight;
            /* f average, D4 part (LanczosFunctions.c:2199-2230) */
            weight = 0;
            for (int mu = 0; mu < M; ++mu)
                for (int nu = 0; nu < M; ++nu)
                    weight -= disp[mu] * disp[nu] * Y1[mu * M + nu] / 2;
            for (int mu = 0; mu < M; ++mu)
                J->f_acc[mu] += wi * weight * force[mu] / 3;
            weight = 0;
            for (int mu = 0; mu < M; ++mu) {
                double f_mu = fps[mu] * force[mu];
                for (int nu = 0; nu < M; ++nu) {
                    double f_nu = fps[nu] * force[nu];
                    weight -= disp[mu] * f_nu * Y1[mu * M + nu] / 4;
                    weight -= disp[nu] * f_mu * Y1[mu * M + nu] / 4;
                }
            }
            for (int mu = 0; mu < M; ++mu) {
                double u_mu = fus[mu] * disp[mu];
                J->f_acc[mu] += wi * weight * u_mu * 2 / 3.;
            }
            /* d2v, D3 part (LanczosFunctions.c:2374-2408) */
            weight = 0;
            for (int mu = 0; mu < M; ++mu) weight += fus[mu] * R1[mu] * disp[mu];
            for (int mu = 0; mu < M; ++mu) {
                double u_mu = fus[mu] * disp[mu];
                for (int nu = 0; nu < M; ++nu) {
                    J->d3_acc[mu * M + nu] -= u_mu * force[nu] * weight * wi / 3;
                    J->d3_acc[nu * M + mu] -= u_mu * force[nu] * weight * wi / 3;
                }
            }
            weight = 0;
            for (int mu = 0; mu < M; ++mu) weight += R1[mu] * force[mu];
            for (int mu = 0; mu < M; ++mu) {
                double u_mu = fus[mu] * disp[mu];
                for (int nu = 0; nu < M; ++nu) {
                    double u_nu = fus[nu] * disp[nu];
                    J->d3_acc[mu * M + nu] -= u_mu * u_nu * weight * wi / 3;
                }
            }
            if (!J->apply_d4) continue;
            /* d2v, D4 part (LanczosFunctions.c:2687-2725) */
            weight = 0;
            for (int mu = 0; mu < M; ++mu)
                for (int nu = 0; nu < M; ++nu)
                    weight -= disp[mu] * disp[nu] * Y1[mu * M + nu];
            weight *= wi / 8;
            for (int mu = 0; mu < M; ++mu) {
                double u_mu = fus[mu] * disp[mu];
                for (int nu = 0; nu < M; ++nu) {
                    J->d4_acc[mu * M + nu] -= force[nu] * u_mu * weight;
                    J->d4_acc[nu * M + mu] -= force[nu] * u_mu * weight;
                }
            }
            weight = 0;
            for (int mu = 0; mu < M; ++mu) {
                double f_mu = fps[mu] * force[mu];
                for (int nu = 0; nu < M; ++nu) {
                    double f_nu = fps[nu] * force[nu];
                    weight -= f_mu * disp[nu] * Y1[mu * M + nu];
                    weight -= f_nu * disp[mu] * Y1[mu * M + nu];
                }
            }
            weight *= wi / 8;
            for (int mu = 0; mu < M; ++mu) {
                double u_mu = fus[mu] * disp[mu];
                for (int nu = 0; nu < M; ++nu) {
                    double u_nu = fus[nu] * disp[nu];
                    J->d4_acc[mu * M + nu] -= u_nu * u_mu * weight;
                }
            }
        }
    }
    free(force);
    free(disp);
    return NULL;
}

/*
 * Returns 0, or -1 on a bad argument.  f_out (M) and d2v_out (M*M) are
 * overwritten, as GetPerturbAverageSym does (f and the D3 term overwrite,
 * the D4 term is added on top: LanczosFunctions.c:2741-2745).
 */
int oracle_perturb_averages(const double *X, const double *Y, const double *w,
                            const double *rho, const double *R1, const double *Y1,
                            double T, int apply_d4, int M, int N, int S,
                            int n_blocks, const int *n_deg, const int *deg_space,
                            const double *sym, const int *blocks_ids,
                            double *f_out, double *d2v_out, int n_threads) {
    if (M <= 0 || N <= 0 || S <= 0 || n_blocks <= 0) return -1;
    if (apply_d4 != 0 && apply_d4 != 1) return -1;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > N) n_threads = N;

    int *deg_off = (int *)malloc(sizeof(int) * n_blocks);
    long *sym_off = (long *)malloc(sizeof(long) * n_blocks);
    int acc_d = 0;
    long acc_s = 0;
    for (int b = 0; b < n_blocks; ++b) {
        deg_off[b] = acc_d;
        sym_off[b] = acc_s;
        acc_d += n_deg[b];
        acc_s += (long)S * n_deg[b] * n_deg[b];
    }
    double *fps = (double *)malloc(sizeof(double) * M);
    double *fus = (double *)malloc(sizeof(double) * M);
    for (int mu = 0; mu < M; ++mu) {
        fps[mu] = o_f_psi(w[mu], T);
        fus[mu] = o_f_ups(w[mu], T);
    }

    oracle_job *jobs = (oracle_job *)calloc(n_threads, sizeof(oracle_job));
    pthread_t *th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    int count = N / n_threads, rem = N % n_threads;
    for (int r = 0; r < n_threads; ++r) {
        oracle_job *J = &jobs[r];
        J->X = X; J->Y = Y; J->w = w; J->rho = rho; J->R1 = R1; J->Y1 = Y1;
        J->T = T; J->apply_d4 = apply_d4; J->M = M; J->N = N; J->S = S;
        J->n_deg = n_deg; J->deg_space = deg_space; J->blocks_ids = blocks_ids;
        J->deg_off = deg_off; J->sym_off = sym_off; J->sym = sym;
        J->fps = fps; J->fus = fus;
        J->start = r < rem ? r * (count + 1) : r * count + rem;
        J->stop = J->start + count + (r < rem ? 1 : 0);
        J->f_acc = (double *)calloc(M, sizeof(double));
        J->d3_acc = (double *)calloc((size_t)M * M, sizeof(double));
        J->d4_acc = (double *)calloc((size_t)M * M, sizeof(double));
    }
    if (n_threads == 1) {
        oracle_worker(&jobs[0]);
    } else {
        for (int r = 0; r < n_threads; ++r) pthread_create(&th[r], NULL, oracle_worker, &jobs[r]);
        for (int r = 0; r < n_threads; ++r) pthread_join(th[r], NULL);
    }

    double N_eff = 0;
    for (int i = 0; i < N; ++i) N_eff += rho[i];
    for (int mu = 0; mu < M; ++mu) {
        double s = 0;
        for (int r = 0; r < n_threads; ++r) s += jobs[r].f_acc[mu];
        f_out[mu] = s;
        f_out[mu] /= N_eff * S;
    }
    for (long k = 0; k < (long)M * M; ++k) {
        double s3 = 0, s4 = 0;
        for (int r = 0; r < n_threads; ++r) {
            s3 += jobs[r].d3_acc[k];
            s4 += jobs[r].d4_acc[k];
        }
        d2v_out[k] = s3;
        d2v_out[k] /= N_eff * S;
        if (apply_d4) d2v_out[k] += s4 / (N_eff * S);
    }
    for (int r = 0; r < n_threads; ++r) {
        free(jobs[r].f_acc);
        free(jobs[r].d3_acc);
        free(jobs[r].d4_acc);
    }
    free(jobs); free(th); free(fps); free(fus); free(deg_off); free(sym_off);
    return 0;
}
