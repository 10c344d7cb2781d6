/* CPU restatement of PSOCI's Hamiltonian-build / sigma path — TEST INFRASTRUCTURE ONLY.
 *
 * Used by tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU baseline
 * leg.  The psoci_gb300 product never links or loads this library.
 */
#ifndef PSOCI_ORACLE_H
#define PSOCI_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* h, so: nbf*nbf row-major (symmetric one-electron, antisymmetric spin-orbit);
 * eri: canonical 8-fold packed two-electron table of nbf(nbf+1)/2*(nbf(nbf+1)/2+1)/2 doubles;
 * occ: nconf*nbf bytes of 0/1/2; jsym: nconf 1-based spatial symmetry labels. */
orc_ctx *orc_create(int nbf, int nelec, int ksym, int mx_open, int nconf, const int *jsym,
                    const unsigned char *occ, const double *h, const double *so, const double *eri);
void orc_destroy(orc_ctx *c);
long orc_num_sefs(const orc_ctx *c);
void orc_config_counts(const orc_ctx *c, int *out);
int orc_config_dets(const orc_ctx *c, int i, int *out);
double orc_fetch1e(const orc_ctx *c, int i, int j);
double orc_fetch2e(const orc_ctx *c, int i, int j, int k, int l);
int orc_block(const orc_ctx *c, int i, int j, double *out);
long orc_build_lower(orc_ctx *c, int nthreads);
void orc_copy_lower(const orc_ctx *c, long *rowptr, int *cols, double *vals);
long orc_build_rows(orc_ctx *c, int nthreads, const int *rows, int nrows);
/* the rows of the last orc_build_rows (the sampled configurations' SEF rows, in order) */
void orc_sample_counts(const orc_ctx *c, long *nrows, long *nnz);
void orc_copy_sample(const orc_ctx *c, long *rowptr, int *cols, double *vals);
void orc_diag(const orc_ctx *c, double *diag);
void orc_sigma_lower(long n, const long *rowptr, const int *cols, const double *vals, int k,
                     const double *x, double *y, int nthreads);
/* 1-particle density (CIDEN): block of pair (i, j) and the packed densities of k roots
 * (vecs: k x N root-major; dens: k x nbf(nbf+1)/2). */
int orc_ciden_block(const orc_ctx *c, int i, int j, double *out);
void orc_density1(const orc_ctx *c, int k, const double *vecs, double *dens);
/* the reference's CPU sigma (one vector, rows over threads) and Davidson loop (see .c) */
void orc_sigma_lower_rows(long n, const long *rowptr, const int *cols, const double *vals, const double *x,
                          double *y, int nthreads);
int orc_davidson_ref(long n, const long *rowptr, const int *cols, const double *vals, const double *diag,
                     int nroots, int maxsub, double rtol, int max_iter, int nthreads, double *evals, double *rnorms,
                     long *stats);
/* energy gradients with respect to the packed tables (see psoci_oracle.c) */
void orc_energy_gradient(const orc_ctx *c, int k, const double *vecs, int nonzero_only, double *grad_one,
                         double *grad_eri, int nthreads);
void orc_density1_rows(const orc_ctx *c, int k, const double *vecs, int nrows, const int *rows, double *dens);

#ifdef __cplusplus
}
#endif
#endif
