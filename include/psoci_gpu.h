/* psoci_gpu.h — C ABI of the GB300 Hamiltonian-build / Davidson-sigma library
 * (libpsoci_gpu.so, built from psoci_gb300/csrc for sm_103a).
 *
 * The library replaces, on one GPU, the data-parallel path of PSOCI that runs from the
 * determinant layer through the Davidson subspace step.  Each entry point names the
 * reference interface it stands in for (paths inside psociRestart-Cori/).  Global Arrays /
 * DRA storage becomes device arrays owned by the context; there are no MPI ranks.
 *
 * Conventions
 *   - every function returns a psoci_status; none aborts the process;
 *   - orbital, configuration and SEF indices are 0-based;
 *   - one context = one device + one CUDA stream; calls on one context are not thread-safe;
 *   - "host" pointers are ordinary host memory; the *_device variants take device pointers
 *     valid on the context's device and run on the context's stream.
 */
#ifndef PSOCI_GPU_H
#define PSOCI_GPU_H
#include <stdint.h>
#include <stddef.h>

#if defined(__GNUC__)
#define PSOCI_API __attribute__((visibility("default")))
#else
#define PSOCI_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PSOCI_OK = 0,
  PSOCI_ERR_INVALID_ARG = 1,  /* bad sizes, null pointers, out-of-range labels          */
  PSOCI_ERR_UNSUPPORTED = 2,  /* > 11 open shells, nbf > 128, ... (reference limits)     */
  PSOCI_ERR_STATE = 3,        /* call order violated (e.g. sigma before build)           */
  PSOCI_ERR_CUDA = 4,         /* CUDA runtime error; psoci_last_error() has the text      */
  PSOCI_ERR_NOMEM = 5,        /* device allocation failed                                 */
  PSOCI_ERR_TIMEOUT = 6,      /* a bounded device-side wait ran out                       */
  PSOCI_ERR_NOT_CONVERGED = 7,/* Davidson hit its iteration limit                         */
  PSOCI_ERR_NUMERIC = 8,      /* NaN/Inf met in a residual or subspace matrix             */
  PSOCI_ERR_IO = 9            /* file missing, truncated or of the wrong format           */
} psoci_status;

typedef struct psoci_ctx psoci_ctx;

typedef struct {
  int device;        /* CUDA device ordinal                                       */
  int verbose;       /* 0 silent, 1 phase timings on stderr                        */
} psoci_opts;

/* Precision of the stored Hamiltonian used by sigma. */
typedef enum {
  PSOCI_PREC_FP64 = 0,   /* FP64 elements, FP64 products and sums                        */
  PSOCI_PREC_MIXED = 1,  /* FP32 elements and FP32 products, FP64 accumulation            */
  PSOCI_PREC_FF = 2      /* FP64 elements and inputs as FP32 hi+lo pairs, float-float      */
                         /* products and sums (about 47 bits) on the FP32 pipe             */
} psoci_prec;

typedef enum {
  PSOCI_HMODE_CSR_FP64 = 0,   /* stored FP64 CSR only                                   */
  PSOCI_HMODE_CSR_BOTH = 1,   /* stored FP64 CSR plus an FP32 copy of the elements      */
  PSOCI_HMODE_DIRECT = 2      /* nothing stored: neighbour lists and the diagonal only;  */
                              /* every sigma evaluates the elements again (FP64)         */
} psoci_hmode;

/* Replaces GA::Initialize + the PsociGAhamiltonian constructor
 * (driver.PSOCI.splittest.C:296, PsociGAhamiltonian.C:269). */
PSOCI_API psoci_status psoci_create(psoci_ctx **ctx, const psoci_opts *opts);
/* Replaces PsociGAhamiltonian::destroyGAspace and friends. */
PSOCI_API void psoci_destroy(psoci_ctx *ctx);
PSOCI_API const char *psoci_status_str(psoci_status s);
/* Text of the last error on this context (CUDA message, bad argument, ...). */
PSOCI_API const char *psoci_last_error(const psoci_ctx *ctx);

/* Replaces PsociIntegrals::fetchAndProcessIntegrals (PsociIntegrals.C:914-961) and the
 * broadcast of the packed tables (:559, :780).
 *   one_packed: nbf(nbf+1)/2 doubles, entry (i>=j) at i(i+1)/2+j, holding h_ij for equal
 *               irreps and the spin-orbit value SO_ij (i>j) otherwise — the table layout
 *               of PsociIntegrals.C:505-535;
 *   eri_packed: canonical 8-fold table, NNDAF(NNDAF(nbf)) doubles (PsociIntegrals.C:889). */
PSOCI_API psoci_status psoci_set_integrals(psoci_ctx *ctx, int nbf, const double *one_packed,
                                 const double *eri_packed, double ecore);

/* Replaces PsociConfigs::readConfigsToGA (PsociConfigs.C:336-496) once the file is parsed:
 * nconf configurations in file order (SEF index = running sum of nsef in this order),
 * occ = nconf*nbf bytes of 0/1/2, jsym = 1-based spatial symmetry per configuration.
 * Unlike the reference (PsociConfigs.C:247), all-open-shell configurations are accepted. */
PSOCI_API psoci_status psoci_set_configs(psoci_ctx *ctx, int nbf, int nelec, int ksym, int mx_open,
                               int nconf, const int32_t *jsym, const uint8_t *occ);

/* Replaces PsociGADeterminants::generateDistributedDeterminantsSmallMemoryGA
 * (PsociGADeterminants.C:1608-1731) / PsociDeterminants::computeConfigs
 * (PsociDeterminants.C:856-975) and computeNsefEntryPoints (PsociGAhamiltonian.C:4022).
 * Builds determinant bit-strings, phases and spin projections on the device. */
PSOCI_API psoci_status psoci_build_determinants(psoci_ctx *ctx);
/* Counts after psoci_build_determinants. */
PSOCI_API psoci_status psoci_get_counts(const psoci_ctx *ctx, int64_t *nsef_total, int64_t *ndet_total,
                              int *max_nsef, int *max_ndet);
/* Host copy of the determinant table, for parity checks.  Per determinant d:
 * alpha[d*words+w], beta[d*words+w] (bit p = orbital p), phase[d] (0/1), ms[d]
 * (the reference's spin_projection); detoff/sefoff: nconf+1 prefix sums.  words = ceil(nbf/64).
 * Any output pointer may be NULL. */
PSOCI_API psoci_status psoci_get_determinants(const psoci_ctx *ctx, uint64_t *alpha, uint64_t *beta,
                                    uint8_t *phase, int32_t *ms, int64_t *detoff, int64_t *sefoff);

/* Replaces PsociGAhamiltonian::constructGlobalHamiltonianAltOrbMapDirectChunkJmap
 * (PsociGAhamiltonian.C:2530-2857) with packSefsef (:4077-4136): the full symmetric H in CSR
 * (both triangles; each off-diagonal element is the reference's lower-triangle value), elements
 * with |x| >= 1e-8 or on the diagonal.  *nnz receives the stored count.
 * PSOCI_HMODE_DIRECT stands in for the reference's direct products
 * (matrixVectorProductsSplitChunkMultipleJchunksLowLevelAccumulateDirectFetch,
 * PsociGAhamiltonian.C:7549-7826, built with DIRECTMATRIXPRODUCTS): only the screened
 * neighbour lists and the diagonal are kept (*nnz = 0); psoci_sigma / psoci_sigma_device /
 * psoci_davidson then evaluate every element again on each call, in FP64 whatever the
 * precision asked for, applying the same |x| >= 1e-8 rule.  psoci_get_hamiltonian,
 * psoci_save_hamiltonian and psoci_sigma_mixed_noalloc answer PSOCI_ERR_STATE. */
PSOCI_API psoci_status psoci_build_hamiltonian(psoci_ctx *ctx, psoci_hmode mode, int64_t *nnz);
/* Counters and phase times of the last psoci_build_hamiltonian.  Times are CUDA-event
 * intervals on the library stream, in milliseconds; the evaluation time covers the final
 * attempt only (an undersized value slab makes the build evaluate twice).  The reference
 * reports its build time through PsociTimer; there is no direct counterpart. */
typedef struct {
  int64_t candidates;    /* configuration pairs the screen tested one by one (ordered): all   */
                         /* pairs within two excitations (all-pairs screen), or those left  */
                         /* after the per-hi-pattern integral test (lookup screen)          */
  int64_t pairs;         /* of those, pairs whose block is not zero from the integrals alone */
  int64_t segments;      /* warp work items (<= 32 neighbours of one row configuration)      */
  int64_t nnz;           /* stored elements, both triangles                                  */
  int64_t nnz_lower;     /* the reference's lower-triangle count, (nnz + N) / 2              */
  int64_t slab_slots;    /* value-slab slots taken by the evaluation                         */
  int evaluations;       /* 1, or 2 after a slab overflow                                    */
  int fast;              /* 1: lower blocks evaluated once and mirrored; 0: generic path      */
  int lookup_screen;     /* 1: neighbours found by table lookup; 0: all-pairs test            */
  int eval_launches;     /* fast path: 2 masks and elements launched apart, 1 one launch;    */
                         /* 0 otherwise                                                     */
  double screen_ms, evaluate_ms, rows_ms, assemble_ms, total_ms;
} psoci_build_info;
PSOCI_API psoci_status psoci_build_stats(const psoci_ctx *ctx, psoci_build_info *info);
/* The fast build evaluates its elements in two launches (the determinant-connectivity masks,
 * 8 bytes per (pair, row SEF), then the elements) when those masks fit in a quarter of the
 * free device memory, else in one launch.  launches = 1 asks for the one-launch form (less
 * memory, slower), 0 for the automatic choice (the default).  The stored matrix is the same
 * bit for bit either way.  No counterpart in the reference (a GPU scheduling choice). */
PSOCI_API psoci_status psoci_set_eval_launches(psoci_ctx *ctx, int launches);

/* Replaces PsociHamiltonian::generateSOCIblocks (PsociHamiltonian.C:401-558) for a batch of
 * configuration pairs: block q is the reference's nsef_A x nsef_B sefsef matrix for
 * (A[q], B[q]) in the reference's roles, row-major, stored consecutively in out (host) in
 * pair order; pairs beyond a double excitation give zero blocks.  Needs the determinants. */
PSOCI_API psoci_status psoci_blocks(psoci_ctx *ctx, int npairs, const int32_t *A, const int32_t *B, double *out);
/* Host copy of the CSR (rowptr[N+1], cols[nnz], vals[nnz]); NULLs allowed. */
PSOCI_API psoci_status psoci_get_hamiltonian(const psoci_ctx *ctx, int64_t *rowptr, int32_t *cols, double *vals);
/* Host copy of selected rows of the stored CSR (both triangles), replacing the row fetches of
 * PsociGAhamiltonian::fetchLocalHblock (PsociGAhamiltonian.C:11791-11852): rows[nrows] SEF
 * indices; rowptr[nrows+1] receives the offsets of each row's entries; cols / vals (both NULL
 * to ask for the counts only) receive rowptr[nrows] entries, rows in the order given and each
 * in ascending column order. */
PSOCI_API psoci_status psoci_get_rows(const psoci_ctx *ctx, int nrows, const int64_t *rows, int64_t *rowptr,
                                      int32_t *cols, double *vals);
/* Replaces PsociGAhamiltonian::fetchDIAG_SEF / fetchDiags (PsociGAhamiltonian.C:9014). */
PSOCI_API psoci_status psoci_get_diag(const psoci_ctx *ctx, double *diag);

/* Replaces PsociGAhamiltonian::matrixVectorProductsSplitChunkMultipleJchunks
 * (PsociGAhamiltonian.C:6921-7270), k vectors at once.  X, Y: N x k, row-major (element
 * (r, v) at r*k+v), host memory. */
PSOCI_API psoci_status psoci_sigma(psoci_ctx *ctx, int k, const double *X, double *Y, psoci_prec prec);
/* Same on device memory, rows of leading dimension ld (>= k), on the context stream. */
PSOCI_API psoci_status psoci_sigma_device(psoci_ctx *ctx, int k, const double *dX, int ldx, double *dY,
                                int ldy, psoci_prec prec);

/* Mixed-precision sigma that allocates no device memory, for callers that cannot call
 * cudaMalloc while they run: host programs whose own allocator owns the whole GPU memory
 * budget (as the reference's Global Arrays runtime takes a fixed memory size per rank up
 * front), and loops that must not take the implicit device synchronisation an allocation
 * can cause.  Same arguments and result as psoci_sigma_device with PSOCI_PREC_MIXED, but
 * the FP32 copy of the input is staged in a fixed 16 MiB device array compiled into the
 * library (held by every device that loads it until the process exits) instead of a buffer
 * grown with cudaMalloc.  Limit: N * 8 <= 4 Mi floats, i.e. at most 524,288 SEFs; larger
 * problems get PSOCI_ERR_UNSUPPORTED, a direct-mode build or one without the FP32 copy
 * PSOCI_ERR_STATE.  All calls and all contexts on a device share the array, which keeps the
 * last call's contents (each call overwrites what it reads first, so nothing must start at
 * zero); calls that overlap on the GPU race and must be serialised by the caller.  The first
 * call on a device looks up the array's address (cudaGetSymbolAddress) and caches it: make
 * that first call before any stream capture begins.
 * No counterpart in the reference. */
PSOCI_API psoci_status psoci_sigma_mixed_noalloc(psoci_ctx *ctx, int k, const double *dX, int ldx, double *dY,
                                                 int ldy);

typedef struct {
  int nroots;          /* roots wanted                                                  */
  int max_subspace;    /* basis size that triggers a collapse; 0: 8*nroots, at most 96  */
                       /* (the reference collapses at 4*nroots)                          */
  int max_iter;        /* iteration limit (reference: 1000 per tolerance)                */
  double rtol;         /* residual-norm tolerance for convergence                        */
  psoci_prec prec;     /* sigma precision during the iterations                          */
  int refine;          /* after a MIXED run: 1 refine with PSOCI_PREC_FF sigma,          */
                       /* 2 refine with PSOCI_PREC_FP64 sigma, 0 no refinement           */
  int block;           /* 1: block Davidson (all unconverged roots per iteration);
                          0: one new vector per iteration, as the reference does          */
  double precond_min;  /* |D_i - lambda| guard of the preconditioner (reference 1e-3)     */
} psoci_dav_opts;

typedef struct {
  int iterations;      /* Davidson iterations                                            */
  int sigma_calls;     /* H*v products (counted per vector)                              */
  int collapses;       /* subspace contractions                                          */
  int refine_iters;    /* refinement iterations after the mixed phase                    */
  double seconds;      /* wall time of psoci_davidson                                    */
  double sigma_seconds;/* device time inside sigma kernels                               */
} psoci_dav_stats;

/* Replaces the Davidson loop of driver.PSOCI.splittest.C:1186-1311 with
 * PsociGAsubspace::generateIncrementalSubspace / diagSubspaceGOP / computeRnormSingle
 * (PsociGAsubspace.C:273-366, :1088-1171, :874-1000) and PsociGAbasis precondition /
 * orthonormalize / expandAndReplaceVectorsNew (PsociGAbasis.C:1860-1919, :1371-1474,
 * :483-583).  Initial guess: unit vectors on the nroots lowest diagonal elements.
 * evals[nroots] are electronic energies (add ecore for totals); evecs (N x nroots,
 * column-major: root r at r*N) and rnorms[nroots] may be NULL. */
PSOCI_API psoci_status psoci_davidson(psoci_ctx *ctx, const psoci_dav_opts *opts, double *evals,
                            double *evecs, double *rnorms, psoci_dav_stats *stats);

/* Sigma autotuner: times each of the 6 variants of the mixed-precision sigma kernel — lanes
 * per row x stored elements in flight per lane: 0 (32 x 4), 1 (32 x 2), 2 (16 x 4), 3 (16 x 2),
 * 4 (8 x 4), 5 (16 x 6) — on k random vectors with CUDA events on the context's stream and
 * keeps the fastest for this Hamiltonian (a new build resets it to variant 0).  choice
 * receives it; times_ms (6 entries, may be NULL) the best of three runs of each.  k = 0 times
 * nothing and installs the variant given in *choice (0..5).  Needs a stored build with the
 * FP32 copy.  No counterpart in the reference. */
PSOCI_API psoci_status psoci_autotune_sigma(psoci_ctx *ctx, int k, int *choice, float *times_ms);

/* Batched Davidson over several double-group symmetry blocks, one context each (the reference
 * solves one ksym block per job, driver.PSOCI.splittest.C:1186-1311): block b is solved as
 * psoci_davidson(ctxs[b], &opts[b], evals[b], evecs[b], rnorms[b], &stats[b]) would solve it,
 * all blocks at once — each on its context's own stream, driven by its own host thread, so
 * the kernels of the blocks overlap on the GPU and one block's host-side eigen-solve overlaps
 * the others' kernels.  Before a block's first MIXED solve after a build, its sigma variant is
 * chosen by psoci_autotune_sigma.  evecs and rnorms may be NULL, or hold NULL entries;
 * block_status (may be NULL) receives each block's status; the return value is the first
 * failing block's status.  The contexts must be distinct. */
PSOCI_API psoci_status psoci_davidson_batch(psoci_ctx *const *ctxs, int nblocks, const psoci_dav_opts *opts,
                                            double *const *evals, double *const *evecs, double *const *rnorms,
                                            psoci_dav_stats *stats, psoci_status *block_status);

/* Tall-skinny projection C = A^T B on device memory — the product behind
 * PsociGAsubspace::generateIncrementalSubspace (PsociGAsubspace.C:273-366) — by one of three
 * methods: 0 float-float sums on the FP32 pipe (what psoci_davidson runs), 1 FP64 FMA, 2 FP64
 * tensor-core MMA (mma.sync m8n8k4 .f64).  A: n x m (row stride lda), B: n x k (row stride ldb),
 * C: m x k row-major; 1 <= m <= 40, 1 <= k <= 8.  Runs on the context's stream and returns
 * when C is written.  For measuring the methods against one another. */
PSOCI_API psoci_status psoci_tsprod(psoci_ctx *ctx, int method, int64_t n, const double *dA, int lda, int m,
                                    const double *dB, int ldb, int k, double *dC);

/* Step-level Davidson: the basis and subspace of the reference's own loop
 * (driver.PSOCI.splittest.C:1186-1311), held on the device between calls so that a host
 * program keeps that loop as it is.  One basis per context: V and H*V (N x max_vectors), the
 * projected matrix G = V^T H V, its eigenpairs and the residuals of the sought roots.  The
 * vectors are kept orthonormal, so the overlap S of the reference is the identity and its
 * generalised eigen-solve (dsygv) a symmetric one.  psoci_davidson stays the fast path.
 * Calls that change the basis invalidate what depends on it (a new vector needs its G
 * columns, a new G its eigen-solve, a new eigen-solve its residuals); calls made out of that
 * order answer PSOCI_ERR_STATE.  Rebuilding the Hamiltonian of another space invalidates the
 * basis. */
/* PsociGAbasis(numSoughtRoots, hamilton, g_v, g_Hv) and PsociGAsubspace(basis, diag, g_rnorms)
 * constructors (PsociGAbasis.C, PsociGAsubspace.C): room for max_vectors (nroots+1 .. 96)
 * vectors of the built Hamiltonian's dimension; replaces an earlier basis. */
PSOCI_API psoci_status psoci_basis_create(psoci_ctx *ctx, int nroots, int max_vectors);
/* PsociGAsubspace::destroySubspace (PsociGAsubspace.C:194) with the basis's arrays. */
PSOCI_API void psoci_basis_destroy(psoci_ctx *ctx);
/* PsociGAvectors::specifyDiagonalGuessVectors (PsociGAvectors.C:687-726): nroots unit vectors;
 * mode 0 on the first nroots SEFs (the reference), 1 on the nroots lowest diagonal elements,
 * 2 the vectors of psoci_set_guess (the -r restart) completed as in mode 1.  No products yet. */
PSOCI_API psoci_status psoci_basis_guess(psoci_ctx *ctx, int mode);
/* PsociGAbasis::normAllVectors + orthonormalizeAllVectors (PsociGAbasis.C:1044, :1210) of the
 * guess set (at most nroots vectors); a linear dependency gives PSOCI_ERR_NUMERIC with the
 * 1-based column in *dependent_at (may be NULL). */
PSOCI_API psoci_status psoci_basis_orthonormalize_all(psoci_ctx *ctx, int *dependent_at);
/* PsociGAbasis::computeHvProducts(start, num) (PsociGAbasis.C:1610): H*v of vectors
 * start..start+num-1 with the sigma of the given precision. */
PSOCI_API psoci_status psoci_basis_compute_hv(psoci_ctx *ctx, int start, int num, psoci_prec prec);
/* PsociGAsubspace::generateIncrementalSubspace(num) (PsociGAsubspace.C:273-366): the columns of
 * G = V^T (H V) for the last num vectors (FP64 sums, float-float on the FP32 pipe). */
PSOCI_API psoci_status psoci_subspace_generate_incremental(psoci_ctx *ctx, int num);
/* PsociGAsubspace::diagSubspaceGOP + brdcstEvals (PsociGAsubspace.C:1088-1171): eigenpairs of
 * G (host, as the reference's dsygv); evals receives the existing-count eigenvalues ascending. */
PSOCI_API psoci_status psoci_subspace_diag(psoci_ctx *ctx, double *evals);
/* PsociGAsubspace::computeRnormSingle (PsociGAsubspace.C:874-1000): the residual norm of Ritz
 * vector iroot (1-based, <= nroots); the residual is kept for psoci_basis_precondition_new. */
PSOCI_API psoci_status psoci_subspace_rnorm_single(psoci_ctx *ctx, int iroot, double *rnorm);
/* PsociGAsubspace::computeRnorms (PsociGAsubspace.C:775-872): the residual norms of all sought
 * roots (rnorms[nroots]); the residuals are kept. */
PSOCI_API psoci_status psoci_subspace_rnorms(psoci_ctx *ctx, double *rnorms);
/* PsociGAbasis::preconditionAndNewVectorIncore (PsociGAbasis.C:1807-1919): the scratch vector
 * t_i = r_i / (D_i - shift) where |D_i - shift| > precond_min (reference 1e-3), else r_i, from
 * the kept residual of root curroot (1-based). */
PSOCI_API psoci_status psoci_basis_precondition_new(psoci_ctx *ctx, int curroot, double shift, double precond_min);
/* PsociGAbasis::appendScratchVector -> appendVectors (PsociGAbasis.C:362, :725-842):
 * orthonormalise the scratch vector against the basis, append it and form its H*v; *appended
 * receives 1, or 0 when no new direction survived (the basis is unchanged).  A full basis
 * answers PSOCI_ERR_STATE (the reference fails there too): call psoci_basis_expand_replace. */
PSOCI_API psoci_status psoci_basis_append_scratch(psoci_ctx *ctx, psoci_prec prec, int *appended);
/* PsociGAbasis::expandAndReplaceVectorsNew(evecs, num) (PsociGAbasis.C:483-583): the num lowest
 * Ritz vectors of the last eigen-solve replace the basis, V <- V Y and H*V <- (H*V) Y without
 * new products; G becomes diagonal.  Y spans the vectors of that eigen-solve, so a vector
 * appended after it is dropped, as in the reference's collapse.  With num = existing after
 * the last eigen-solve the first nroots vectors are the solution. */
PSOCI_API psoci_status psoci_basis_expand_replace(psoci_ctx *ctx, int num);
/* CurrentExistingRoots, CurrentNumSoughtRoots, CurrentMaxRoots, present_matrixProducts of
 * PsociGAbasis (PsociGAbasis.C:137-173); NULLs allowed. */
PSOCI_API psoci_status psoci_basis_info(const psoci_ctx *ctx, int *existing, int *sought, int *max_vectors,
                                        int *products);
/* The first k basis vectors to the host, root-major (vector j at j*N). */
PSOCI_API psoci_status psoci_basis_vectors(psoci_ctx *ctx, int k, double *vecs);

/* Eigenpairs of a symmetric n x n matrix G (row stride ldg; the halves are averaged): the
 * eigen-solve of PsociGAsubspace::diagSubspaceGOP (PsociGAsubspace.C:1088-1171, LAPACK dsygv)
 * with the unit metric of an orthonormal basis, as psoci_davidson runs it.  w[n] ascending;
 * Y (row stride ldy) column c = eigenvector c.  Householder tridiagonalisation and implicit
 * QR with the Wilkinson shift.  Host computation; needs no context or device. */
PSOCI_API psoci_status psoci_subspace_eigen(int n, const double *G, int ldg, double *w, double *Y, int ldy);

/* Initial guess for the next psoci_davidson (the reference's -r vector restart,
 * driver.PSOCI.splittest.C:962-972): k vectors of length N, root-major (vector r at r*N).
 * Missing roots are completed with unit vectors on the lowest diagonal elements.
 * k = 0 clears the guess. */
PSOCI_API psoci_status psoci_set_guess(psoci_ctx *ctx, int k, const double *vecs);

/* Spin-free 1-particle density of k CI vectors (the reference's CI-density path,
 * PsociGAhamiltonian::constructCIdensityAltOrbMapChunkJmap, PsociGAhamiltonian.C:11570-11760,
 * with blocks from PsociHamiltonian::generateSOCIblocksForCIDEN, PsociHamiltonian.C:572-705,
 * contracted as transformSEFSEFtoMOGET, PsociGAhamiltonian.C:10027-10099).  vecs: k vectors
 * of length N, root-major (as psoci_davidson returns them).  dens: k x nbf(nbf+1)/2 doubles,
 * root-major, packed lower triangle D[p(p+1)/2 + q], p >= q (twoDindex).  The diagonal holds
 * the orbital occupations; an off-diagonal element holds the sum over unordered configuration
 * pairs one electron apart (same jsym) of c_I S_IJ c_J, once per pair, as the reference
 * accumulates it.  Needs psoci_build_determinants; the Hamiltonian is not used. */
PSOCI_API psoci_status psoci_density1(psoci_ctx *ctx, int k, const double *vecs, double *dens);
/* psoci_density1 on device memory: dV k vectors with stride ldv (root-major), dD k x
 * nbf(nbf+1)/2 (overwritten); runs on the context's stream and returns without waiting.
 * The first call after new configurations also forms the configuration groups. */
PSOCI_API psoci_status psoci_density1_device(psoci_ctx *ctx, int k, const double *dV, int64_t ldv, double *dD);

/* Energy gradients with respect to the integral tables (Hellmann-Feynman): for each of k CI
 * vectors c_r (normalised eigenvectors, root-major k x N), dE_r/d one[t] and dE_r/d eri[t] of
 * E_r = c_r^T H c_r, in the packed layouts psoci_set_integrals takes.  grad_one (k x
 * nbf(nbf+1)/2): the spin-free 1-particle density on entries of equal irreps (diagonal: the
 * occupations of psoci_density1; off the diagonal: twice its value) and the spin-orbit density
 * dE/dSO_pq on entries of unequal irreps; grad_eri (k x NNDAF(NNDAF(nbf))): the 2-particle
 * density in the reference's canonical 8-fold packed layout (PsociIntegrals.C:889-909).
 * There is no counterpart in the reference, whose only density is the CIDEN 1-particle
 * density; the kernel is the adjoint of the element evaluation (PsociHamiltonian.C:139-1118):
 * every determinant coupling adds its weight to the table entries its element reads.
 * mode 0: every pair of configurations within two excitations, so every entry's derivative
 * (also of integrals that are zero); mode 1: pairs whose integral prefactors are all zero are
 * skipped and the entries of zero integrals are reported as 0 (the derivatives of the
 * non-zero integrals, at less work).  prec: PSOCI_PREC_FP64, or PSOCI_PREC_MIXED (sums within
 * a configuration pair in FP32, across pairs in FP64).  The state average of the k roots is
 * the mean of the k gradients.  Needs psoci_build_determinants; the Hamiltonian is not used. */
PSOCI_API psoci_status psoci_energy_gradient(psoci_ctx *ctx, int k, const double *vecs, int mode, psoci_prec prec,
                                             double *grad_one, double *grad_eri);
/* The same on device memory: dV k vectors with stride ldv (root-major), dG1 k x nbf(nbf+1)/2,
 * dG2 k x NNDAF(NNDAF(nbf)) (overwritten); returns after the kernels have finished. */
PSOCI_API psoci_status psoci_energy_gradient_device(psoci_ctx *ctx, int k, const double *dV, int64_t ldv, int mode,
                                                    psoci_prec prec, double *dG1, double *dG2);

/* Natural orbitals and occupations of one packed 1-particle density (the MO-basis part of
 * PsociNOpopulations::constructNaturalOrbitals, PsociNOpopulations.C:569-669: per symmetry
 * block diagonalizeNOinMObasis :456-497 with a unit metric, then sortNOinMObasis :269-344,
 * largest occupation first).  orb_sym[nbf]: a symmetry label per orbital; a block holds the
 * orbitals of one label in ascending order, blocks in ascending label order (the reference's
 * nstart/nsize split when MOs are ordered by symmetry).  Outputs, blocks concatenated:
 * occ[nbf] occupations; vecs[sum of n_b^2] per block n_b x n_b, natural orbital i's
 * coefficients over the block's orbitals contiguous; orb_order[nbf] (may be NULL) the
 * orbitals of the blocks in output order.  Host computation; needs no context or device. */
PSOCI_API psoci_status psoci_natural_orbitals(int nbf, const double *dens, const int32_t *orb_sym, double *occ,
                                              double *vecs, int32_t *orb_order);

/* CI vector files in the reference's PsociVector "scalable" layout (PsociVector.C:530-706,
 * written by PsociGAvectors::dumpVectorScalable, PsociGAvectors.C:207-326).  binary = 0:
 * ASCII (header "nbasis nroots" / "width prec", per root its 1-based number then nbasis
 * values fixed with 14 decimals in 18 columns, title trailer); binary = 1: int64 header,
 * per root an int64 tag and nbasis doubles, title bytes.  vecs is root-major. */
PSOCI_API psoci_status psoci_write_vectors(const char *path, int binary, int64_t nbasis, int nroots,
                                           const double *vecs, const char *title);
/* Reads up to max_roots vectors of length nbasis (readVectorScalable, PsociGAvectors.C:539-658);
 * PSOCI_ERR_IO on a missing, truncated or mismatched file. */
PSOCI_API psoci_status psoci_read_vectors(const char *path, int binary, int64_t nbasis, int max_roots,
                                          double *vecs, int *nroots_read);

/* Hamiltonian checkpoint, replacing SendHamiltonianToDRA / FetchHamiltonianFromDRA
 * (PsociConstructHamiltonian.C:461-696) with one file in this library's own format (CSR,
 * diagonal, optional FP32 copy, a hash of the configuration space and a payload checksum).
 * Loading needs psoci_build_determinants on the same configurations; a file from other
 * configurations, a truncated file or a checksum mismatch gives PSOCI_ERR_IO. */
PSOCI_API psoci_status psoci_save_hamiltonian(const psoci_ctx *ctx, const char *path);
PSOCI_API psoci_status psoci_load_hamiltonian(psoci_ctx *ctx, const char *path);

/* The cudaStream_t (as void*) that every kernel of this context is launched on, for callers
 * that time or order work around the library's calls.  No reference counterpart. */
PSOCI_API void *psoci_stream(const psoci_ctx *ctx);

/* Number of kernels this library has launched in this process, over all contexts, so that
 * a caller can count the launches a call makes (difference of two readings).  No reference
 * counterpart. */
PSOCI_API unsigned long long psoci_launch_count(void);

/* Core energy passed to psoci_set_integrals (PsociIntegrals::fetchCoreEnergy). */
PSOCI_API double psoci_core_energy(const psoci_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* PSOCI_GPU_H */
