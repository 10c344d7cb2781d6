// Internal declarations shared by the translation units of libpsoci_gpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/psoci_gpu.h"

#define PSOCI_MAX_OPEN 11     // reference limit (PsociDeterminants.hpp:95-101)
#define PSOCI_MAX_WORDS 2     // nbf <= 128
#define PSOCI_SEG 32          // neighbours per warp segment in the H build
#define PSOCI_MIN_VALUE 1.0e-8  // packSefsef threshold (PsociHamiltonian.hpp:37)
// mixed-sigma kernel variants (sigma.cu) and the one used until psoci_autotune_sigma runs:
// a warp per row, 4 gathers in flight per lane (variant 1, 2 in flight, measured within 1%)
#define PSOCI_SIGMA_VARIANTS 6
#define PSOCI_SIGMA_DEFAULT 0

// ------------------------------------------------------------------------------------
// host-side context
// ------------------------------------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct psoci_ctx {
  int device = 0;
  int verbose = 0;
  int eval_launches = 0;  // 0: automatic; 1: the element evaluation in one launch
  cudaStream_t stream = nullptr;
  std::string err;
  // released device blocks kept for reuse (size -> pointer), see psoci_alloc
  std::multimap<size_t, void *> pool;
  size_t pool_bytes = 0, pool_cap = 0;

  // integrals
  int nbf = 0;
  double ecore = 0.0;
  double *d_one = nullptr;  // packed 1-e (SO folded), nbf(nbf+1)/2
  double *d_eri = nullptr;  // canonical packed 2-e
  int64_t n1 = 0, n2 = 0;
  bool have_ints = false;

  // configurations
  int nelec = 0, ksym = 0, mx_open = 0, nconf = 0, words = 1;
  bool have_cfgs = false;
  std::vector<int32_t> h_jsym;
  std::vector<uint8_t> h_occ;
  uint64_t *d_e1 = nullptr;   // [nconf*words] bit p: occ_p >= 1
  uint64_t *d_e2 = nullptr;   // [nconf*words] bit p: occ_p == 2
  int32_t *d_jsym = nullptr;  // [nconf]
  int32_t *d_nopen = nullptr; // [nconf]

  // neighbour screen by lookup ("split join"): usable when every configuration holds at
  // most two electrons in the orbitals >= join_s (MRCI-type spaces); built by set_configs
  bool join_ok = false;
  int join_s = 0, join_nh = 0, join_G = 0, join_L = 0;
  int32_t *d_jgid = nullptr;    // [nconf] pattern id of the orbitals >= s
  int32_t *d_jlid = nullptr;    // [nconf] pattern id of the orbitals < s
  int32_t *d_jT = nullptr;      // [L*G] configuration of (lo pattern, hi pattern), or -1
  int32_t *d_jlnoff = nullptr;  // [4*(5L+1)] per distance tau = 1..4, lo pattern, electron difference -2..2: offsets into d_jln
  int32_t *d_jln = nullptr;     // lo patterns within tau of each lo pattern, ascending
  int32_t *d_jhdec = nullptr;   // [G] hi pattern: kind | a << 8 | b << 20
  uint32_t *d_jlokey = nullptr; // [L] lo pattern: e1 bits | e2 bits << s

  // determinants
  bool have_dets = false;
  std::vector<int64_t> h_sefoff, h_detoff;  // nconf+1
  int64_t nsef_total = 0, ndet_total = 0;
  int max_nsef = 0, max_ndet = 0;
  int64_t *d_sefoff = nullptr, *d_detoff = nullptr;
  uint64_t *d_alpha = nullptr, *d_beta = nullptr;  // [ndet*words]
  uint8_t *d_phase = nullptr;                      // [ndet]
  uint8_t *d_nalpha = nullptr;                     // [ndet]
  int32_t *d_ms = nullptr;                         // [ndet]
  // template table: per (class, nopen) a run of (amask, bmask, msoff)
  uint32_t *d_tmpl = nullptr;   // packed: amask | bmask<<12 ; ms offset stored separately
  int32_t *d_tmpl_ms = nullptr;
  int32_t *d_tmpl_off = nullptr;  // [4*12+1] start of each (class, nopen) run

  // Hamiltonian
  bool have_h = false;
  int64_t nnz = 0;
  int64_t npairs = 0, nseg = 0, ncand = 0;
  int64_t *d_rowptr = nullptr;
  int32_t *d_col = nullptr;
  double *d_val = nullptr;
  float *d_val32 = nullptr;
  double *d_diag = nullptr;
  double build_seconds = 0.0;
  psoci_build_info binfo{};
  // direct mode (no stored elements): the screened neighbour lists and their segments
  bool direct = false;
  int64_t *dir_nbroff = nullptr;  // [nconf+1]
  int32_t *dir_nbr = nullptr;     // [npairs]
  int32_t *dir_segcfg = nullptr, *dir_segn = nullptr;
  int64_t *dir_segk0 = nullptr;
  int64_t slab_hint = 0;  // value-slab slots the last build of this space used
  int64_t join_hint = 0;  // join-slab slots the last build of this space used

  // 1-particle density: configuration groups sharing a hole key (density.cu)
  bool den_ready = false;
  int64_t den_ng = 0, den_npairs = 0;
  int64_t *den_geoff = nullptr;  // [ng+1] first member of each group
  int64_t *den_gpoff = nullptr;  // [ng+1] first candidate pair of each group
  int32_t *den_gcfg = nullptr;   // members: configuration
  uint8_t *den_gorb = nullptr;   // members: orbital the key removed
  int4 *den_gmem = nullptr;      // members packed with their configuration's offsets
  uint8_t *den_gflag = nullptr;  // [ng] 1: members' exact keys differ (hash collision)
  uint64_t *den_gopen = nullptr; // members: open shells of the configuration [words]
  float2 *den_vs = nullptr;      // float-float copy of the roots of one pass
  size_t den_vs_cap = 0;

  // mixed-sigma variant in use (sigma.cu; psoci_autotune_sigma picks it, a build resets it)
  int sigma_variant = PSOCI_SIGMA_DEFAULT;
  bool sigma_tuned = false;

  // neighbour lists of the energy gradient (hbuild.cu): every pair within two excitations
  // (grad_mode 0) or those with a non-zero integral prefactor (1)
  int64_t *grad_nbroff = nullptr;
  int32_t *grad_nbr = nullptr;
  int grad_mode = -1;
  int64_t grad_npairs = 0;

  // step-level Davidson basis (psoci_basis_*, davidson.cu)
  struct psoci_dav_basis *basis = nullptr;

  // initial guess for the next Davidson run (root-major, guess_k x nsef)
  std::vector<double> guess;
  int guess_k = 0;

  // scratch for host-pointer sigma
  double *d_x = nullptr, *d_y = nullptr;
  size_t xy_cap = 0;
  float *d_x32 = nullptr;
  size_t x32_cap = 0;
};

// host loops over configurations: f(lo, hi, t) on contiguous ranges of [0, n), one thread
// per host core (ranges of at least 16384), t = 0..threads-1; returns the thread count
template <class F>
int psoci_parallel_ranges(int64_t n, F &&f, int64_t grain = 16384) {
  int nt = (int)std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  nt = (int)std::min<int64_t>(nt, std::max<int64_t>(1, n / std::max<int64_t>(grain, 1)));
  if (nt <= 1) {
    f((int64_t)0, n, 0);
    return 1;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; ++t) th.emplace_back([&f, n, nt, t]() { f(n * t / nt, n * (t + 1) / nt, t); });
  for (auto &x : th) x.join();
  return nt;
}

// error helpers -----------------------------------------------------------------------
psoci_status psoci_fail(psoci_ctx *c, psoci_status s, const std::string &msg);
psoci_status psoci_cuda_fail(psoci_ctx *c, cudaError_t e, const char *where);
#define PSOCI_CUDA(c, call)                                            \
  do {                                                                 \
    cudaError_t _e = (call);                                           \
    if (_e != cudaSuccess) return psoci_cuda_fail((c), _e, #call);     \
  } while (0)

// Device memory of a context goes through a cache (util.cu): a released block is kept for
// a later allocation of the same context of at most 25% smaller size, so a repeated build
// or solve reuses its buffers instead of paying cudaFree (which waits for the device) and
// cudaMalloc (page mapping) for tens of GB each time.  Reuse waits for the context's stream
// first, as cudaFree would have.  The caches of all contexts on one device hold at most
// half its memory together; all of them are emptied when a cudaMalloc on that device fails
// (and the allocation is retried), and a context's own on psoci_destroy.
void psoci_pool_register(psoci_ctx *c);
void *psoci_device_alloc(psoci_ctx *c, size_t bytes, cudaError_t *err);
void psoci_device_free(void *p);
void psoci_pool_flush(psoci_ctx *c);
void psoci_pool_forget(psoci_ctx *c);

template <typename T>
psoci_status psoci_alloc(psoci_ctx *c, T **p, size_t count) {
  if (*p) { psoci_device_free((void *)*p); *p = nullptr; }
  if (count == 0) count = 1;
  cudaError_t e = cudaSuccess;
  *p = (T *)psoci_device_alloc(c, count * sizeof(T), &e);
  if (!*p) {
    cudaGetLastError();
    return psoci_fail(c, e == cudaErrorMemoryAllocation ? PSOCI_ERR_NOMEM : PSOCI_ERR_CUDA,
                      std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return PSOCI_OK;
}
template <typename T>
void psoci_free(T *&p) {
  psoci_device_free((void *)p);
  p = nullptr;
}

// device-wide exclusive scan of int64 counts (in place allowed); returns total on host
// counts one kernel launch (read back through psoci_launch_count)
void psoci_note_launch();
psoci_status psoci_scan_i64(psoci_ctx *c, const int64_t *d_in, int64_t *d_out, int64_t n, int64_t *total);

// sigma (sigma.cu) — device pointers, row-major N x k with leading dims
psoci_status psoci_sigma_launch(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy,
                                psoci_prec prec, float *dX32);

psoci_status psoci_sigma_autotune_run(psoci_ctx *c, int k, int *choice, float *times_ms);

// determinant templates (dets.cu)
psoci_status psoci_dets_build(psoci_ctx *c);
psoci_status psoci_h_build(psoci_ctx *c, psoci_hmode mode, int64_t *nnz);
psoci_status psoci_h_blocks(psoci_ctx *c, int npairs, const int32_t *A, const int32_t *B, double *out);
// sigma of a direct-mode build: every element evaluated again (hbuild.cu)
psoci_status psoci_direct_sigma(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy, psoci_prec prec,
                                float *x32);
psoci_status psoci_join_prepare(psoci_ctx *c);  // after h_occ is set
void psoci_join_release(psoci_ctx *c);
void psoci_h_release(psoci_ctx *c);
void psoci_dets_release(psoci_ctx *c);
void psoci_density_release(psoci_ctx *c);
void psoci_basis_release(psoci_ctx *c);
void psoci_grad_release(psoci_ctx *c);
// energy gradient with respect to the integral tables (hbuild.cu): device vectors k x ldv
// root-major, gradients k x n1 and k x n2
psoci_status psoci_energy_grad_run(psoci_ctx *c, int k, const double *dV, int64_t ldv, int mode, psoci_prec prec,
                                   double *dG1, double *dG2);

// ------------------------------------------------------------------------------------
// device helpers
// ------------------------------------------------------------------------------------
// determinant template classes (generateDeterminants, PsociDeterminants.C:1467-1505)
enum { CLS_EVEN = 0, CLS_ODD = 1, CLS_FRAC_P = 2, CLS_FRAC_M = 3, PSOCI_NCLS = 4 };
#define PSOCI_NOPEN_SLOTS (PSOCI_MAX_OPEN + 1)
__host__ __device__ __forceinline__ int psoci_det_class(int parity, int jsym, int ksym) {
  if (parity == 1) return ((((jsym + 1) / 2) % 2) == 0) ? CLS_FRAC_M : CLS_FRAC_P;
  return ((jsym + 1) / 2 == (ksym + 1) / 2) ? CLS_EVEN : CLS_ODD;
}

__device__ __forceinline__ int64_t tri64(int64_t i, int64_t j) {
  int64_t a = i > j ? i : j, b = i > j ? j : i;
  return a * (a + 1) / 2 + b;
}
// canonical 8-fold index (PsociIntegrals.C:889-898), 0-based
__device__ __forceinline__ int64_t canon4(int i, int j, int k, int l) {
  return tri64(tri64(i, j), tri64(k, l));
}
