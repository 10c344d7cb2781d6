// C ABI of libpsoci_gpu.so (declared in include/psoci_gpu.h).
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "psoci_internal.cuh"

psoci_status psoci_davidson_impl(psoci_ctx *c, const psoci_dav_opts *o, double *evals, double *evecs, double *rnorms,
                                 psoci_dav_stats *stats);

namespace {
psoci_status set_device(psoci_ctx *c) {
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  return PSOCI_OK;
}
void release_all(psoci_ctx *c) {
  psoci_basis_release(c);
  psoci_h_release(c);
  psoci_dets_release(c);
  psoci_join_release(c);
  psoci_density_release(c);
  psoci_free(c->d_one);
  psoci_free(c->d_eri);
  psoci_free(c->d_e1);
  psoci_free(c->d_e2);
  psoci_free(c->d_jsym);
  psoci_free(c->d_nopen);
  psoci_free(c->d_x);
  psoci_free(c->d_y);
  psoci_free(c->d_x32);
}
// psoci_get_rows: lengths of the requested rows, then their columns and values, one warp
// per row
__global__ void k_row_lengths(int n, const int64_t *__restrict__ rows, const int64_t *__restrict__ rowptr,
                              int64_t *__restrict__ len) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) len[q] = rowptr[rows[q] + 1] - rowptr[rows[q]];
}
__global__ void k_row_gather(int n, const int64_t *__restrict__ rows, const int64_t *__restrict__ rowptr,
                             const int64_t *__restrict__ outoff, const int32_t *__restrict__ col,
                             const double *__restrict__ val, int32_t *__restrict__ ocol, double *__restrict__ oval) {
  const int q = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (q >= n) return;
  const int64_t a = rowptr[rows[q]], m = rowptr[rows[q] + 1] - a, o = outoff[q];
  for (int64_t e = lane; e < m; e += 32) {
    ocol[o + e] = col[a + e];
    oval[o + e] = val[a + e];
  }
}
}  // namespace

extern "C" {

const char *psoci_status_str(psoci_status s) {
  switch (s) {
    case PSOCI_OK: return "ok";
    case PSOCI_ERR_INVALID_ARG: return "invalid argument";
    case PSOCI_ERR_UNSUPPORTED: return "unsupported";
    case PSOCI_ERR_STATE: return "call order";
    case PSOCI_ERR_CUDA: return "cuda error";
    case PSOCI_ERR_NOMEM: return "out of device memory";
    case PSOCI_ERR_TIMEOUT: return "device wait timed out";
    case PSOCI_ERR_NOT_CONVERGED: return "not converged";
    case PSOCI_ERR_NUMERIC: return "non-finite value";
    case PSOCI_ERR_IO: return "i/o error";
  }
  return "unknown status";
}

const char *psoci_last_error(const psoci_ctx *c) { return c ? c->err.c_str() : "null context"; }

psoci_status psoci_create(psoci_ctx **out, const psoci_opts *opts) {
  if (!out) return PSOCI_ERR_INVALID_ARG;
  *out = nullptr;
  psoci_ctx *c = new psoci_ctx();
  c->device = opts ? opts->device : 0;
  c->verbose = opts ? opts->verbose : 0;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    delete c;
    return PSOCI_ERR_CUDA;
  }
  if (c->device < 0 || c->device >= ndev) {
    delete c;
    return PSOCI_ERR_INVALID_ARG;
  }
  if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return PSOCI_ERR_CUDA;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) c->pool_cap = total_b / 2;
  cudaGetLastError();
  psoci_pool_register(c);
  *out = c;
  return PSOCI_OK;
}

void psoci_destroy(psoci_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  release_all(c);
  psoci_pool_flush(c);
  psoci_pool_forget(c);
  c->pool_cap = 0;
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

double psoci_core_energy(const psoci_ctx *c) { return c ? c->ecore : 0.0; }

psoci_status psoci_build_stats(const psoci_ctx *c, psoci_build_info *info) {
  if (!c || !info) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(const_cast<psoci_ctx *>(c), PSOCI_ERR_STATE, "build_stats: no Hamiltonian built");
  *info = c->binfo;
  return PSOCI_OK;
}

void *psoci_stream(const psoci_ctx *c) { return c ? (void *)c->stream : nullptr; }

psoci_status psoci_set_integrals(psoci_ctx *c, int nbf, const double *one, const double *eri, double ecore) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (nbf < 1 || !one || !eri) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "set_integrals: bad arguments");
  if (nbf > 64 * PSOCI_MAX_WORDS) return psoci_fail(c, PSOCI_ERR_UNSUPPORTED, "set_integrals: nbf > 128");
  if (c->have_cfgs && c->nbf != nbf) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "set_integrals: nbf differs from configurations");
  psoci_status s;
  if ((s = set_device(c))) return s;
  psoci_h_release(c);
  int64_t n1 = (int64_t)nbf * (nbf + 1) / 2, n2 = n1 * (n1 + 1) / 2;
  if ((s = psoci_alloc(c, &c->d_one, n1)) || (s = psoci_alloc(c, &c->d_eri, n2))) return s;
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_one, one, sizeof(double) * n1, cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_eri, eri, sizeof(double) * n2, cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  c->nbf = nbf;
  c->n1 = n1;
  c->n2 = n2;
  c->ecore = ecore;
  c->have_ints = true;
  return PSOCI_OK;
}

psoci_status psoci_set_configs(psoci_ctx *c, int nbf, int nelec, int ksym, int mx_open, int nconf, const int32_t *jsym,
                               const uint8_t *occ) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (nbf < 1 || nelec < 1 || nconf < 1 || !jsym || !occ || ksym < 1 || mx_open < 0)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "set_configs: bad arguments");
  if (nbf > 64 * PSOCI_MAX_WORDS) return psoci_fail(c, PSOCI_ERR_UNSUPPORTED, "set_configs: nbf > 128");
  if (c->have_ints && c->nbf != nbf) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "set_configs: nbf differs from integrals");
  const int W = (nbf + 63) / 64;
  std::vector<uint64_t> e1((size_t)nconf * W, 0), e2((size_t)nconf * W, 0);
  std::vector<int32_t> nopen(nconf);
  // bit-planes and checks on the host's cores; each range keeps its first failing
  // configuration, and the lowest one is reported, with the serial loop's message
  struct Bad {
    int i = -1;
    psoci_status st = PSOCI_OK;
    std::string msg;
  };
  std::vector<Bad> bad(std::max<unsigned>(1u, std::thread::hardware_concurrency()));
  const int nthr = psoci_parallel_ranges(nconf, [&](int64_t lo, int64_t hi, int t) {
    for (int64_t ii = lo; ii < hi; ++ii) {
      const int i = (int)ii;
      const uint8_t *o = occ + (size_t)i * nbf;
      int ne = 0, no = 0;
      char b[128];
      for (int p = 0; p < nbf; ++p) {
        if (o[p] > 2) {
          snprintf(b, sizeof(b), "set_configs: configuration %d orbital %d occupation %d", i, p, (int)o[p]);
          bad[t] = {i, PSOCI_ERR_INVALID_ARG, b};
          return;
        }
        ne += o[p];
        no += (o[p] == 1);
        if (o[p] >= 1) e1[(size_t)i * W + p / 64] |= 1ull << (p % 64);
        if (o[p] == 2) e2[(size_t)i * W + p / 64] |= 1ull << (p % 64);
      }
      if (ne != nelec) {
        snprintf(b, sizeof(b), "set_configs: configuration %d holds %d electrons, expected %d", i, ne, nelec);
        bad[t] = {i, PSOCI_ERR_INVALID_ARG, b};
        return;
      }
      if (no > PSOCI_MAX_OPEN) { bad[t] = {i, PSOCI_ERR_UNSUPPORTED, "set_configs: more than 11 open shells"}; return; }
      if (jsym[i] < 1) { bad[t] = {i, PSOCI_ERR_INVALID_ARG, "set_configs: jsym labels are 1-based"}; return; }
      nopen[i] = no;
    }
  });
  for (int t = 0; t < nthr; ++t)
    if (bad[t].i >= 0) return psoci_fail(c, bad[t].st, bad[t].msg);  // ranges ascend: the first is the lowest
  psoci_status s;
  if ((s = set_device(c))) return s;
  psoci_h_release(c);
  psoci_dets_release(c);
  psoci_density_release(c);
  if ((s = psoci_alloc(c, &c->d_e1, e1.size())) || (s = psoci_alloc(c, &c->d_e2, e2.size())) ||
      (s = psoci_alloc(c, &c->d_jsym, nconf)) || (s = psoci_alloc(c, &c->d_nopen, nconf)))
    return s;
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_e1, e1.data(), sizeof(uint64_t) * e1.size(), cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_e2, e2.data(), sizeof(uint64_t) * e2.size(), cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jsym, jsym, sizeof(int32_t) * nconf, cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_nopen, nopen.data(), sizeof(int32_t) * nconf, cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  c->nbf = nbf;
  c->nelec = nelec;
  c->ksym = ksym;
  c->mx_open = mx_open;
  c->nconf = nconf;
  c->words = W;
  c->h_jsym.assign(jsym, jsym + nconf);
  // host copy of the occupations, in parallel (a repeated call with the same size reuses
  // the buffer: no fill)
  if (c->h_occ.size() != (size_t)nconf * nbf) c->h_occ.assign((size_t)nconf * nbf, 0);
  psoci_parallel_ranges(nconf, [&](int64_t lo, int64_t hi, int) {
    memcpy(c->h_occ.data() + (size_t)lo * nbf, occ + (size_t)lo * nbf, (size_t)(hi - lo) * nbf);
  });
  c->slab_hint = 0;
  c->join_hint = 0;
  c->have_cfgs = true;
  return psoci_join_prepare(c);
}

psoci_status psoci_build_determinants(psoci_ctx *c) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  psoci_status s;
  if ((s = set_device(c))) return s;
  return psoci_dets_build(c);
}

psoci_status psoci_get_counts(const psoci_ctx *c, int64_t *nsef, int64_t *ndet, int *max_nsef, int *max_ndet) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_dets) return PSOCI_ERR_STATE;
  if (nsef) *nsef = c->nsef_total;
  if (ndet) *ndet = c->ndet_total;
  if (max_nsef) *max_nsef = c->max_nsef;
  if (max_ndet) *max_ndet = c->max_ndet;
  return PSOCI_OK;
}

psoci_status psoci_get_determinants(const psoci_ctx *cc, uint64_t *alpha, uint64_t *beta, uint8_t *phase, int32_t *ms,
                                    int64_t *detoff, int64_t *sefoff) {
  psoci_ctx *c = const_cast<psoci_ctx *>(cc);
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "get_determinants: not built");
  psoci_status s;
  if ((s = set_device(c))) return s;
  size_t nd = (size_t)c->ndet_total;
  if (alpha) PSOCI_CUDA(c, cudaMemcpy(alpha, c->d_alpha, sizeof(uint64_t) * nd * c->words, cudaMemcpyDeviceToHost));
  if (beta) PSOCI_CUDA(c, cudaMemcpy(beta, c->d_beta, sizeof(uint64_t) * nd * c->words, cudaMemcpyDeviceToHost));
  if (phase) PSOCI_CUDA(c, cudaMemcpy(phase, c->d_phase, nd, cudaMemcpyDeviceToHost));
  if (ms) PSOCI_CUDA(c, cudaMemcpy(ms, c->d_ms, sizeof(int32_t) * nd, cudaMemcpyDeviceToHost));
  if (detoff) memcpy(detoff, c->h_detoff.data(), sizeof(int64_t) * (c->nconf + 1));
  if (sefoff) memcpy(sefoff, c->h_sefoff.data(), sizeof(int64_t) * (c->nconf + 1));
  return PSOCI_OK;
}

psoci_status psoci_build_hamiltonian(psoci_ctx *c, psoci_hmode mode, int64_t *nnz) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (mode != PSOCI_HMODE_CSR_FP64 && mode != PSOCI_HMODE_CSR_BOTH && mode != PSOCI_HMODE_DIRECT)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "build_hamiltonian: unknown mode");
  psoci_status s;
  if ((s = set_device(c))) return s;
  int64_t n = 0;
  s = psoci_h_build(c, mode, &n);
  if (nnz) *nnz = (s == PSOCI_OK) ? n : 0;
  return s;
}

psoci_status psoci_blocks(psoci_ctx *c, int npairs, const int32_t *A, const int32_t *B, double *out) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  psoci_status s;
  if ((s = set_device(c))) return s;
  return psoci_h_blocks(c, npairs, A, B, out);
}

psoci_status psoci_get_hamiltonian(const psoci_ctx *cc, int64_t *rowptr, int32_t *cols, double *vals) {
  psoci_ctx *c = const_cast<psoci_ctx *>(cc);
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "get_hamiltonian: not built");
  if (c->direct) return psoci_fail(c, PSOCI_ERR_STATE, "get_hamiltonian: direct mode stores no matrix");
  psoci_status s;
  if ((s = set_device(c))) return s;
  if (rowptr)
    PSOCI_CUDA(c, cudaMemcpy(rowptr, c->d_rowptr, sizeof(int64_t) * (c->nsef_total + 1), cudaMemcpyDeviceToHost));
  if (cols) PSOCI_CUDA(c, cudaMemcpy(cols, c->d_col, sizeof(int32_t) * c->nnz, cudaMemcpyDeviceToHost));
  if (vals) PSOCI_CUDA(c, cudaMemcpy(vals, c->d_val, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost));
  return PSOCI_OK;
}

psoci_status psoci_get_rows(const psoci_ctx *cc, int nrows, const int64_t *rows, int64_t *rowptr, int32_t *cols,
                            double *vals) {
  psoci_ctx *c = const_cast<psoci_ctx *>(cc);
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (nrows < 0 || (nrows > 0 && (!rows || !rowptr)) || (!cols) != (!vals))
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "get_rows: bad arguments");
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "get_rows: not built");
  if (c->direct) return psoci_fail(c, PSOCI_ERR_STATE, "get_rows: direct mode stores no matrix");
  for (int q = 0; q < nrows; ++q)
    if (rows[q] < 0 || rows[q] >= c->nsef_total) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "get_rows: row out of range");
  if (rowptr) rowptr[0] = 0;
  if (nrows == 0) return PSOCI_OK;
  psoci_status s;
  if ((s = set_device(c))) return s;
  cudaStream_t st = c->stream;
  int64_t *d_rows = nullptr, *d_len = nullptr, *d_off = nullptr;
  int32_t *d_col = nullptr;
  double *d_val = nullptr;
  auto done = [&](psoci_status r) {
    psoci_free(d_rows); psoci_free(d_len); psoci_free(d_off); psoci_free(d_col); psoci_free(d_val);
    return r;
  };
  if ((s = psoci_alloc(c, &d_rows, nrows)) || (s = psoci_alloc(c, &d_len, nrows)) || (s = psoci_alloc(c, &d_off, nrows + 1)))
    return done(s);
  std::vector<int64_t> len(nrows);
  cudaError_t e = cudaMemcpyAsync(d_rows, rows, sizeof(int64_t) * nrows, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    psoci_note_launch();
    k_row_lengths<<<(nrows + 255) / 256, 256, 0, st>>>(nrows, d_rows, c->d_rowptr, d_len);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(len.data(), d_len, sizeof(int64_t) * nrows, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "get_rows"));
  for (int q = 0; q < nrows; ++q) rowptr[q + 1] = rowptr[q] + len[q];
  const int64_t tot = rowptr[nrows];
  if (!cols || tot == 0) return done(PSOCI_OK);
  if ((s = psoci_alloc(c, &d_col, tot)) || (s = psoci_alloc(c, &d_val, tot))) return done(s);
  e = cudaMemcpyAsync(d_off, rowptr, sizeof(int64_t) * (nrows + 1), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    psoci_note_launch();
    k_row_gather<<<(unsigned)(((int64_t)nrows * 32 + 255) / 256), 256, 0, st>>>(nrows, d_rows, c->d_rowptr, d_off,
                                                                                 c->d_col, c->d_val, d_col, d_val);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(cols, d_col, sizeof(int32_t) * tot, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(vals, d_val, sizeof(double) * tot, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "get_rows"));
  return done(PSOCI_OK);
}

psoci_status psoci_energy_gradient_device(psoci_ctx *c, int k, const double *dV, int64_t ldv, int mode,
                                          psoci_prec prec, double *dG1, double *dG2) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  psoci_status s;
  if ((s = set_device(c))) return s;
  return psoci_energy_grad_run(c, k, dV, ldv, mode, prec, dG1, dG2);
}

psoci_status psoci_energy_gradient(psoci_ctx *c, int k, const double *vecs, int mode, psoci_prec prec,
                                   double *grad_one, double *grad_eri) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (k < 1 || !vecs || !grad_one || !grad_eri)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "energy_gradient: bad arguments");
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "energy_gradient: determinants not built");
  psoci_status s;
  if ((s = set_device(c))) return s;
  const int64_t N = c->nsef_total, n1 = c->n1, n2 = c->n2;
  double *dV = nullptr, *dG1 = nullptr, *dG2 = nullptr;
  auto done = [&](psoci_status r) {
    psoci_free(dV); psoci_free(dG1); psoci_free(dG2);
    return r;
  };
  if ((s = psoci_alloc(c, &dV, (size_t)k * N)) || (s = psoci_alloc(c, &dG1, (size_t)k * n1)) ||
      (s = psoci_alloc(c, &dG2, (size_t)k * n2)))
    return done(s);
  cudaError_t e = cudaMemcpyAsync(dV, vecs, sizeof(double) * k * N, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "energy_gradient"));
  if ((s = psoci_energy_grad_run(c, k, dV, N, mode, prec, dG1, dG2))) return done(s);
  e = cudaMemcpyAsync(grad_one, dG1, sizeof(double) * k * n1, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(grad_eri, dG2, sizeof(double) * k * n2, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "energy_gradient"));
  return done(PSOCI_OK);
}

psoci_status psoci_get_diag(const psoci_ctx *cc, double *diag) {
  psoci_ctx *c = const_cast<psoci_ctx *>(cc);
  if (!c || !diag) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "get_diag: not built");
  psoci_status s;
  if ((s = set_device(c))) return s;
  PSOCI_CUDA(c, cudaMemcpy(diag, c->d_diag, sizeof(double) * c->nsef_total, cudaMemcpyDeviceToHost));
  return PSOCI_OK;
}

psoci_status psoci_sigma_device(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy, psoci_prec prec) {
  if (!c || !dX || !dY) return PSOCI_ERR_INVALID_ARG;
  psoci_status s;
  if ((s = set_device(c))) return s;
  if (prec == PSOCI_PREC_MIXED || prec == PSOCI_PREC_FF) {
    size_t need = (size_t)c->nsef_total * (prec == PSOCI_PREC_FF ? 16 : 8);
    if (c->x32_cap < need) {
      if ((s = psoci_alloc(c, &c->d_x32, need))) return s;
      c->x32_cap = need;
    }
  }
  return psoci_sigma_launch(c, k, dX, ldx, dY, ldy, prec, c->d_x32);
}

psoci_status psoci_sigma(psoci_ctx *c, int k, const double *X, double *Y, psoci_prec prec) {
  if (!c || !X || !Y || k < 1) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "sigma: Hamiltonian not built");
  psoci_status s;
  if ((s = set_device(c))) return s;
  size_t need = (size_t)c->nsef_total * k;
  if (c->xy_cap < need) {
    if ((s = psoci_alloc(c, &c->d_x, need)) || (s = psoci_alloc(c, &c->d_y, need))) return s;
    c->xy_cap = need;
  }
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_x, X, sizeof(double) * need, cudaMemcpyHostToDevice, c->stream));
  if ((s = psoci_sigma_device(c, k, c->d_x, k, c->d_y, k, prec))) return s;
  PSOCI_CUDA(c, cudaMemcpyAsync(Y, c->d_y, sizeof(double) * need, cudaMemcpyDeviceToHost, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  return PSOCI_OK;
}

psoci_status psoci_set_guess(psoci_ctx *c, int k, const double *vecs) {
  if (!c || k < 0 || (k > 0 && !vecs)) return PSOCI_ERR_INVALID_ARG;
  if (k == 0) {
    c->guess.clear();
    c->guess_k = 0;
    return PSOCI_OK;
  }
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "set_guess: build the determinants first");
  c->guess.assign(vecs, vecs + (size_t)k * c->nsef_total);
  c->guess_k = k;
  return PSOCI_OK;
}

psoci_status psoci_davidson(psoci_ctx *c, const psoci_dav_opts *opts, double *evals, double *evecs, double *rnorms,
                            psoci_dav_stats *stats) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  psoci_status s;
  if ((s = set_device(c))) return s;
  return psoci_davidson_impl(c, opts, evals, evecs, rnorms, stats);
}

psoci_status psoci_set_eval_launches(psoci_ctx *c, int launches) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (launches != 0 && launches != 1)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "psoci_set_eval_launches: launches must be 0 or 1");
  c->eval_launches = launches;
  return PSOCI_OK;
}

psoci_status psoci_autotune_sigma(psoci_ctx *c, int k, int *choice, float *times_ms) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  psoci_status s;
  if ((s = set_device(c))) return s;
  return psoci_sigma_autotune_run(c, k, choice, times_ms);
}

psoci_status psoci_davidson_batch(psoci_ctx *const *ctxs, int nblocks, const psoci_dav_opts *opts,
                                  double *const *evals, double *const *evecs, double *const *rnorms,
                                  psoci_dav_stats *stats, psoci_status *block_status) {
  if (!ctxs || !opts || !evals || nblocks < 1) return PSOCI_ERR_INVALID_ARG;
  for (int b = 0; b < nblocks; ++b) {
    if (!ctxs[b] || !evals[b]) return PSOCI_ERR_INVALID_ARG;
    for (int a = 0; a < b; ++a)
      if (ctxs[a] == ctxs[b]) return psoci_fail(ctxs[b], PSOCI_ERR_INVALID_ARG, "davidson_batch: a context twice");
  }
  std::vector<psoci_status> st(nblocks, PSOCI_OK);
  auto run = [&](int b) {
    psoci_ctx *c = ctxs[b];
    psoci_status s = set_device(c);
    // the sigma variant for this block's Hamiltonian, chosen once per build
    if (s == PSOCI_OK && opts[b].prec == PSOCI_PREC_MIXED && c->have_h && !c->direct && c->d_val32 && !c->sigma_tuned) {
      s = psoci_sigma_autotune_run(c, std::min(8, std::max(1, opts[b].nroots)), nullptr, nullptr);
      if (s == PSOCI_OK) c->sigma_tuned = true;
    }
    if (s == PSOCI_OK)
      s = psoci_davidson_impl(c, &opts[b], evals[b], evecs ? evecs[b] : nullptr, rnorms ? rnorms[b] : nullptr,
                              stats ? &stats[b] : nullptr);
    st[b] = s;
  };
  std::vector<std::thread> th;
  for (int b = 1; b < nblocks; ++b) th.emplace_back(run, b);
  run(0);
  for (auto &t : th) t.join();
  psoci_status worst = PSOCI_OK;
  for (int b = 0; b < nblocks; ++b) {
    if (block_status) block_status[b] = st[b];
    if (st[b] != PSOCI_OK && worst == PSOCI_OK) worst = st[b];
  }
  return worst;
}

}  // extern "C"
