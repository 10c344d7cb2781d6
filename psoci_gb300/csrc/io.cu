// Host-side file formats: CI vector files (the reference's PsociVector "scalable" layout)
// and the Hamiltonian checkpoint (replacing the Disk Resident Array store).
//
// Vector files follow PsociVector.C:530-706 and PsociGAvectors.C:207-326:
//   ASCII (the production build's format; -DBINARY is off in Makefile:64):
//     "<nbasis> <nroots>\n<width> <prec>\n", then per root "<root number, 1-based>\n",
//     nbasis values each printed fixed with <prec> decimals in a field of <width>, "\n";
//     finally the title and "\n".  Defaults width 18, prec 14 (PsociVector.hpp:39-40).
//   BINARY: int64 nbasis, int64 nroots, int32 width, int32 prec; per root an int64 root
//     number and nbasis doubles; the title bytes.  The reference writes the root tag from an
//     int with sizeof(int64_t) (PsociVector.C:627-643), leaving the high half undefined;
//     here it is a proper int64.  Readers ignore the tag, as the reference's does.
//
// Hamiltonian checkpoint (own format; the reference stores H in DRA files, driver.PSOCI.hpp:58):
//   "PSOCIH01", int64 N, int64 nnz, int64 flags (bit 0: FP32 copy present),
//   uint64 FNV-1a hash of (nbf, nelec, ksym, occupations, jsym), uint64 hash of the payload,
//   rowptr[N+1] int64, cols[nnz] int32, vals[nnz] double, diag[N] double, [vals32[nnz] float].
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "psoci_internal.cuh"

namespace {

struct File {
  FILE *f = nullptr;
  File(const char *p, const char *m) { f = fopen(p, m); }
  ~File() {
    if (f) fclose(f);
  }
};

uint64_t fnv1a(const void *data, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char *p = (const unsigned char *)data;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t config_hash(const psoci_ctx *c) {
  int32_t hdr[3] = {c->nbf, c->nelec, c->ksym};
  uint64_t h = fnv1a(hdr, sizeof(hdr));
  h = fnv1a(c->h_occ.data(), c->h_occ.size(), h);
  h = fnv1a(c->h_jsym.data(), c->h_jsym.size() * sizeof(int32_t), h);
  return h;
}

const char kMagic[8] = {'P', 'S', 'O', 'C', 'I', 'H', '0', '1'};

}  // namespace

extern "C" {

psoci_status psoci_write_vectors(const char *path, int binary, int64_t nbasis, int nroots, const double *vecs,
                                 const char *title) {
  if (!path || nbasis < 1 || nroots < 1 || !vecs) return PSOCI_ERR_INVALID_ARG;
  const int width = 18, prec = 14;
  std::string t = title ? title : "";
  File fh(path, binary ? "wb" : "w");
  if (!fh.f) return PSOCI_ERR_IO;
  FILE *f = fh.f;
  if (binary) {
    int64_t h64[2] = {nbasis, nroots};
    int32_t h32[2] = {width, prec};
    if (fwrite(h64, sizeof(h64), 1, f) != 1 || fwrite(h32, sizeof(h32), 1, f) != 1) return PSOCI_ERR_IO;
    for (int r = 0; r < nroots; ++r) {
      int64_t tag = r + 1;
      if (fwrite(&tag, sizeof(tag), 1, f) != 1) return PSOCI_ERR_IO;
      if (fwrite(vecs + (size_t)r * nbasis, sizeof(double), (size_t)nbasis, f) != (size_t)nbasis) return PSOCI_ERR_IO;
    }
    if (!t.empty() && fwrite(t.data(), 1, t.size(), f) != t.size()) return PSOCI_ERR_IO;
  } else {
    if (fprintf(f, "%" PRId64 " %d\n%d %d\n", nbasis, nroots, width, prec) < 0) return PSOCI_ERR_IO;
    for (int r = 0; r < nroots; ++r) {
      if (fprintf(f, "%d\n", r + 1) < 0) return PSOCI_ERR_IO;
      for (int64_t i = 0; i < nbasis; ++i)
        if (fprintf(f, "%*.*f", width, prec, vecs[(size_t)r * nbasis + i]) < 0) return PSOCI_ERR_IO;
      if (fputc('\n', f) == EOF) return PSOCI_ERR_IO;
    }
    if (fprintf(f, "%s\n", t.c_str()) < 0) return PSOCI_ERR_IO;
  }
  return (fflush(f) == 0) ? PSOCI_OK : PSOCI_ERR_IO;
}

psoci_status psoci_read_vectors(const char *path, int binary, int64_t nbasis, int max_roots, double *vecs,
                                int *nroots_read) {
  if (!path || nbasis < 1 || max_roots < 1 || !vecs) return PSOCI_ERR_INVALID_ARG;
  File fh(path, binary ? "rb" : "r");
  if (!fh.f) return PSOCI_ERR_IO;
  FILE *f = fh.f;
  int64_t nb = 0, nr = 0;
  if (binary) {
    int64_t h64[2];
    int32_t h32[2];
    if (fread(h64, sizeof(h64), 1, f) != 1 || fread(h32, sizeof(h32), 1, f) != 1) return PSOCI_ERR_IO;
    nb = h64[0];
    nr = h64[1];
  } else {
    int w = 0, p = 0;
    if (fscanf(f, "%" SCNd64 " %" SCNd64 " %d %d", &nb, &nr, &w, &p) != 4) return PSOCI_ERR_IO;
  }
  if (nb != nbasis || nr < 1 || nr > (int64_t)1 << 30) return PSOCI_ERR_IO;
  int keep = (int)std::min<int64_t>(nr, max_roots);
  for (int r = 0; r < keep; ++r) {
    double *dst = vecs + (size_t)r * nbasis;
    if (binary) {
      int64_t tag;
      if (fread(&tag, sizeof(tag), 1, f) != 1) return PSOCI_ERR_IO;
      if (fread(dst, sizeof(double), (size_t)nbasis, f) != (size_t)nbasis) return PSOCI_ERR_IO;
    } else {
      int64_t tag;
      if (fscanf(f, "%" SCNd64, &tag) != 1) return PSOCI_ERR_IO;
      for (int64_t i = 0; i < nbasis; ++i)
        if (fscanf(f, "%lf", dst + i) != 1) return PSOCI_ERR_IO;
    }
    for (int64_t i = 0; i < nbasis; ++i)
      if (!std::isfinite(dst[i])) return PSOCI_ERR_IO;
  }
  if (nroots_read) *nroots_read = keep;
  return PSOCI_OK;
}

psoci_status psoci_save_hamiltonian(const psoci_ctx *cc, const char *path) {
  psoci_ctx *c = const_cast<psoci_ctx *>(cc);
  if (!c || !path) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "save_hamiltonian: not built");
  if (c->direct) return psoci_fail(c, PSOCI_ERR_STATE, "save_hamiltonian: direct mode stores no matrix");
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  const int64_t N = c->nsef_total, nnz = c->nnz;
  std::vector<int64_t> rp(N + 1);
  std::vector<int32_t> ci(nnz);
  std::vector<double> va(nnz), dg(N);
  std::vector<float> v32(c->d_val32 ? nnz : 0);
  PSOCI_CUDA(c, cudaMemcpy(rp.data(), c->d_rowptr, sizeof(int64_t) * (N + 1), cudaMemcpyDeviceToHost));
  PSOCI_CUDA(c, cudaMemcpy(ci.data(), c->d_col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost));
  PSOCI_CUDA(c, cudaMemcpy(va.data(), c->d_val, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
  PSOCI_CUDA(c, cudaMemcpy(dg.data(), c->d_diag, sizeof(double) * N, cudaMemcpyDeviceToHost));
  if (c->d_val32) PSOCI_CUDA(c, cudaMemcpy(v32.data(), c->d_val32, sizeof(float) * nnz, cudaMemcpyDeviceToHost));
  uint64_t ph = fnv1a(rp.data(), rp.size() * 8);
  ph = fnv1a(ci.data(), ci.size() * 4, ph);
  ph = fnv1a(va.data(), va.size() * 8, ph);
  ph = fnv1a(dg.data(), dg.size() * 8, ph);
  ph = fnv1a(v32.data(), v32.size() * 4, ph);
  File fh(path, "wb");
  if (!fh.f) return psoci_fail(c, PSOCI_ERR_IO, "save_hamiltonian: cannot open file");
  int64_t hdr[3] = {N, nnz, c->d_val32 ? 1 : 0};
  uint64_t hashes[2] = {config_hash(c), ph};
  bool ok = fwrite(kMagic, 8, 1, fh.f) == 1 && fwrite(hdr, sizeof(hdr), 1, fh.f) == 1 &&
            fwrite(hashes, sizeof(hashes), 1, fh.f) == 1 && fwrite(rp.data(), 8, rp.size(), fh.f) == rp.size() &&
            fwrite(ci.data(), 4, ci.size(), fh.f) == ci.size() && fwrite(va.data(), 8, va.size(), fh.f) == va.size() &&
            fwrite(dg.data(), 8, dg.size(), fh.f) == dg.size() &&
            (v32.empty() || fwrite(v32.data(), 4, v32.size(), fh.f) == v32.size());
  if (!ok || fflush(fh.f) != 0) return psoci_fail(c, PSOCI_ERR_IO, "save_hamiltonian: write failed");
  return PSOCI_OK;
}

psoci_status psoci_load_hamiltonian(psoci_ctx *c, const char *path) {
  if (!c || !path) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "load_hamiltonian: build the determinants first");
  File fh(path, "rb");
  if (!fh.f) return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: cannot open file");
  char magic[8];
  int64_t hdr[3];
  uint64_t hashes[2];
  if (fread(magic, 8, 1, fh.f) != 1 || memcmp(magic, kMagic, 8) != 0)
    return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: not a Hamiltonian checkpoint");
  if (fread(hdr, sizeof(hdr), 1, fh.f) != 1 || fread(hashes, sizeof(hashes), 1, fh.f) != 1)
    return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: truncated header");
  const int64_t N = hdr[0], nnz = hdr[1];
  const bool has32 = hdr[2] & 1;
  if (N != c->nsef_total || nnz < N || nnz > N * N)
    return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: dimension differs from the configuration space");
  if (hashes[0] != config_hash(c))
    return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: checkpoint belongs to other configurations");
  std::vector<int64_t> rp(N + 1);
  std::vector<int32_t> ci(nnz);
  std::vector<double> va(nnz), dg(N);
  std::vector<float> v32(has32 ? nnz : 0);
  bool ok = fread(rp.data(), 8, rp.size(), fh.f) == rp.size() && fread(ci.data(), 4, ci.size(), fh.f) == ci.size() &&
            fread(va.data(), 8, va.size(), fh.f) == va.size() && fread(dg.data(), 8, dg.size(), fh.f) == dg.size() &&
            (v32.empty() || fread(v32.data(), 4, v32.size(), fh.f) == v32.size());
  if (!ok) return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: truncated payload");
  uint64_t ph = fnv1a(rp.data(), rp.size() * 8);
  ph = fnv1a(ci.data(), ci.size() * 4, ph);
  ph = fnv1a(va.data(), va.size() * 8, ph);
  ph = fnv1a(dg.data(), dg.size() * 8, ph);
  ph = fnv1a(v32.data(), v32.size() * 4, ph);
  if (ph != hashes[1]) return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: payload checksum mismatch");
  // structural checks: monotone row pointers and in-range columns
  if (rp[0] != 0 || rp[N] != nnz) return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: bad row pointers");
  for (int64_t r = 0; r < N; ++r)
    if (rp[r + 1] < rp[r]) return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: bad row pointers");
  for (int64_t t = 0; t < nnz; ++t)
    if (ci[t] < 0 || ci[t] >= N) return psoci_fail(c, PSOCI_ERR_IO, "load_hamiltonian: column out of range");
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  psoci_h_release(c);
  psoci_status s;
  if ((s = psoci_alloc(c, &c->d_rowptr, N + 1)) || (s = psoci_alloc(c, &c->d_col, nnz)) ||
      (s = psoci_alloc(c, &c->d_val, nnz)) || (s = psoci_alloc(c, &c->d_diag, N)))
    return s;
  if (has32 && (s = psoci_alloc(c, &c->d_val32, nnz))) return s;
  PSOCI_CUDA(c, cudaMemcpy(c->d_rowptr, rp.data(), 8 * (N + 1), cudaMemcpyHostToDevice));
  PSOCI_CUDA(c, cudaMemcpy(c->d_col, ci.data(), 4 * nnz, cudaMemcpyHostToDevice));
  PSOCI_CUDA(c, cudaMemcpy(c->d_val, va.data(), 8 * nnz, cudaMemcpyHostToDevice));
  PSOCI_CUDA(c, cudaMemcpy(c->d_diag, dg.data(), 8 * N, cudaMemcpyHostToDevice));
  if (has32) PSOCI_CUDA(c, cudaMemcpy(c->d_val32, v32.data(), 4 * nnz, cudaMemcpyHostToDevice));
  c->nnz = nnz;
  c->binfo = psoci_build_info{};  // loaded, not built: counts only
  c->binfo.nnz = nnz;
  c->binfo.nnz_lower = (nnz + c->nsef_total) / 2;
  c->have_h = true;
  return PSOCI_OK;
}

}  // extern "C"
