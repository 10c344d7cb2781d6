/* Reference oracle harness — TEST INFRASTRUCTURE ONLY.
 *
 * Links the reference's own compute sources (PsociConfigs.C, PsociDeterminants.C,
 * PsociIntegrals.C, PsociHamiltonian.C, PsociTimer.C), compiled unchanged from the
 * reference tree against the single-process GA/MPI shim in oracle/ref_shim, and
 * exposes them through a small C API for ctypes.  It is built into oracle/_ref/ by
 * oracle/Makefile and is used only to pin the C restatement (oracle/psoci_oracle.c)
 * and to generate the golden fixtures under tests/golden/.  Nothing in the
 * psoci_gb300 package loads it.
 *
 * Integrals reach PsociIntegrals through stand-ins for the Columbus SIFS readers
 * (sifrh1_/sifrh2_/sifrd1_/sifrd2_), so the reference's own packing code
 * (PsociIntegrals.C:424-540 one-electron + spin-orbit sign convention,
 * :613-720 two-electron canonical packing) runs on the synthetic integrals.
 *
 * The H build follows the reference's production loop
 * (PsociGAhamiltonian.C:2530-2857: rows i, columns j <= i, generateSOCIblocks per
 * pair) and restates packSefsef (PsociGAhamiltonian.C:4077-4136: keep |x| >= 1e-8
 * or the diagonal, lower triangle inside the diagonal block) because the GA class
 * itself cannot be built without Global Arrays.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "PsociConfigs.hpp"
#include "PsociDeterminants.hpp"
#include "PsociHamiltonian.hpp"
#include "PsociIntegrals.hpp"
#include "PsociVector.hpp"

using namespace std;

/* ---------------- fake SIFS feeder ---------------- */
static int g_nbf = 0;
static vector<double> g_h;    /* nbf*nbf symmetric one-electron (same-irrep support) */
static vector<double> g_so;   /* nbf*nbf antisymmetric spin-orbit (cross-irrep support) */
static vector<double> g_eri;  /* canonical packed two-electron table */
static double g_ecore = 0.0;
static int g_rd1_calls = 0;

static inline long nndaf(long i) { return i * (i + 1) / 2; }

extern "C" {
void ftocxxopen_(Fint &, const char *, Fint &, Fint &istatus) { istatus = 0; }
void ftocxxclose_(Fint &) {}
void sifrh1_(Fint &, Fint &ntitle, Fint &nsym, Fint &nbft, Fint &ninfo, Fint &nenrgy, Fint &nmap,
             Fint &ierr) {
  ntitle = 1; nsym = 1; nbft = g_nbf; ninfo = 5; nenrgy = 1; nmap = 0; ierr = 0;
  g_rd1_calls = 0;
}
void sifrh2_(Fint &, Fint &ntitle, Fint &nsym, Fint &nbft, Fint &ninfo, Fint &nenrgy, Fint &,
             char *title, Fint *nbpsy, char *slabels, Fint *info, char *bfnlabs, Fint *ietype,
             Fdouble *energy, Fint *, Fint *, Fint &ierr) {
  memset(title, ' ', (size_t)ntitle * MAX_TITLE_LENGTH);
  memset(slabels, ' ', (size_t)nsym * MAX_LABEL_LENGTH);
  memset(bfnlabs, ' ', (size_t)nbft * MAX_BFNLAB_LENGTH);
  nbpsy[0] = nbft;
  info[0] = 1;                                 /* fsplit: combined file */
  info[1] = 1;                                 /* l1rec */
  info[2] = (Fint)nbft * nbft;                 /* n1max: everything in one record */
  info[3] = 1;                                 /* l2rec */
  info[4] = (Fint)nndaf(nndaf(nbft));          /* n2max */
  (void)ninfo;
  ietype[0] = -1;
  energy[0] = g_ecore;
  (void)nenrgy;
  ierr = 0;
}
/* call 1: one type-0 record (h, accumulated with +=); call 2: one type-2 record
 * (spin-orbit, stored with the reference's i<j sign flip). */
void sifrd1_(Fint &, Fint *, Fint &, Fint &, Fdouble *, Fint &num, Fint &last, Fint &itypea,
             Fint &itypeb, Fint &ifmt, Fint &ibvtyp, Fdouble *values, Fint *labels,
             Fdouble &fcore, Fint *, Fint &ierr) {
  int n = g_nbf;
  num = 0; ifmt = 0; ibvtyp = 0; fcore = 0.0; ierr = 0;
  if (g_rd1_calls == 0) {
    itypea = 0; itypeb = 1;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j <= i; ++j) {
        double v = g_h[(size_t)i * n + j];
        if (v == 0.0) continue;
        values[num] = v; labels[2 * num] = i + 1; labels[2 * num + 1] = j + 1; ++num;
      }
    last = 1;
  } else {
    itypea = 2; itypeb = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) {
        double v = g_so[(size_t)i * n + j];
        if (v == 0.0) continue;
        /* emit half the records with swapped labels to exercise the sign rule */
        if (((i + j) & 1) == 0) {
          values[num] = v; labels[2 * num] = i + 1; labels[2 * num + 1] = j + 1;
        } else {
          values[num] = -v; labels[2 * num] = j + 1; labels[2 * num + 1] = i + 1;
        }
        ++num;
      }
    last = 2;
  }
  ++g_rd1_calls;
}
void sifrd2_(Fint &, Fint *, Fint &, Fint &, Fdouble *, Fint &num, Fint &last, Fint &itypea,
             Fint &itypeb, Fint &ifmt, Fint &ibvtyp, Fdouble *values, Fint *labels, Fint *,
             Fint &ierr) {
  int n = g_nbf;
  num = 0;
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= i; ++j)
      for (int k = 1; k <= i; ++k) {
        int lmax = (k == i) ? j : k;
        for (int l = 1; l <= lmax; ++l) {
          long ij = nndaf(i - 1) + j, kl = nndaf(k - 1) + l;
          long idx = nndaf(max(ij, kl) - 1) + min(ij, kl);
          values[num] = g_eri[idx - 1];
          labels[4 * num] = i; labels[4 * num + 1] = j; labels[4 * num + 2] = k; labels[4 * num + 3] = l;
          ++num;
        }
      }
  last = 2; itypea = 3; itypeb = 0; ifmt = 0; ibvtyp = 0; ierr = 0;
}
void siftyp_(Fint &, Fint &, char chrtyp[MAX_TYPE_LENGTH]) { memset(chrtyp, ' ', MAX_TYPE_LENGTH); }
}

/* ---------------- state ---------------- */
static PsociIntegrals *s_ints = nullptr;
static PsociConfigs *s_cfg = nullptr;
static PsociDeterminants *s_det = nullptr;
static vector<JOUTFG> s_J;
static int s_nbf = 0, s_nelec = 0, s_ksym = 0, s_maxdet = 0, s_maxsef = 0;
static vector<long> s_sefoff;

extern "C" {

int ref_set_integrals(int nbf, const double *h, const double *so, const double *eri, double ecore) {
  g_nbf = nbf;
  g_h.assign(h, h + (size_t)nbf * nbf);
  g_so.assign(so, so + (size_t)nbf * nbf);
  g_eri.assign(eri, eri + nndaf(nndaf(nbf)));
  g_ecore = ecore;
  delete s_ints;
  s_ints = new PsociIntegrals(0, 2, "moints");
  s_ints->fetchAndProcessIntegrals();
  return 0;
}

double ref_fetch1e(int i, int j) { return s_ints->fetch1eIntegralValue(i, j); }
double ref_fetch2e(int i, int j, int k, int l) { return s_ints->fetch2eIntegralValue(i, j, k, l); }
double ref_core_energy(void) { return s_ints->fetchCoreEnergy(); }

/* occ: nconf*nbf bytes of 0/1/2.  Configurations are fed through setParams +
 * convertVectorToVectormap (PsociConfigs.C:516-531, :897-946), which keeps file order
 * and accepts all-open-shell configurations; determinants through the range overload
 * computeConfigs(start, stop, vector&) (PsociDeterminants.C:856-975). */
int ref_set_configs(int nbf, int nelec, int ksym, int mx_open, int nconf, const int *jsym,
                    const unsigned char *occ) {
  delete s_det; delete s_cfg;
  s_cfg = new PsociConfigs();
  vector<int> params = {nbf, nelec, ksym, nconf, mx_open, nelec % 2};
  s_cfg->setParams(params);
  vector<int> isym(jsym, jsym + nconf);
  vector<short> confs((size_t)nconf * nbf);
  for (size_t t = 0; t < confs.size(); ++t) confs[t] = (short)('0' + occ[t]);
  s_cfg->convertVectorToVectormap(isym, confs);
  s_det = new PsociDeterminants(s_cfg);
  s_J.clear();
  s_det->computeConfigs(1, nconf, s_J);
  s_nbf = nbf; s_nelec = nelec; s_ksym = ksym;
  s_maxdet = 0; s_maxsef = 0;
  s_sefoff.assign(nconf + 1, 0);
  for (int i = 0; i < nconf; ++i) {
    s_maxdet = max(s_maxdet, s_J[i].ndeti);
    s_maxsef = max(s_maxsef, s_J[i].nsefi);
    s_sefoff[i + 1] = s_sefoff[i] + s_J[i].nsefi;
  }
  return (int)s_J.size();
}

long ref_num_sefs(void) { return s_sefoff.empty() ? 0 : s_sefoff.back(); }

/* Per-config counts: out[3*i] = ndet, out[3*i+1] = nsef, out[3*i+2] = nopen. */
void ref_config_counts(int *out) {
  for (size_t i = 0; i < s_J.size(); ++i) {
    out[3 * i] = s_J[i].ndeti; out[3 * i + 1] = s_J[i].nsefi; out[3 * i + 2] = s_J[i].num_singly;
  }
}

/* Determinant table of config i: per det d (row stride 4 + 2*nbf):
 *   [nalpha, nbeta, ms, phase, sumsa, sumsb, alpha[0..nbf-1] (-1 padded), beta[0..nbf-1]] */
int ref_config_dets(int i, int *out) {
  const JOUTFG &c = s_J[i];
  int stride = 6 + 2 * s_nbf;
  for (int d = 0; d < c.ndeti; ++d) {
    int *row = out + (size_t)d * stride;
    row[0] = c.nalpha[d]; row[1] = c.nbeta[d]; row[2] = c.spin_projection[d]; row[3] = c.phases[d];
    row[4] = c.sumsa[d]; row[5] = c.sumsb[d];
    for (int t = 0; t < 2 * s_nbf; ++t) row[6 + t] = -1;
    for (int t = 0; t < c.nalpha[d]; ++t) row[6 + t] = c.alpha_spins[d][t];
    for (int t = 0; t < c.nbeta[d]; ++t) row[6 + s_nbf + t] = c.beta_spins[d][t];
  }
  return c.ndeti;
}

/* sefsef block for configurations (i, j), 0-based, via generateSOCIblocks
 * (PsociHamiltonian.C:401-558).  Returns the reference's status; out has nsef_i*nsef_j. */
int ref_block(int i, int j, double *out) {
  PsociHamiltonian H(s_nbf, s_nelec);
  H.specifyIntegrals(s_ints);
  H.setKsym(s_ksym);
  H.setPerSpatialValues(s_maxdet, s_maxsef);
  vector<double> sefsef;
  int st = H.generateSOCIblocks(s_J[i], s_J[j], sefsef);
  for (size_t t = 0; t < sefsef.size(); ++t) out[t] = sefsef[t];
  return st;
}

/* quick occupancy screen restating compareOrbMap (PsociGADeterminants.C:2249-2277):
 * excitation level <= 2 (and therefore |nopen_i - nopen_j| <= 4) */
static inline bool interacts(const unsigned char *oi, const unsigned char *oj, int nbf) {
  int d = 0;
  for (int p = 0; p < nbf; ++p) { d += abs((int)oi[p] - (int)oj[p]); if (d > 4) return false; }
  return true;
}

struct RowBuf { vector<long> cols; vector<double> vals; };

/* Lower-triangle H (rows of config i, columns of configs j <= i) in CSR, entries in the
 * reference's append order (j ascending, columns ascending inside a block, diagonal last).
 * Pass cols/vals = NULL to get nnz only.  occ is the same array given to ref_set_configs. */
long ref_build_lower(const unsigned char *occ, int nthreads, long *rowptr, int *cols, double *vals) {
  int nconf = (int)s_J.size();
  long N = s_sefoff.back();
  vector<vector<RowBuf>> rows(nconf);
  if (nthreads < 1) nthreads = 1;
  auto worker = [&](int tid) {
    PsociHamiltonian H(s_nbf, s_nelec);
    H.specifyIntegrals(s_ints);
    H.setKsym(s_ksym);
    H.setPerSpatialValues(s_maxdet, s_maxsef);
    vector<double> sefsef;
    for (int i = tid; i < nconf; i += nthreads) {
      int nsi = s_J[i].nsefi;
      rows[i].assign(nsi, RowBuf());
      long isef = s_sefoff[i];
      for (int j = 0; j <= i; ++j) {
        if (!interacts(occ + (size_t)i * s_nbf, occ + (size_t)j * s_nbf, s_nbf)) continue;
        H.generateSOCIblocks(s_J[i], s_J[j], sefsef);
        int nsj = s_J[j].nsefi;
        long jsef = s_sefoff[j];
        if ((long)sefsef.size() != (long)nsi * nsj) continue;
        for (int a = 0; a < nsi; ++a) {
          int jmax = (isef == jsef) ? a : nsj - 1;
          for (int b = 0; b <= jmax; ++b) {
            double x = sefsef[(size_t)a * nsj + b];
            if (fabs(x) >= MIN_DOUBLE_VALUE || (isef == jsef && a == b)) {
              rows[i][a].cols.push_back(jsef + b);
              rows[i][a].vals.push_back(x);
            }
          }
        }
      }
    }
  };
  vector<thread> th;
  for (int t = 0; t < nthreads; ++t) th.emplace_back(worker, t);
  for (auto &t : th) t.join();
  long nnz = 0;
  long r = 0;
  if (rowptr) rowptr[0] = 0;
  for (int i = 0; i < nconf; ++i)
    for (auto &rb : rows[i]) {
      if (cols) {
        for (size_t t = 0; t < rb.cols.size(); ++t) { cols[nnz + t] = (int)rb.cols[t]; vals[nnz + t] = rb.vals[t]; }
      }
      nnz += rb.cols.size();
      ++r;
      if (rowptr) rowptr[r] = nnz;
    }
  (void)N;
  return nnz;
}

/* CI vector files through the reference's PsociVector, in the call sequence of
 * PsociGAvectors::dumpVectorScalable / readVectorScalable (PsociGAvectors.C:207-326,
 * :539-658), one burst per root.  The exact file name is used (PsociVector(filename)). */
int ref_vec_write(const char *path, int binary, long nbasis, int nroots, const double *vecs, const char *title) {
  PsociVector pv{string(path)};
  pv.setMode(VECTOR_WRITE);
  pv.OpenFile();
  pair<int64_t, int64_t> info(nbasis, nroots);
  if (binary) pv.scalable_WriteHeaderBurstBinary(info);
  else pv.scalable_WriteHeaderBurst(info);
  for (int j = 0; j < nroots; ++j) {
    vector<double> v(vecs + (size_t)j * nbasis, vecs + (size_t)(j + 1) * nbasis);
    if (binary) pv.WriteBurstBinaryScalable(true, j + 1, v, info);
    else {
      pv.WriteBurstScalable(true, j + 1, v, info);
      pv.WriteBurstScalableEOL();
    }
  }
  (void)title;
  if (binary) pv.WriteBurstScalableBinaryTrailer();
  else pv.WriteBurstScalableTrailer();
  pv.CloseFile();
  return 0;
}

int ref_vec_read(const char *path, int binary, long nbasis, int maxroots, double *out) {
  PsociVector pv{string(path)};
  pv.setMode(VECTOR_READ);
  pv.OpenFile();
  pair<int64_t, int64_t> info;
  if (binary) pv.scalable_ReadHeaderBurstBinary(info);
  else pv.scalable_ReadHeaderBurst(info);
  if (info.first != nbasis) return -1;
  int n = (int)min<int64_t>(info.second, maxroots);
  for (int j = 0; j < n; ++j) {
    vector<double> v(nbasis);
    if (binary) pv.ReadBurstScalableBinary(true, (int)nbasis, v, info);
    else pv.ReadBurstScalable(true, (int)nbasis, v, info);
    /* the binary reader clears the vector and reads into its storage (PsociVector.C:461-480) */
    memcpy(out + (size_t)j * nbasis, v.data(), sizeof(double) * nbasis);
  }
  pv.CloseFile();
  return n;
}

/* CI-density block of configurations (i, j), 0-based, via the reference's own
 * generateSOCIblocksForCIDEN (PsociHamiltonian.C:572-705).  Returns its status. */
int ref_ciden_block(int i, int j, double *out) {
  PsociHamiltonian H(s_nbf, s_nelec);
  H.specifyIntegrals(s_ints);
  H.setKsym(s_ksym);
  H.setPerSpatialValues(s_maxdet, s_maxsef);
  vector<double> sefsef;
  int st = H.generateSOCIblocksForCIDEN(s_J[i], s_J[j], sefsef);
  for (size_t t = 0; t < sefsef.size(); ++t) out[t] = sefsef[t];
  return st;
}

/* Packed 1-particle densities of k roots (vecs: k x N root-major) from the reference's block
 * function, with the contraction of transformSEFSEFtoMOGET (PsociGAhamiltonian.C:10027-10099)
 * and the pair order j <= i of constructCIdensityAltOrbMapChunkJmap (:11570-11760) restated
 * here (they need Global Arrays).  occ is the array given to ref_set_configs. */
void ref_density1(const unsigned char *occ, int k, const double *vecs, double *dens) {
  const int nconf = (int)s_J.size();
  const long N = s_sefoff.back();
  const long ntri = (long)s_nbf * (s_nbf + 1) / 2;
  memset(dens, 0, sizeof(double) * k * ntri);
  PsociHamiltonian H(s_nbf, s_nelec);
  H.specifyIntegrals(s_ints);
  H.setKsym(s_ksym);
  H.setPerSpatialValues(s_maxdet, s_maxsef);
  vector<double> sefsef;
  auto two_d = [](int m, int n) { int a = max(m, n) + 1, b = min(m, n) + 1; return a * (a - 1) / 2 + b - 1; };
  for (int q = 0; q < k; ++q) {
    const double *v = vecs + (size_t)q * N;
    double *D = dens + (size_t)q * ntri;
    for (int i = 0; i < nconf; ++i) {
      const unsigned char *oi = occ + (size_t)i * s_nbf;
      for (int j = 0; j <= i; ++j) {
        const unsigned char *oj = occ + (size_t)j * s_nbf;
        /* compareOrbMapCIDEN + the open-shell difference test of the pair list */
        int ni = 0, nj = 0, ie = -1, je = -1;
        bool ok = abs(s_J[i].num_singly - s_J[j].num_singly) <= 2;
        for (int p = 0; p < s_nbf && ok; ++p) {
          int d = (int)oi[p] - (int)oj[p];
          if (d < 0) { nj -= d; je = p; if (nj > 1) ok = false; }
          else if (d > 0) { ni += d; ie = p; if (ni > 1) ok = false; }
        }
        if (!ok) continue;
        if (!H.generateSOCIblocksForCIDEN(s_J[i], s_J[j], sefsef)) continue;
        int nsi = s_J[i].nsefi, nsj = s_J[j].nsefi;
        const double *vi = v + s_sefoff[i], *vj = v + s_sefoff[j];
        if (i == j) {
          vector<pair<int, int>> mo;
          for (int t = 0; t < s_J[i].num_doubly; ++t) mo.push_back({s_J[i].doubly[t], 2});
          for (int t = 0; t < s_J[i].num_singly; ++t) mo.push_back({s_J[i].singly[t], 1});
          for (auto &po : mo) {
            double value = 0.0;
            for (int a = 0; a < nsi; ++a) {
              double temp = vj[a];
              for (int b = 0; b < nsj; ++b) value += sefsef[(size_t)a * nsj + b] * temp * vj[b] * po.second;
            }
            D[two_d(po.first, po.first)] += value;
          }
        } else {
          double value = 0.0;
          for (int a = 0; a < nsi; ++a) {
            double temp = vi[a];
            for (int b = 0; b < nsj; ++b) value += sefsef[(size_t)a * nsj + b] * temp * vj[b];
          }
          D[two_d(ie, je)] += value;
        }
      }
    }
  }
}

}  /* extern "C" */
