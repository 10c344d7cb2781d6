/* CPU restatement of PSOCI's Hamiltonian-build / sigma path — TEST INFRASTRUCTURE ONLY.
 *
 * This file is the oracle: a plain-C restatement of the reference algorithm, written
 * list-by-list the way the reference evaluates it, so that it checks the bit-string
 * CUDA path in psoci_gb300/csrc independently.  It is loaded (via ctypes) only by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm.
 *
 * Parity of this restatement is pinned against the reference's own compute sources,
 * compiled unchanged into oracle/_ref/libpsoci_ref.so (see oracle/ref_harness.cpp),
 * by tests/test_oracle_vs_reference.py and the fixtures in tests/golden/.
 *
 * What is restated, with the reference lines it follows (paths inside psociRestart-Cori/):
 *   integral tables     PsociIntegrals.C:424-540 (1-e + SO packing, SO overwrites h),
 *                       :853-909 (fetch1e / fetch2e / canonicalIndex / TwoEIndex)
 *   determinants        PsociDeterminants.C:856-975 (per-config counts), :1467-1505 (class
 *                       choice), :1680-2779 (fractional templates), :2780-2846 (alpha/beta
 *                       swap), :2848-3633 (EVEN), :3634-4353 (ODD), :4355-4476 (phase, sums)
 *   block elements      PsociHamiltonian.C:401-558 (generateSOCIblocks), :139-186 (double),
 *                       :190-261 (single + SO), :306-388 (diagonal), :709-858 (socig),
 *                       :860-1118 (generateSEFCIG), :1304-1322 + :1350-1516 (ciout / CDC^T)
 *   packing             PsociGAhamiltonian.C:4077-4136 (packSefsef: |x| >= 1e-8 or diagonal)
 *   H build loop        PsociGAhamiltonian.C:2530-2857 (rows i, j <= i, orbmap pre-screen
 *                       PsociGADeterminants.C:2249-2277)
 *   sigma               PsociGAhamiltonian.C:6921-7270 (lower-triangle symmetric product)
 */
#include "psoci_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MIN_VALUE 1.0e-8 /* PsociHamiltonian.hpp:37 MIN_DOUBLE_VALUE */
#define ORC_MAXOPEN 11
#define ORC_MAXDET 1024

typedef struct {
  int ndet, nsef, nopen, ndbl, jsym;
  int singly[ORC_MAXOPEN];
  long det0; /* first det record */
} orc_cfg;

struct orc_ctx {
  int nbf, nelec, ksym, mx_open, nconf;
  int stride; /* ints per det record: na, nb, ms, phase, suma, sumb, alpha[nelec], beta[nelec] */
  double *one; /* packed lower triangle, nbf(nbf+1)/2 */
  double *eri; /* canonical packed */
  unsigned char *occ;
  orc_cfg *cfg;
  int *dets;
  long *sefoff;
  int maxdet, maxsef;
  /* built lower CSR */
  long nnz;
  long *rowptr;
  int *cols;
  double *vals;
  /* rows of the last orc_build_rows sample: the SEF rows of the sampled configurations in
   * the order given, each the reference's lower-triangle row */
  int linear;  /* 1: keep blocks whose integral prefactors are zero (gradient oracle) */
  long s_nrows, s_nnz;
  long *s_rowptr;
  int *s_cols;
  double *s_vals;
};

static inline long tri(long i, long j) { /* 0-based (max,min) -> packed position */
  long a = i > j ? i : j, b = i > j ? j : i;
  return a * (a + 1) / 2 + b;
}
static inline long canon(int i, int j, int k, int l) {
  long ij = tri(i, j), kl = tri(k, l);
  return tri(ij, kl);
}
static inline double f1(const orc_ctx *c, int i, int j) { return c->one[tri(i, j)]; }
static inline double f2(const orc_ctx *c, int i, int j, int k, int l) { return c->eri[canon(i, j, k, l)]; }

double orc_fetch1e(const orc_ctx *c, int i, int j) { return f1(c, i, j); }
double orc_fetch2e(const orc_ctx *c, int i, int j, int k, int l) { return f2(c, i, j, k, l); }

/* ---------------------------------------------------------------------------
 * Determinants.  Open-shell positions 0..nopen-1 index the ascending singly list.
 * A "combo" is a bitmask over positions; enumerating masks of a given popcount in
 * increasing numeric order is the reference's nested-loop (co-lexicographic) order,
 * and the complement of the c-th combo is the (C-1-c)-th combo of the other size.
 * ------------------------------------------------------------------------- */
typedef struct { unsigned amask, bmask; int ms; } det_spec;

static int combos(int n, int k, unsigned *out) {
  int cnt = 0;
  for (unsigned m = 0; m < (1u << n); ++m)
    if (__builtin_popcount(m) == k) out[cnt++] = m;
  return cnt;
}

/* Returns ndet.  Paired scheme (even electron count, PsociDeterminants.C:2848-4353):
 * for each |delta| section, det 2c gets alpha = combo c (size m+delta), beta = complement,
 * ms = msbas+delta; det 2c+1 is its spin-flip partner with ms = msbas-delta.  The delta=0
 * section uses only the first half of the combos.  Sequential scheme (odd electron count,
 * :1680-2779): section s gives one det per combo of size m+1+s of the forward spin
 * (alpha for even s, beta for odd s), the other spin holds the complement,
 * ms = msbas + (1 + k*isgn)/2 with k = +-(2s+1); isgn = -1 swaps alpha and beta (:2833). */
static int det_specs(int nopen, int parity, int jsym, int ksym, int msbas, det_spec *out) {
  unsigned full = (nopen >= 32) ? 0xffffffffu : ((1u << nopen) - 1u);
  unsigned cb[ORC_MAXDET];
  int nd = 0;
  if (parity == 1) {
    int isgn = ((((jsym + 1) / 2) % 2) == 0) ? -1 : 1; /* :1475 */
    int m = (nopen - 1) / 2;
    for (int s = 0; m + 1 + s <= nopen; ++s) {
      int f = m + 1 + s;
      int n = combos(nopen, f, cb);
      int k = (2 * s + 1) * ((s % 2 == 0) ? 1 : -1);
      for (int t = 0; t < n; ++t) {
        unsigned fw = cb[t], bw = full & ~cb[t];
        det_spec d;
        if (s % 2 == 0) { d.amask = fw; d.bmask = bw; } else { d.amask = bw; d.bmask = fw; }
        if (isgn == -1) { unsigned x = d.amask; d.amask = d.bmask; d.bmask = x; }
        d.ms = msbas + (1 + k * isgn) / 2;
        out[nd++] = d;
      }
    }
    return nd;
  }
  if (nopen == 0) {
    out[0].amask = 0; out[0].bmask = 0; out[0].ms = msbas;
    return 1;
  }
  int m = nopen / 2;
  int even_class = ((jsym + 1) / 2 == (ksym + 1) / 2); /* :1476 */
  for (int delta = even_class ? 0 : 1; delta <= m; delta += 2) {
    int n = combos(nopen, m + delta, cb);
    int used = (delta == 0) ? n / 2 : n;
    for (int t = 0; t < used; ++t) {
      unsigned a = cb[t], b = full & ~cb[t];
      out[nd].amask = a; out[nd].bmask = b; out[nd].ms = msbas + delta; ++nd;
      out[nd].amask = b; out[nd].bmask = a; out[nd].ms = msbas - delta; ++nd;
    }
  }
  return nd;
}

/* computePhaseAndSort (:4355-4476): phase = parity of the inversions of the insertion
 * order (doubles ascending, then this spin's open shells ascending), summed over both
 * spins; sums = sum(orb+1); lists stored sorted. */
static void fill_det(const orc_ctx *c, const int *dbl, int ndbl, const int *sng, const det_spec *d,
                     int *rec) {
  int seqa[64], seqb[64], na = 0, nb = 0;
  for (int t = 0; t < ndbl; ++t) { seqa[na++] = dbl[t]; seqb[nb++] = dbl[t]; }
  for (int p = 0; p < ORC_MAXOPEN; ++p) {
    if (d->amask & (1u << p)) seqa[na++] = sng[p];
    if (d->bmask & (1u << p)) seqb[nb++] = sng[p];
  }
  int inv = 0, suma = 0, sumb = 0;
  for (int x = 0; x < na; ++x) { suma += seqa[x] + 1; for (int y = 0; y < x; ++y) inv += seqa[y] > seqa[x]; }
  for (int x = 0; x < nb; ++x) { sumb += seqb[x] + 1; for (int y = 0; y < x; ++y) inv += seqb[y] > seqb[x]; }
  /* insertion sort */
  for (int x = 1; x < na; ++x) { int v = seqa[x], y = x - 1; while (y >= 0 && seqa[y] > v) { seqa[y + 1] = seqa[y]; --y; } seqa[y + 1] = v; }
  for (int x = 1; x < nb; ++x) { int v = seqb[x], y = x - 1; while (y >= 0 && seqb[y] > v) { seqb[y + 1] = seqb[y]; --y; } seqb[y + 1] = v; }
  rec[0] = na; rec[1] = nb; rec[2] = d->ms; rec[3] = inv % 2; rec[4] = suma; rec[5] = sumb;
  int *al = rec + 6, *be = rec + 6 + c->nelec;
  for (int x = 0; x < c->nelec; ++x) { al[x] = -1; be[x] = -1; }
  for (int x = 0; x < na; ++x) al[x] = seqa[x];
  for (int x = 0; x < nb; ++x) be[x] = seqb[x];
}

orc_ctx *orc_create(int nbf, int nelec, int ksym, int mx_open, int nconf, const int *jsym,
                    const unsigned char *occ, const double *h, const double *so, const double *eri) {
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  c->nbf = nbf; c->nelec = nelec; c->ksym = ksym; c->mx_open = mx_open; c->nconf = nconf;
  long n1 = (long)nbf * (nbf + 1) / 2;
  long n2 = n1 * (n1 + 1) / 2;
  c->one = (double *)malloc(sizeof(double) * n1);
  c->eri = (double *)malloc(sizeof(double) * n2);
  /* PsociIntegrals.C:505-535: type-0 (h) records accumulate, type-2 (SO) records overwrite */
  for (int i = 0; i < nbf; ++i)
    for (int j = 0; j <= i; ++j) {
      double v = h[(size_t)i * nbf + j];
      double s = (i != j) ? so[(size_t)i * nbf + j] : 0.0;
      c->one[tri(i, j)] = (s != 0.0) ? s : v;
    }
  memcpy(c->eri, eri, sizeof(double) * n2);
  c->occ = (unsigned char *)malloc((size_t)nconf * nbf);
  memcpy(c->occ, occ, (size_t)nconf * nbf);
  c->cfg = (orc_cfg *)calloc(nconf, sizeof(orc_cfg));
  c->sefoff = (long *)calloc(nconf + 1, sizeof(long));
  c->stride = 6 + 2 * nelec;
  long totdet = 0;
  for (int i = 0; i < nconf; ++i) {
    orc_cfg *g = &c->cfg[i];
    const unsigned char *o = occ + (size_t)i * nbf;
    g->jsym = jsym[i];
    for (int p = 0; p < nbf; ++p) {
      if (o[p] == 1) g->singly[g->nopen++] = p;
      if (o[p] == 2) g->ndbl++;
    }
    int k = g->nopen - 1 > 0 ? g->nopen - 1 : 0; /* :954-955 */
    g->ndet = 1 << k;
    g->nsef = (1 << (k / 2)) * (1 << (k / 2));
    g->det0 = totdet;
    totdet += g->ndet;
    c->sefoff[i + 1] = c->sefoff[i] + g->nsef;
    if (g->ndet > c->maxdet) c->maxdet = g->ndet;
    if (g->nsef > c->maxsef) c->maxsef = g->nsef;
  }
  c->dets = (int *)malloc(sizeof(int) * (size_t)totdet * c->stride);
  det_spec spec[ORC_MAXDET];
  int dbl[128];
  for (int i = 0; i < nconf; ++i) {
    orc_cfg *g = &c->cfg[i];
    const unsigned char *o = occ + (size_t)i * nbf;
    int nd = 0;
    for (int p = 0; p < nbf; ++p) if (o[p] == 2) dbl[nd++] = p;
    int n = det_specs(g->nopen, nelec % 2, g->jsym, ksym, mx_open / 2, spec);
    (void)n;
    for (int d = 0; d < g->ndet; ++d)
      fill_det(c, dbl, nd, g->singly, &spec[d], c->dets + (size_t)(g->det0 + d) * c->stride);
  }
  return c;
}

void orc_destroy(orc_ctx *c) {
  if (!c) return;
  free(c->one); free(c->eri); free(c->occ); free(c->cfg); free(c->dets); free(c->sefoff);
  free(c->rowptr); free(c->cols); free(c->vals);
  free(c->s_rowptr); free(c->s_cols); free(c->s_vals);
  free(c);
}

long orc_num_sefs(const orc_ctx *c) { return c->sefoff[c->nconf]; }

void orc_config_counts(const orc_ctx *c, int *out) {
  for (int i = 0; i < c->nconf; ++i) {
    out[3 * i] = c->cfg[i].ndet; out[3 * i + 1] = c->cfg[i].nsef; out[3 * i + 2] = c->cfg[i].nopen;
  }
}

/* same layout as the reference harness: [na, nb, ms, phase, suma, sumb, alpha[nbf], beta[nbf]] */
int orc_config_dets(const orc_ctx *c, int i, int *out) {
  const orc_cfg *g = &c->cfg[i];
  int st = 6 + 2 * c->nbf;
  for (int d = 0; d < g->ndet; ++d) {
    const int *r = c->dets + (size_t)(g->det0 + d) * c->stride;
    int *w = out + (size_t)d * st;
    for (int t = 0; t < 6; ++t) w[t] = r[t];
    for (int t = 0; t < 2 * c->nbf; ++t) w[6 + t] = -1;
    for (int t = 0; t < r[0]; ++t) w[6 + t] = r[6 + t];
    for (int t = 0; t < r[1]; ++t) w[6 + c->nbf + t] = r[6 + c->nelec + t];
  }
  return g->ndet;
}

/* ---------------------------------------------------------------------------
 * Matrix elements of one configuration pair.
 * ------------------------------------------------------------------------- */
#define REC(c, g, d) ((c)->dets + (size_t)((g)->det0 + (d)) * (c)->stride)
#define NA(r) ((r)[0])
#define NB(r) ((r)[1])
#define MS(r) ((r)[2])
#define PH(r) ((r)[3])
#define SA(r) ((r)[4])
#define SB(r) ((r)[5])
#define AL(c, r) ((r) + 6)
#define BE(c, r) ((r) + 6 + (c)->nelec)

/* processDiagExcitation (PsociHamiltonian.C:306-388) */
static void diag_vnt(const orc_ctx *c, const orc_cfg *g, const unsigned char *occ, double *vnt) {
  int mm = 1;
  for (int i = 1; i < g->nopen; ++i)
    for (int j = 0; j < i; ++j) {
      int a = g->singly[i], b = g->singly[j];
      vnt[mm++] = f2(c, a, b, b, a);
    }
  double v = 0.0;
  for (int ib = 0; ib < c->nbf; ++ib) {
    if (occ[ib] == 0) continue;
    if (occ[ib] == 1) v += f1(c, ib, ib);
    else v += 2.0 * f1(c, ib, ib) + f2(c, ib, ib, ib, ib);
    for (int jb = 0; jb < ib; ++jb) {
      if (occ[jb] == 0) continue;
      int ninj = occ[ib] * occ[jb];
      if (ninj == 1) v += f2(c, ib, ib, jb, jb);
      else {
        double buf = 2.0 * f2(c, ib, ib, jb, jb);
        buf -= f2(c, ib, jb, ib, jb);
        if (ninj == 2) v += buf; else v += 2.0 * buf;
      }
    }
  }
  vnt[0] = v;
}

/* generateSEFCIG (PsociHamiltonian.C:860-1118) */
static void sefcig(const orc_ctx *c, const orc_cfg *gi, const orc_cfg *gj, const int *iex, const int *jex,
                   const double *vnt, double *dd) {
  int nbf = c->nbf;
  unsigned char figa[256], figb[256];
  for (int ii = 0; ii < gi->ndet; ++ii) {
    const int *ri = REC(c, gi, ii);
    const int *ai = AL(c, ri), *bi = BE(c, ri);
    memset(figa, 0, nbf); memset(figb, 0, nbf);
    for (int t = 0; t < NA(ri); ++t) figa[ai[t]] = 1;
    for (int t = 0; t < NB(ri); ++t) figb[bi[t]] = 1;
    for (int jj = 0; jj < gj->ndet; ++jj) {
      const int *rj = REC(c, gj, jj);
      if (MS(ri) != MS(rj)) continue;
      const int *aj = AL(c, rj), *bj = BE(c, rj);
      int nij[4] = {0, 0, 0, 0};
      int nmarka = 0;
      for (int ka = 0; ka < NA(rj); ++ka)
        if (figa[aj[ka]] != 1) { ++nmarka; if (nmarka > 2) break; nij[nmarka - 1] = ka; }
      int nmarkb = nmarka;
      for (int ka = 0; ka < NB(rj); ++ka)
        if (figb[bj[ka]] != 1) { ++nmarkb; if (nmarkb > 2) break; nij[nmarkb - 1] = ka; }
      if (!(nmarkb <= 2 && nmarka <= 2)) continue;
      double *out = dd + (size_t)ii * gj->ndet + jj;
      if (nmarkb == 0) {
        int mm = 0;
        *out = vnt[0];
        for (int io = 1; io < gi->nopen; ++io) {
          int iorb = gi->singly[io];
          for (int jo = 0; jo < io; ++jo) {
            int jorb = gj->singly[jo];
            ++mm;
            if (figa[iorb] == figa[jorb]) *out -= vnt[mm];
          }
        }
      } else if (nmarkb == 1) {
        int ncount = PH(ri) + PH(rj);
        if (abs(iex[0] - jex[0]) > 1) {
          int kbs = (iex[0] > jex[0] ? iex[0] : jex[0]) - 1;
          int ka = iex[0] + jex[0] - kbs;
          const int *lst = (nmarka != 0) ? ai : bi;
          int nl = (nmarka != 0) ? NA(ri) : NB(ri);
          for (int t = 0; t < nl; ++t) { if (lst[t] > kbs) break; if (lst[t] >= ka) ++ncount; }
        }
        double v = vnt[0];
        for (int ia = 0; ia < nbf; ++ia) {
          int tmp = (nmarka == 0) ? figb[ia] : figa[ia];
          if (tmp != 0 && ia != iex[0] && ia != jex[0] && figa[ia] + figb[ia] != 2)
            v -= f2(c, iex[0], ia, ia, jex[0]);
        }
        *out = (ncount % 2 == 1) ? -v : v;
      } else if (nmarka == 1) {
        int ncount = PH(ri) + PH(rj);
        int iex2 = aj[nij[0]], jex2 = bj[nij[1]];
        int iex3 = SA(ri) - SA(rj) + iex2;
        int jex3 = SB(ri) - SB(rj) + jex2;
        if (abs(iex2 - iex3) > 1) {
          int kbs = (iex2 > iex3 ? iex2 : iex3) - 1, ka = iex2 + iex3 - kbs;
          for (int t = 0; t < NA(ri); ++t) { if (ai[t] > kbs) break; if (ai[t] >= ka) ++ncount; }
        }
        if (abs(jex2 - jex3) > 1) {
          int kbs = (jex2 > jex3 ? jex2 : jex3) - 1, ka = jex2 + jex3 - kbs;
          for (int t = 0; t < NB(ri); ++t) { if (bi[t] > kbs) break; if (bi[t] >= ka) ++ncount; }
        }
        double v = f2(c, jex2, jex3, iex2, iex3);
        *out = (ncount % 2 == 1) ? -v : v;
      } else {
        int ncount = PH(ri) + PH(rj) + nij[1] - nij[0] - 1;
        if (iex[1] - iex[0] > 1) {
          const int *lst = (nmarka != 0) ? ai : bi;
          int nl = (nmarka != 0) ? NA(ri) : NB(ri);
          for (int t = 0; t < nl; ++t) { if (lst[t] >= iex[1]) break; if (lst[t] > iex[0]) ++ncount; }
        }
        double v = vnt[0] - vnt[1];
        *out = (ncount % 2 == 1) ? -v : v;
      }
    }
  }
}

/* socig (PsociHamiltonian.C:709-858): spin-orbit single excitations, no ms restriction */
static void socig(const orc_ctx *c, const orc_cfg *gi, const orc_cfg *gj, const int *iex, const int *jex,
                  double vnt0, double *dd) {
  int nbf = c->nbf;
  unsigned char figa[256], figb[256];
  int jsi = gi->jsym, jsj = gj->jsym;
  for (int ii = 0; ii < gi->ndet; ++ii) {
    const int *ri = REC(c, gi, ii);
    const int *ai = AL(c, ri), *bi = BE(c, ri);
    memset(figa, 0, nbf); memset(figb, 0, nbf);
    for (int t = 0; t < NA(ri); ++t) figa[ai[t]] = 1;
    for (int t = 0; t < NB(ri); ++t) figb[bi[t]] = 1;
    for (int jj = 0; jj < gj->ndet; ++jj) {
      const int *rj = REC(c, gj, jj);
      const int *aj = AL(c, rj), *bj = BE(c, rj);
      int nmarka = 0;
      for (int ka = 0; ka < NA(rj); ++ka) if (figa[aj[ka]] != 1) { ++nmarka; if (nmarka > 1) break; }
      int nmarkb = nmarka;
      for (int ka = 0; ka < NB(rj); ++ka) if (figb[bj[ka]] != 1) { ++nmarkb; if (nmarkb > 1) break; }
      if (!(nmarka <= 1 && nmarkb <= 1)) continue;
      int ncount = PH(ri) + PH(rj);
      if (NA(ri) < NA(rj)) {
        for (int t = 0; t < NB(ri); ++t) if (bi[t] < iex[0]) ++ncount;
        for (int t = 0; t < NA(rj); ++t) if (aj[t] > jex[0]) ++ncount;
        if ((jsi + jsj) % 2 == 0) ++ncount;
        else if (jsi % 2 == 1) ++ncount;
      } else if (NA(ri) > NA(rj)) {
        for (int t = 0; t < NA(ri); ++t) if (ai[t] > iex[0]) ++ncount;
        for (int t = 0; t < NB(rj); ++t) if (bj[t] < jex[0]) ++ncount;
        if ((jsi + jsj) % 2 != 0 && (jsi % 2) == 1) ++ncount;
      } else {
        if (nmarka == 0) ++ncount;
        if (jsi % 2 == 1) ++ncount;
        if (abs(iex[0] - jex[0]) > 1) {
          int kbs = (iex[0] > jex[0] ? iex[0] : jex[0]) - 1, ka = iex[0] + jex[0] - kbs;
          const int *lst = (nmarka != 0) ? ai : bi;
          int nl = (nmarka != 0) ? NA(ri) : NB(ri);
          for (int t = 0; t < nl; ++t) { if (lst[t] > kbs) break; if (lst[t] >= ka) ++ncount; }
        }
      }
      dd[(size_t)ii * gj->ndet + jj] = (ncount % 2 == 1) ? -vnt0 : vnt0;
    }
  }
}

/* ciout + transformCDCt (PsociHamiltonian.C:1350-1516) */
static void cdct(const orc_ctx *c, const orc_cfg *gi, const orc_cfg *gj, const double *dd, double *ss,
                 double *scratch) {
  int ndi = gi->ndet, ndj = gj->ndet, nsi = gi->nsef, nsj = gj->nsef;
  if (c->nelec % 2 == 1) { memcpy(ss, dd, sizeof(double) * ndi * ndj); return; }
  int ncpi = (gi->jsym % 2 != c->ksym % 2) ? 2 : 1;
  int ncpj = (gj->jsym % 2 != c->ksym % 2) ? 2 : 1;
  double r = sqrt(0.5);
  double mj = (ncpj == 2) ? -1.0 : 1.0, mi = (ncpi == 2) ? -1.0 : 1.0;
  const double *ds;
  int cols;
  if (gj->nopen != 0) {
    for (int ii = 0; ii < ndi; ++ii)
      for (int jj = 0; jj < nsj; ++jj) {
        double t = dd[(size_t)ii * ndj + 2 * jj];
        t += mj * dd[(size_t)ii * ndj + 2 * jj + 1];
        scratch[(size_t)ii * nsj + jj] = t * r;
      }
    ds = scratch; cols = nsj;
  } else {
    ds = dd; cols = ndj;
  }
  if (gi->nopen != 0) {
    for (int ii = 0; ii < nsi; ++ii)
      for (int jj = 0; jj < cols; ++jj) {
        double t = r * ds[(size_t)(2 * ii) * cols + jj];
        t += mi * r * ds[(size_t)(2 * ii + 1) * cols + jj];
        ss[(size_t)ii * cols + jj] = t;
      }
  } else {
    memcpy(ss, ds, sizeof(double) * ndi * cols);
  }
}

/* generateSOCIblocks (PsociHamiltonian.C:401-558).  out: nsef_i*nsef_j (zeros when the
 * reference produces no block).  Returns the reference's status. */
static int block_impl(const orc_ctx *c, int I, int J, double *out, double *dd, double *scratch) {
  const orc_cfg *gi = &c->cfg[I], *gj = &c->cfg[J];
  int nsi = gi->nsef, nsj = gj->nsef;
  memset(out, 0, sizeof(double) * nsi * nsj);
  if (abs(gi->nopen - gj->nopen) > 4) return 0;
  const unsigned char *io = c->occ + (size_t)I * c->nbf, *jo = c->occ + (size_t)J * c->nbf;
  int iex[2], jex[2], ni = 0, nj = 0;
  for (int p = 0; p < c->nbf; ++p) {
    int d = (int)io[p] - (int)jo[p];
    if (d < 0) { if (nj - d > 2) return 0; for (int t = 0; t < -d; ++t) jex[nj++] = p; }
    else if (d > 0) { if (ni + d > 2) return 0; for (int t = 0; t < d; ++t) iex[ni++] = p; }
  }
  memset(dd, 0, sizeof(double) * gi->ndet * gj->ndet);
  double vnt[1 + ORC_MAXOPEN * (ORC_MAXOPEN - 1) / 2 + 2];
  int sefstatus = 0;
  if (I == J) {
    diag_vnt(c, gi, io, vnt);
    sefcig(c, gi, gj, iex, jex, vnt, dd);
    sefstatus = 1;
  } else {
    int status = 0;
    sefstatus = 1;
    if (ni == 2) { /* processDoubleExcitation :139-186 */
      vnt[0] = f2(c, iex[0], jex[0], iex[1], jex[1]);
      vnt[1] = f2(c, iex[0], jex[1], iex[1], jex[0]);
      status = (vnt[0] == 0.0 && vnt[1] == 0.0 && !c->linear) ? 0 : 1;
    } else if (ni == 1) { /* processSingleExcitation :190-261 */
      int ie = iex[0], je = jex[0];
      if (gi->jsym != gj->jsym) {
        double v = f1(c, ie, je);
        if (v != 0.0 || c->linear) {
          if (je > ie) v = -v;
          v = v / 2;
          socig(c, gi, gj, iex, jex, v, dd);
        }
        status = 2;
      } else {
        double v = f1(c, ie, je) - f2(c, ie, je, ie, ie);
        for (int p = 0; p < c->nbf; ++p) {
          if (io[p] == 0) continue;
          double buf = f2(c, ie, je, p, p);
          v += buf;
          if (io[p] == 2) v += buf;
          if (io[p] == 2 && jo[p] == 2) v -= f2(c, ie, p, p, je);
        }
        vnt[0] = v;
        status = (v == 0.0 && !c->linear) ? 0 : 1;
      }
    }
    if (status == 1) sefcig(c, gi, gj, iex, jex, vnt, dd);
    if (status == 0) sefstatus = 0;
  }
  if (sefstatus == 1) cdct(c, gi, gj, dd, out, scratch);
  return sefstatus;
}

int orc_block(const orc_ctx *c, int i, int j, double *out) {
  double *dd = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *sc = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  int st = block_impl(c, i, j, out, dd, sc);
  free(dd); free(sc);
  return st;
}

/* ---------------------------------------------------------------------------
 * Lower-triangle H build (PsociGAhamiltonian.C:2530-2857 + packSefsef :4077-4136).
 * Threads take configurations round-robin, as the reference's -DSTATIC ranks do.
 * ------------------------------------------------------------------------- */
typedef struct { long n, cap; int *col; double *val; } rowbuf;
static void rb_push(rowbuf *r, int col, double v) {
  if (r->n == r->cap) {
    r->cap = r->cap ? 2 * r->cap : 64;
    r->col = (int *)realloc(r->col, sizeof(int) * r->cap);
    r->val = (double *)realloc(r->val, sizeof(double) * r->cap);
  }
  r->col[r->n] = col; r->val[r->n] = v; ++r->n;
}

typedef struct {
  orc_ctx *c; int tid, nth; rowbuf *rows; uint64_t *e1, *e2; int words;
  const int *only; int nonly;  /* optional list of row configurations */
} build_arg;

static void *build_worker(void *p) {
  build_arg *a = (build_arg *)p;
  orc_ctx *c = a->c;
  double *dd = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *sc = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *blk = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  int W = a->words;
  int count = a->only ? a->nonly : c->nconf;
  for (int ii = a->tid; ii < count; ii += a->nth) {
    int i = a->only ? a->only[ii] : ii;
    const orc_cfg *gi = &c->cfg[i];
    long isef = c->sefoff[i];
    for (int j = 0; j <= i; ++j) {
      /* orbmap pre-screen (compareOrbMap): sum |occ_i - occ_j| <= 4 */
      int d = 0;
      for (int w = 0; w < W; ++w)
        d += __builtin_popcountll(a->e1[(size_t)i * W + w] ^ a->e1[(size_t)j * W + w]) +
             __builtin_popcountll(a->e2[(size_t)i * W + w] ^ a->e2[(size_t)j * W + w]);
      if (d > 4) continue;
      int st = block_impl(c, i, j, blk, dd, sc);
      (void)st;
      const orc_cfg *gj = &c->cfg[j];
      long jsef = c->sefoff[j];
      for (int r = 0; r < gi->nsef; ++r) {
        int jmax = (isef == jsef) ? r : gj->nsef - 1;
        for (int s = 0; s <= jmax; ++s) {
          double x = blk[(size_t)r * gj->nsef + s];
          if (fabs(x) >= ORC_MIN_VALUE || (isef == jsef && r == s)) rb_push(&a->rows[isef + r], (int)(jsef + s), x);
        }
      }
    }
  }
  free(dd); free(sc); free(blk);
  return NULL;
}

long orc_build_lower(orc_ctx *c, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  long N = c->sefoff[c->nconf];
  int W = (c->nbf + 63) / 64;
  uint64_t *e1 = (uint64_t *)calloc((size_t)c->nconf * W, 8), *e2 = (uint64_t *)calloc((size_t)c->nconf * W, 8);
  for (int i = 0; i < c->nconf; ++i)
    for (int p = 0; p < c->nbf; ++p) {
      unsigned char o = c->occ[(size_t)i * c->nbf + p];
      if (o >= 1) e1[(size_t)i * W + p / 64] |= 1ull << (p % 64);
      if (o == 2) e2[(size_t)i * W + p / 64] |= 1ull << (p % 64);
    }
  rowbuf *rows = (rowbuf *)calloc(N, sizeof(rowbuf));
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  build_arg *args = (build_arg *)malloc(sizeof(build_arg) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    args[t].c = c; args[t].tid = t; args[t].nth = nthreads; args[t].rows = rows;
    args[t].e1 = e1; args[t].e2 = e2; args[t].words = W;
    args[t].only = NULL; args[t].nonly = 0;
    pthread_create(&th[t], NULL, build_worker, &args[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(th); free(args); free(e1); free(e2);
  free(c->rowptr); free(c->cols); free(c->vals);
  c->rowptr = (long *)malloc(sizeof(long) * (N + 1));
  long nnz = 0;
  c->rowptr[0] = 0;
  for (long r = 0; r < N; ++r) { nnz += rows[r].n; c->rowptr[r + 1] = nnz; }
  c->cols = (int *)malloc(sizeof(int) * (nnz ? nnz : 1));
  c->vals = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
  for (long r = 0; r < N; ++r) {
    memcpy(c->cols + c->rowptr[r], rows[r].col, sizeof(int) * rows[r].n);
    memcpy(c->vals + c->rowptr[r], rows[r].val, sizeof(double) * rows[r].n);
    free(rows[r].col); free(rows[r].val);
  }
  free(rows);
  c->nnz = nnz;
  return nnz;
}

void orc_copy_lower(const orc_ctx *c, long *rowptr, int *cols, double *vals) {
  long N = c->sefoff[c->nconf];
  memcpy(rowptr, c->rowptr, sizeof(long) * (N + 1));
  memcpy(cols, c->cols, sizeof(int) * c->nnz);
  memcpy(vals, c->vals, sizeof(double) * c->nnz);
}

/* Rows of a subset of configurations only (each against all j <= i), for timing samples.
 * Returns the stored element count; the rows are not kept. */
long orc_build_rows(orc_ctx *c, int nthreads, const int *rows, int nrows) {
  if (nthreads < 1) nthreads = 1;
  long N = c->sefoff[c->nconf];
  int W = (c->nbf + 63) / 64;
  uint64_t *e1 = (uint64_t *)calloc((size_t)c->nconf * W, 8), *e2 = (uint64_t *)calloc((size_t)c->nconf * W, 8);
  for (int i = 0; i < c->nconf; ++i)
    for (int p = 0; p < c->nbf; ++p) {
      unsigned char o = c->occ[(size_t)i * c->nbf + p];
      if (o >= 1) e1[(size_t)i * W + p / 64] |= 1ull << (p % 64);
      if (o == 2) e2[(size_t)i * W + p / 64] |= 1ull << (p % 64);
    }
  rowbuf *rb = (rowbuf *)calloc(N, sizeof(rowbuf));
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  build_arg *args = (build_arg *)malloc(sizeof(build_arg) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    args[t].c = c; args[t].tid = t; args[t].nth = nthreads; args[t].rows = rb;
    args[t].e1 = e1; args[t].e2 = e2; args[t].words = W; args[t].only = rows; args[t].nonly = nrows;
    pthread_create(&th[t], NULL, build_worker, &args[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  long nnz = 0, nr = 0;
  for (int q = 0; q < nrows; ++q) nr += c->sefoff[rows[q] + 1] - c->sefoff[rows[q]];
  free(c->s_rowptr); free(c->s_cols); free(c->s_vals);
  c->s_rowptr = (long *)malloc(sizeof(long) * (nr + 1));
  c->s_rowptr[0] = 0;
  c->s_nrows = nr;
  nr = 0;
  for (int q = 0; q < nrows; ++q)
    for (long r = c->sefoff[rows[q]]; r < c->sefoff[rows[q] + 1]; ++r, ++nr) c->s_rowptr[nr + 1] = c->s_rowptr[nr] + rb[r].n;
  c->s_nnz = c->s_rowptr[nr];
  c->s_cols = (int *)malloc(sizeof(int) * (c->s_nnz ? c->s_nnz : 1));
  c->s_vals = (double *)malloc(sizeof(double) * (c->s_nnz ? c->s_nnz : 1));
  nr = 0;
  for (int q = 0; q < nrows; ++q)
    for (long r = c->sefoff[rows[q]]; r < c->sefoff[rows[q] + 1]; ++r, ++nr) {
      memcpy(c->s_cols + c->s_rowptr[nr], rb[r].col, sizeof(int) * rb[r].n);
      memcpy(c->s_vals + c->s_rowptr[nr], rb[r].val, sizeof(double) * rb[r].n);
    }
  for (long r = 0; r < N; ++r) { nnz += rb[r].n; free(rb[r].col); free(rb[r].val); }
  free(rb); free(th); free(args); free(e1); free(e2);
  return nnz;
}

/* The rows kept by the last orc_build_rows: counts, then the CSR (rowptr[nrows+1], cols,
 * vals), rows in the order of the sampled configurations and their SEFs. */
void orc_sample_counts(const orc_ctx *c, long *nrows, long *nnz) {
  *nrows = c->s_nrows;
  *nnz = c->s_nnz;
}
void orc_copy_sample(const orc_ctx *c, long *rowptr, int *cols, double *vals) {
  memcpy(rowptr, c->s_rowptr, sizeof(long) * (c->s_nrows + 1));
  memcpy(cols, c->s_cols, sizeof(int) * c->s_nnz);
  memcpy(vals, c->s_vals, sizeof(double) * c->s_nnz);
}

/* diagonal H_rr (the reference keeps it last in each row, g_diag_sef) */
void orc_diag(const orc_ctx *c, double *diag) {
  long N = c->sefoff[c->nconf];
  for (long r = 0; r < N; ++r) {
    diag[r] = 0.0;
    for (long t = c->rowptr[r]; t < c->rowptr[r + 1]; ++t) if (c->cols[t] == r) diag[r] = c->vals[t];
  }
}

/* ---------------------------------------------------------------------------
 * Sigma from lower-triangle storage (matrixVectorProductsSplitChunkMultipleJchunks,
 * PsociGAhamiltonian.C:6921-7270): y_i += H_ij x_j (j <= i) and y_j += H_ij x_i (j < i).
 * x, y: k vectors of length n, vector-major.  Threads own disjoint vectors.
 * ------------------------------------------------------------------------- */
typedef struct {
  long n; const long *rp; const int *ci; const double *v; int k0, k1; const double *x; double *y;
} sig_arg;
static void *sig_worker(void *p) {
  sig_arg *a = (sig_arg *)p;
  for (int q = a->k0; q < a->k1; ++q) {
    const double *x = a->x + (size_t)q * a->n;
    double *y = a->y + (size_t)q * a->n;
    for (long i = 0; i < a->n; ++i) y[i] = 0.0;
    for (long i = 0; i < a->n; ++i) {
      double acc = 0.0, xi = x[i];
      for (long t = a->rp[i]; t < a->rp[i + 1]; ++t) {
        int j = a->ci[t];
        acc += a->v[t] * x[j];
        if (j < i) y[j] += a->v[t] * xi;
      }
      y[i] += acc;
    }
  }
  return NULL;
}
void orc_sigma_lower(long n, const long *rowptr, const int *cols, const double *vals, int k,
                     const double *x, double *y, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > k) nthreads = k;
  pthread_t th[256];
  sig_arg args[256];
  for (int t = 0; t < nthreads; ++t) {
    args[t].n = n; args[t].rp = rowptr; args[t].ci = cols; args[t].v = vals;
    args[t].k0 = (int)((long)k * t / nthreads); args[t].k1 = (int)((long)k * (t + 1) / nthreads);
    args[t].x = x; args[t].y = y;
    pthread_create(&th[t], NULL, sig_worker, &args[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------------------
 * 1-particle density matrix: the reference's CI-density (CIDEN) path.
 *   block               generateSOCIblocksForCIDEN (PsociHamiltonian.C:572-705) and
 *                       generateSEFCIGCIDEN (:1123-1269), transformed by ciout (CDC^T)
 *   contraction         transformSEFSEFtoMOGET (PsociGAhamiltonian.C:10027-10099)
 *   pair loop           constructCIdensityAltOrbMapChunkJmap (:11570-11760): pairs j <= i
 *                       with |nopen_i - nopen_j| <= 2 and at most one electron moved
 *                       (compareOrbMapCIDEN, PsociGADeterminants.C:2219-2240)
 *   packed index        twoDindex (PsociGAhamiltonian.C:10297-10302): lower triangle
 * Output per root: nbf(nbf+1)/2 values.  The diagonal holds sum_I occ_p(I) c_I.c_I (times
 * the transformed identity); an off-diagonal (p, q) holds sum over pairs j < i of the
 * c_i S c_j contraction for the single excitation p <-> q, once per unordered pair, as the
 * reference accumulates it.
 * ------------------------------------------------------------------------- */
static int ciden_block(const orc_ctx *c, int I, int J, double *out, double *dd, double *scratch, int *ie,
                       int *je) {
  const orc_cfg *gi = &c->cfg[I], *gj = &c->cfg[J];
  int nsi = gi->nsef, nsj = gj->nsef;
  memset(out, 0, sizeof(double) * nsi * nsj);
  memset(dd, 0, sizeof(double) * gi->ndet * gj->ndet);
  if (abs(gi->nopen - gj->nopen) > 2) return 0;
  if (gi->jsym != gj->jsym) return 0;
  int iex = -1, jex = -1;
  if (I != J) {
    const unsigned char *io = c->occ + (size_t)I * c->nbf, *jo = c->occ + (size_t)J * c->nbf;
    int ni = 0, nj = 0;
    for (int p = 0; p < c->nbf; ++p) {
      int d = (int)io[p] - (int)jo[p];
      if (d < 0) { if (nj - d > 1) return 0; nj -= d; jex = p; }
      else if (d > 0) { if (ni + d > 1) return 0; ni += d; iex = p; }
    }
  }
  *ie = iex; *je = jex;
  int nbf = c->nbf;
  unsigned char figa[256], figb[256];
  for (int ii = 0; ii < gi->ndet; ++ii) {
    const int *ri = REC(c, gi, ii);
    const int *ai = AL(c, ri), *bi = BE(c, ri);
    memset(figa, 0, nbf); memset(figb, 0, nbf);
    for (int t = 0; t < NA(ri); ++t) figa[ai[t]] = 1;
    for (int t = 0; t < NB(ri); ++t) figb[bi[t]] = 1;
    for (int jj = 0; jj < gj->ndet; ++jj) {
      const int *rj = REC(c, gj, jj);
      if (MS(ri) != MS(rj)) continue;
      const int *aj = AL(c, rj), *bj = BE(c, rj);
      int nmarka = 0, nmarkb;
      for (int t = 0; t < NA(rj); ++t) if (!figa[aj[t]]) { if (++nmarka > 1) break; }
      nmarkb = nmarka;
      for (int t = 0; t < NB(rj); ++t) if (!figb[bj[t]]) { if (++nmarkb > 1) break; }
      double v;
      if (nmarka > 1 || nmarkb > 1) v = 0.0;
      else if (nmarkb == 0) v = 1.0;
      else {
        int ncount = PH(ri) + PH(rj);
        if (abs(iex - jex) > 1) {
          int kbs = (iex > jex ? iex : jex) - 1, ka = iex + jex - kbs;
          const int *lst = (nmarka != 0) ? ai : bi;
          int nl = (nmarka != 0) ? NA(ri) : NB(ri);
          for (int t = 0; t < nl; ++t) { if (lst[t] > kbs) break; if (lst[t] >= ka) ++ncount; }
        }
        v = (ncount % 2 == 1) ? -1.0 : 1.0;
      }
      dd[(size_t)ii * gj->ndet + jj] = v;
    }
  }
  cdct(c, gi, gj, dd, out, scratch);
  return 1;
}

int orc_ciden_block(const orc_ctx *c, int i, int j, double *out) {
  double *dd = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *sc = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  int ie, je;
  int st = ciden_block(c, i, j, out, dd, sc, &ie, &je);
  free(dd); free(sc);
  return st;
}

/* rows: the configurations I whose pairs (I, J <= I) are accumulated (NULL: all, in order) */
static void density1_rows(const orc_ctx *c, int k, const double *vecs, int nrows, const int *rows, double *dens) {
  const long N = c->sefoff[c->nconf];
  const long ntri = (long)c->nbf * (c->nbf + 1) / 2;
  memset(dens, 0, sizeof(double) * k * ntri);
  double *dd = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *sc = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *ss = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  for (int q = 0; q < k; ++q) {
    const double *v = vecs + (size_t)q * N;
    double *D = dens + (size_t)q * ntri;
    for (int t = 0; t < nrows; ++t) {
      const int I = rows ? rows[t] : t;
      const orc_cfg *gi = &c->cfg[I];
      const unsigned char *io = c->occ + (size_t)I * c->nbf;
      for (int J = 0; J <= I; ++J) {
        const orc_cfg *gj = &c->cfg[J];
        int ie, je;
        if (!ciden_block(c, I, J, ss, dd, sc, &ie, &je)) continue;
        const double *vi = v + c->sefoff[I], *vj = v + c->sefoff[J];
        int nsi = gi->nsef, nsj = gj->nsef;
        if (I == J) {
          /* occupied orbitals: doubly occupied first, then singly occupied, ascending */
          for (int pass = 2; pass >= 1; --pass)
            for (int p = 0; p < c->nbf; ++p) {
              if (io[p] != pass) continue;
              double value = 0.0;
              for (int a = 0; a < nsi; ++a) {
                double temp = vj[a];
                for (int b = 0; b < nsj; ++b) value += ss[(size_t)a * nsj + b] * temp * vj[b] * pass;
              }
              D[tri(p, p)] += value;
            }
        } else {
          double value = 0.0;
          for (int a = 0; a < nsi; ++a) {
            double temp = vi[a];
            for (int b = 0; b < nsj; ++b) value += ss[(size_t)a * nsj + b] * temp * vj[b];
          }
          D[tri(ie, je)] += value;
        }
      }
    }
  }
  free(dd); free(sc); free(ss);
}

void orc_density1(const orc_ctx *c, int k, const double *vecs, double *dens) {
  density1_rows(c, k, vecs, c->nconf, NULL, dens);
}

/* the pairs of the listed rows only (a sample of the reference loop, for timing) */
void orc_density1_rows(const orc_ctx *c, int k, const double *vecs, int nrows, const int *rows, double *dens) {
  density1_rows(c, k, vecs, nrows, rows, dens);
}

/* ---------------------------------------------------------------------------
 * Energy gradients with respect to the packed integral tables — the checker of the GPU
 * adjoint.  E_r = c_r^T H c_r.  Each element of H is a sum of table entries with fixed
 * coefficients once the reference's zero-prefactor skips (processDoubleExcitation,
 * processSingleExcitation and the spin-orbit test, PsociHamiltonian.C:139-261) are left out,
 * so dE_r / d table[t] = c_r^T H(e_t) c_r with H(e_t) built from the unit table e_t — one
 * build per entry, no adjoint logic.  H(e_t) holds the reference's stored form: blocks of
 * pairs j < i counted twice, diagonal blocks from their lower triangle mirrored.
 * vecs: k x N root-major; grad_one: k x nbf(nbf+1)/2; grad_eri: k x NNDAF(NNDAF(nbf)).
 * nonzero_only: entries whose table value is zero are skipped (left at 0).
 * ------------------------------------------------------------------------- */
typedef struct {
  const orc_ctx *c; int tid, nth, k, nonzero_only; const double *vecs; double *g1, *g2;
} grad_arg;

static void *grad_worker(void *p) {
  grad_arg *a = (grad_arg *)p;
  const orc_ctx *c0 = a->c;
  orc_ctx cc = *c0;
  long n1 = (long)c0->nbf * (c0->nbf + 1) / 2, n2 = n1 * (n1 + 1) / 2, N = c0->sefoff[c0->nconf];
  cc.one = (double *)calloc(n1, sizeof(double));
  cc.eri = (double *)calloc(n2, sizeof(double));
  cc.linear = 1;
  double *dd = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *sc = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  double *blk = (double *)malloc(sizeof(double) * ORC_MAXDET * ORC_MAXDET);
  for (long t = a->tid; t < n1 + n2; t += a->nth) {
    int in_one = t < n1;
    long u = in_one ? t : t - n1;
    double orig = in_one ? c0->one[u] : c0->eri[u];
    if (a->nonzero_only && orig == 0.0) continue;
    if (in_one) cc.one[u] = 1.0; else cc.eri[u] = 1.0;
    for (int r = 0; r < a->k; ++r) {
      const double *v = a->vecs + (size_t)r * N;
      double e = 0.0;
      for (int i = 0; i < c0->nconf; ++i) {
        const orc_cfg *gi = &c0->cfg[i];
        for (int j = 0; j <= i; ++j) {
          if (block_impl(&cc, i, j, blk, dd, sc) == 0) continue;
          const orc_cfg *gj = &c0->cfg[j];
          const double *vi = v + c0->sefoff[i], *vj = v + c0->sefoff[j];
          for (int x = 0; x < gi->nsef; ++x)
            for (int y = 0; y < gj->nsef; ++y) {
              if (i == j && y > x) continue;
              double f = (i == j && x == y) ? 1.0 : 2.0;
              e += f * vi[x] * blk[(size_t)x * gj->nsef + y] * vj[y];
            }
        }
      }
      if (in_one) a->g1[(size_t)r * n1 + u] = e; else a->g2[(size_t)r * n2 + u] = e;
    }
    if (in_one) cc.one[u] = 0.0; else cc.eri[u] = 0.0;
  }
  free(dd); free(sc); free(blk); free(cc.one); free(cc.eri);
  return NULL;
}

void orc_energy_gradient(const orc_ctx *c, int k, const double *vecs, int nonzero_only, double *grad_one,
                         double *grad_eri, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  long n1 = (long)c->nbf * (c->nbf + 1) / 2, n2 = n1 * (n1 + 1) / 2;
  memset(grad_one, 0, sizeof(double) * k * n1);
  memset(grad_eri, 0, sizeof(double) * k * n2);
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  grad_arg *args = (grad_arg *)malloc(sizeof(grad_arg) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    args[t].c = c; args[t].tid = t; args[t].nth = nthreads; args[t].k = k; args[t].nonzero_only = nonzero_only;
    args[t].vecs = vecs; args[t].g1 = grad_one; args[t].g2 = grad_eri;
    pthread_create(&th[t], NULL, grad_worker, &args[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(th); free(args);
}

/* ---------------------------------------------------------------------------
 * The reference's CPU Davidson, restated for the timed CPU baseline.
 *
 * sigma: y = H x for one vector from the lower triangle, rows split over threads as the
 * reference splits them over MPI ranks (matrixVectorProductsSplitChunkMultipleJchunks,
 * PsociGAhamiltonian.C:6921-7270): y_i += H_ij x_j and y_j += H_ij x_i (j < i) into a
 * private y per thread, then summed (the reference's MPI_Allreduce).
 *
 * loop: driver.PSOCI.splittest.C:1050-1311 with the production flags (INCREMENTAL,
 * NEWRNOMRS, DIAGGOP, MODIFIED_EXPAND): unit-vector guess on the first nroots SEFs
 * (PsociGAvectors.C:687-726); per iteration the new column of G = V^T H V, the subspace
 * eigen-solve, residual norms from root curroot on until one exceeds the tolerance, a
 * preconditioned residual t_i = r_i / (D_i - lambda) where |D_i - lambda| > 1e-3
 * (PsociGAbasis.C:1860-1919), one modified Gram-Schmidt pass and normalisation
 * (:1371-1474), its H*v; tolerance 1e-3 first, then rtol; collapse to 2 nroots Ritz vectors
 * (V and HV, no recompute, :483-583) when the basis exceeds maxsub.  The subspace solve is a
 * cyclic Jacobi (the basis is orthonormal, so dsygv's metric is the identity).
 * ------------------------------------------------------------------------- */
typedef struct {
  long n; const long *rp; const int *ci; const double *v; const double *x; double *y; long r0, r1;
} sigr_arg;

static void *sigr_worker(void *p) {
  sigr_arg *a = (sigr_arg *)p;
  memset(a->y, 0, sizeof(double) * a->n);
  for (long i = a->r0; i < a->r1; ++i) {
    double s = 0.0;
    const double xi = a->x[i];
    for (long e = a->rp[i]; e < a->rp[i + 1]; ++e) {
      const int j = a->ci[e];
      const double h = a->v[e];
      s += h * a->x[j];
      if (j != i) a->y[j] += h * xi;
    }
    a->y[i] += s;
  }
  return NULL;
}

typedef struct {
  long n, nrows;
  const long *rp; const int *ci; const double *v;
  int nthreads;
  double *ybuf;  /* nthreads x n */
  long *cut;     /* nthreads + 1 row boundaries, balanced by stored elements */
} sigr_plan;

static void sigr_apply(const sigr_plan *P, const double *x, double *y) {
  pthread_t th[256];
  sigr_arg args[256];
  for (int t = 0; t < P->nthreads; ++t) {
    args[t].n = P->n; args[t].rp = P->rp; args[t].ci = P->ci; args[t].v = P->v; args[t].x = x;
    args[t].y = P->ybuf + (size_t)t * P->n; args[t].r0 = P->cut[t]; args[t].r1 = P->cut[t + 1];
    pthread_create(&th[t], NULL, sigr_worker, &args[t]);
  }
  for (int t = 0; t < P->nthreads; ++t) pthread_join(th[t], NULL);
  for (long i = 0; i < P->n; ++i) {
    double s = 0.0;
    for (int t = 0; t < P->nthreads; ++t) s += P->ybuf[(size_t)t * P->n + i];
    y[i] = s;
  }
}

static void sigr_init(sigr_plan *P, long n, const long *rp, const int *ci, const double *v, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  P->n = n; P->rp = rp; P->ci = ci; P->v = v; P->nthreads = nthreads;
  P->ybuf = (double *)malloc(sizeof(double) * (size_t)nthreads * n);
  P->cut = (long *)malloc(sizeof(long) * (nthreads + 1));
  long nnz = rp[n], r = 0;
  P->cut[0] = 0;
  for (int t = 1; t < nthreads; ++t) {
    long target = nnz * t / nthreads;
    while (r < n && rp[r] < target) ++r;
    P->cut[t] = r;
  }
  P->cut[nthreads] = n;
}

/* y = H x for one vector, rows over threads (the timed CPU sigma) */
void orc_sigma_lower_rows(long n, const long *rowptr, const int *cols, const double *vals, const double *x,
                          double *y, int nthreads) {
  sigr_plan P;
  sigr_init(&P, n, rowptr, cols, vals, nthreads);
  sigr_apply(&P, x, y);
  free(P.ybuf); free(P.cut);
}

/* cyclic Jacobi eigen-solve of a symmetric m x m matrix (row-major, destroyed); w ascending,
 * Y column c = eigenvector c (row-major m x m) */
static void jacobi_eig(int m, double *A, double *w, double *Y) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) Y[i * m + j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) { tot += A[i * m + j] * A[i * m + j]; if (i != j) off += A[i * m + j] * A[i * m + j]; }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        double apq = A[p * m + q];
        if (fabs(apq) < 1e-300) continue;
        double app = A[p * m + p], aqq = A[q * m + q];
        double th = (aqq - app) / (2.0 * apq);
        double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < m; ++k) {
          double akp = A[k * m + p], akq = A[k * m + q];
          A[k * m + p] = cs * akp - sn * akq;
          A[k * m + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < m; ++k) {
          double apk = A[p * m + k], aqk = A[q * m + k];
          A[p * m + k] = cs * apk - sn * aqk;
          A[q * m + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < m; ++k) {
          double ykp = Y[k * m + p], ykq = Y[k * m + q];
          Y[k * m + p] = cs * ykp - sn * ykq;
          Y[k * m + q] = sn * ykp + cs * ykq;
        }
      }
  }
  /* sort ascending */
  int idx[128];
  for (int i = 0; i < m; ++i) { idx[i] = i; w[i] = A[i * m + i]; }
  for (int i = 1; i < m; ++i)
    for (int j = i; j > 0 && w[idx[j]] < w[idx[j - 1]]; --j) { int t = idx[j]; idx[j] = idx[j - 1]; idx[j - 1] = t; }
  double wt[128], Yt[128 * 128];
  for (int i = 0; i < m; ++i) wt[i] = w[idx[i]];
  for (int i = 0; i < m; ++i)
    for (int c = 0; c < m; ++c) Yt[i * m + c] = Y[i * m + idx[c]];
  memcpy(w, wt, sizeof(double) * m);
  memcpy(Y, Yt, sizeof(double) * m * m);
}

/* Returns 0 when converged, 1 at the iteration limit.  stats[0] iterations, [1] sigma
 * vectors, [2] collapses. */
int orc_davidson_ref(long n, const long *rowptr, const int *cols, const double *vals, const double *diag,
                     int nroots, int maxsub, double rtol, int max_iter, int nthreads, double *evals, double *rnorms,
                     long *stats) {
  if (maxsub > 127) maxsub = 127;
  const int ld = maxsub + 1;
  double *V = (double *)calloc((size_t)n * ld, sizeof(double));   /* vector c at c*n */
  double *HV = (double *)calloc((size_t)n * ld, sizeof(double));
  double *G = (double *)calloc((size_t)ld * ld, sizeof(double));
  double *A = (double *)malloc(sizeof(double) * ld * ld), *Y = (double *)malloc(sizeof(double) * ld * ld);
  double *w = (double *)malloc(sizeof(double) * ld);
  double *r = (double *)malloc(sizeof(double) * n), *t = (double *)malloc(sizeof(double) * n);
  double *xr = (double *)malloc(sizeof(double) * n), *tmp = (double *)malloc(sizeof(double) * (size_t)n * 2 * nroots);
  sigr_plan P;
  sigr_init(&P, n, rowptr, cols, vals, nthreads);
  long nsig = 0, collapses = 0, total = 0;
  int m = nroots;
  for (int c = 0; c < nroots; ++c) V[(size_t)c * n + c] = 1.0;
  for (int c = 0; c < nroots; ++c) { sigr_apply(&P, V + (size_t)c * n, HV + (size_t)c * n); ++nsig; }
  int nupd = m, curroot = 1, converged = 0, count = 0, eig_m = 0;
  const double coarse = 1e-3;
  double cur_rtol = coarse;
  for (int i = 0; i < nroots; ++i) rnorms[i] = -1.0;
  while (count < max_iter && !converged) {
    ++total; ++count;
    /* generateIncrementalSubspace(nupd) */
    for (int j = m - nupd; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        double s = 0.0;
        const double *vi = V + (size_t)i * n, *hj = HV + (size_t)j * n;
        for (long q = 0; q < n; ++q) s += vi[q] * hj[q];
        G[i * ld + j] = s;
        G[j * ld + i] = s;
      }
    /* diagSubspaceGOP */
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) A[i * m + j] = 0.5 * (G[i * ld + j] + G[j * ld + i]);
    jacobi_eig(m, A, w, Y);
    eig_m = m;
    converged = 1;
    for (int it = curroot; it <= nroots; ++it) {
      /* computeRnormSingle */
      const int c = it - 1;
      double nr = 0.0;
      for (long q = 0; q < n; ++q) {
        double hx = 0.0, xx = 0.0;
        for (int s = 0; s < m; ++s) { hx += HV[(size_t)s * n + q] * Y[s * m + c]; xx += V[(size_t)s * n + q] * Y[s * m + c]; }
        r[q] = hx - w[c] * xx;
        nr += r[q] * r[q];
      }
      nr = sqrt(nr);
      rnorms[c] = nr;
      if (nr > cur_rtol) { converged = 0; curroot = it; break; }
    }
    if (!converged) {
      /* preconditionAndNewVectorIncore + appendScratchVector */
      const double shift = w[curroot - 1];
      for (long q = 0; q < n; ++q) {
        double d = diag[q] - shift;
        t[q] = (fabs(d) > 1e-3) ? r[q] / d : r[q];
      }
      for (int s = 0; s < m; ++s) {
        const double *vs = V + (size_t)s * n;
        double dot = 0.0;
        for (long q = 0; q < n; ++q) dot += vs[q] * t[q];
        for (long q = 0; q < n; ++q) t[q] -= dot * vs[q];
      }
      double nt = 0.0;
      for (long q = 0; q < n; ++q) nt += t[q] * t[q];
      nt = sqrt(nt);
      if (nt > 0.0) {
        for (long q = 0; q < n; ++q) V[(size_t)m * n + q] = t[q] / nt;
        sigr_apply(&P, V + (size_t)m * n, HV + (size_t)m * n);
        ++nsig;
        ++m;
      }
      nupd = 1;
    }
    int collapse_to = 0;
    if (converged && cur_rtol == coarse) {
      converged = 0; count = 0; cur_rtol = rtol; curroot = 1;
      if (m >= 2 * nroots) collapse_to = 2 * nroots;
      nupd = m;
    }
    if (m > maxsub) collapse_to = 2 * nroots;
    if (collapse_to) {
      /* expandAndReplaceVectorsNew over the basis of the last eigen-solve */
      for (int pass = 0; pass < 2; ++pass) {
        double *B = pass == 0 ? V : HV;
        for (int c = 0; c < collapse_to; ++c)
          for (long q = 0; q < n; ++q) {
            double s = 0.0;
            for (int k2 = 0; k2 < eig_m; ++k2) s += B[(size_t)k2 * n + q] * Y[k2 * eig_m + c];
            tmp[(size_t)c * n + q] = s;
          }
        memcpy(B, tmp, sizeof(double) * (size_t)n * collapse_to);
      }
      m = collapse_to;
      nupd = m;
      ++collapses;
    }
  }
  for (int i = 0; i < nroots; ++i) evals[i] = w[i];
  stats[0] = total; stats[1] = nsig; stats[2] = collapses;
  free(V); free(HV); free(G); free(A); free(Y); free(w); free(r); free(t); free(xr); free(tmp);
  free(P.ybuf); free(P.cut);
  return converged ? 0 : 1;
}
