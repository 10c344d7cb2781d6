// Hamiltonian build on the device: neighbour screen, Slater-Condon SEF blocks, full CSR.
//
// Reference path (psociRestart-Cori/):
//   PsociGAhamiltonian.C:2530-2857  build loop: rows of configuration i, columns j <= i
//   PsociGADeterminants.C:2249-2277 orbmap screen (excitation level <= 2)
//   PsociHamiltonian.C:401-558      generateSOCIblocks: excitation analysis and dispatch
//   PsociHamiltonian.C:139-388      double / single / spin-orbit / diagonal integral sums
//   PsociHamiltonian.C:709-858      socig: spin-orbit determinant elements
//   PsociHamiltonian.C:860-1118     generateSEFCIG: spin-free determinant elements
//   PsociHamiltonian.C:1350-1516    ciout / transformCDCt: det -> SEF (double group) transform
//   PsociGAhamiltonian.C:4077-4136  packSefsef: keep |x| >= 1e-8 and the diagonal
//
// Storage.  The reference keeps the lower triangle and runs a symmetric product.  On one
// GPU the full matrix in CSR streams twice the bytes but needs no scattered atomics in
// sigma, so both triangles are stored.  Every off-diagonal element is the reference's
// lower-triangle value: a block (I, J) with J > I is evaluated as the reference's block
// (J, I) and transposed, and the upper half of a diagonal block mirrors its lower half.
// Rows are written in ascending column order, deterministically, without atomics:
//
//   1. screen:  per configuration, the sorted list of configurations within two
//               excitations (XOR + popcount on occupancy bit-planes);
//   2. segments of <= 32 neighbours per row configuration, one warp each;
//   3. count:   each warp evaluates its SEF elements and counts kept ones per row;
//   4. scan:    per-row totals -> rowptr; per-segment row offsets;
//   5. fill:    the same evaluation writes columns and values at those offsets.
//
// Floating point follows the reference's operation order; this file is compiled with
// --fmad=false so products and sums round as the reference's do.
#include <algorithm>
#include <chrono>
#include <cstdio>

#include "psoci_internal.cuh"

namespace {

enum { K_NONE = 0, K_DIAG = 1, K_SINGLE = 2, K_DOUBLE = 3, K_SO = 4 };

constexpr int WARPS_PER_CTA = 4;
constexpr int MAXK = 1 + PSOCI_MAX_OPEN * (PSOCI_MAX_OPEN - 1) / 2;  // diagonal vnt list

struct PairInfo {
  int64_t detA, detB;   // first determinant of A, B
  int64_t colbase;      // first SEF of the neighbour J
  int A, B;             // configurations in the reference's roles (A = "iconf")
  int kind, swap;       // swap: J > I, element (t, r) of block (J, I)
  int iex0, iex1, jex0; // excitation orbitals of A -> B (ascending, with multiplicity)
  int nopenA, nopenB, jsA, jsB, nsefJ;
  double v0, v1;
  double X[PSOCI_MAX_OPEN];  // single: (iex0 s|s jex0) over the open shells s of A
  uint64_t SA[PSOCI_MAX_WORDS];
};

struct WarpSmem {
  PairInfo pi[PSOCI_SEG];
  int itemoff[PSOCI_SEG + 1];
  double K[MAXK];  // diagonal: K[0] = vnt(1), K[mm] = open-pair exchange (reference order)
};

struct Params {
  int nconf, nbf, nelec, ksym;
  const uint64_t *e1, *e2;
  const int32_t *jsym, *nopen;
  const int64_t *sefoff, *detoff;
  const uint64_t *alpha, *beta;
  const uint8_t *phase, *nalpha;
  const double *one, *eri;
  // screen
  const int64_t *nbroff;
  int32_t *nbr;
  // segments
  int64_t nseg;
  const int32_t *seg_cfg;
  const int64_t *seg_k0;
  const int32_t *seg_n;
  const int64_t *seg_rowoff;
  int64_t *seg_cnt;        // count pass output / fill pass row offsets (local)
  const int64_t *rowptr;
  int32_t *col;
  double *val;
  float *val32;
  double *diag;
};

// ------------------------------------------------------------------------------------
// bit helpers over W words
// ------------------------------------------------------------------------------------
template <int W>
__device__ __forceinline__ int popc_range(const uint64_t *x, int lo, int hi) {
  if (lo > hi) return 0;
  int c = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    int l = lo - 64 * w, h = hi - 64 * w;
    if (h < 0 || l > 63) continue;
    if (l < 0) l = 0;
    if (h > 63) h = 63;
    uint64_t m = (h == 63 ? ~0ull : ((1ull << (h + 1)) - 1ull)) & (~0ull << l);
    c += __popcll(x[w] & m);
  }
  return c;
}
template <int W>
__device__ __forceinline__ int popc_w(const uint64_t *x) {
  int c = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) c += __popcll(x[w]);
  return c;
}
template <int W>
__device__ __forceinline__ int lowest_bit(const uint64_t *x) {
#pragma unroll
  for (int w = 0; w < W; ++w)
    if (x[w]) return 64 * w + __ffsll((long long)x[w]) - 1;
  return -1;
}
template <int W>
__device__ __forceinline__ int second_bit(const uint64_t *x) {
  uint64_t y[W];
  bool cleared = false;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    y[w] = x[w];
    if (!cleared && y[w]) { y[w] &= y[w] - 1; cleared = true; }
  }
  return lowest_bit<W>(y);
}
__device__ __forceinline__ bool bit_at(const uint64_t *x, int p) { return (x[p >> 6] >> (p & 63)) & 1ull; }

__device__ __forceinline__ double g2(const Params &P, int i, int j, int k, int l) { return __ldg(P.eri + canon4(i, j, k, l)); }
__device__ __forceinline__ double g1(const Params &P, int i, int j) { return __ldg(P.one + tri64(i, j)); }

// ------------------------------------------------------------------------------------
// excitation screen
// ------------------------------------------------------------------------------------
template <int W>
__device__ __forceinline__ bool within_two(const Params &P, const uint64_t *a1, const uint64_t *a2, int64_t j) {
  int d = 0;
#pragma unroll
  for (int w = 0; w < W; ++w)
    d += __popcll(a1[w] ^ __ldg(P.e1 + j * W + w)) + __popcll(a2[w] ^ __ldg(P.e2 + j * W + w));
  return d <= 4;
}

// MODE 0: count neighbours into cnt[i]; MODE 1: write sorted lists at nbroff[i].
template <int W, int MODE>
__global__ void k_screen(Params P, int64_t *cnt) {
  int lane = threadIdx.x & 31;
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < P.nconf; i += nwarps) {
    uint64_t a1[W], a2[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { a1[w] = P.e1[i * W + w]; a2[w] = P.e2[i * W + w]; }
    int64_t n = 0;
    int64_t out = (MODE == 1) ? P.nbroff[i] : 0;
    for (int64_t j0 = 0; j0 < P.nconf; j0 += 32) {
      int64_t j = j0 + lane;
      bool ok = (j < P.nconf) && within_two<W>(P, a1, a2, j);
      unsigned b = __ballot_sync(0xffffffffu, ok);
      if (MODE == 1 && ok) P.nbr[out + n + __popc(b & ((1u << lane) - 1u))] = (int32_t)j;
      n += __popc(b);
    }
    if (MODE == 0 && lane == 0) cnt[i] = n;
  }
}

// per configuration: number of segments and segment-row slots
__global__ void k_seg_counts(int nconf, const int64_t *nbroff, const int64_t *sefoff, int64_t *nseg_i,
                             int64_t *nrow_i) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t nn = nbroff[i + 1] - nbroff[i];
  int64_t ns = (nn + PSOCI_SEG - 1) / PSOCI_SEG;
  nseg_i[i] = ns;
  nrow_i[i] = ns * (sefoff[i + 1] - sefoff[i]);
}

__global__ void k_seg_init(int nconf, const int64_t *nbroff, const int64_t *sefoff, const int64_t *segoff,
                           const int64_t *rowslot, int32_t *seg_cfg, int64_t *seg_k0, int32_t *seg_n,
                           int64_t *seg_rowoff) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t nn = nbroff[i + 1] - nbroff[i];
  int64_t s0 = segoff[i], ns = segoff[i + 1] - s0;
  int64_t nsef = sefoff[i + 1] - sefoff[i];
  for (int64_t s = 0; s < ns; ++s) {
    seg_cfg[s0 + s] = (int32_t)i;
    seg_k0[s0 + s] = nbroff[i] + s * PSOCI_SEG;
    int64_t left = nn - s * PSOCI_SEG;
    seg_n[s0 + s] = (int32_t)(left < PSOCI_SEG ? left : PSOCI_SEG);
    seg_rowoff[s0 + s] = rowslot[i] + s * nsef;
  }
}

// per configuration: exclusive scan over its segments of the per-row counts (in place),
// totals per SEF row into row_nnz
__global__ void k_seg_rowscan(int nconf, const int64_t *sefoff, const int64_t *segoff, const int64_t *seg_rowoff,
                              int64_t *seg_cnt, int64_t *row_nnz) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t nsef = sefoff[i + 1] - sefoff[i];
  for (int64_t r = 0; r < nsef; ++r) {
    int64_t run = 0;
    for (int64_t s = segoff[i]; s < segoff[i + 1]; ++s) {
      int64_t *p = seg_cnt + seg_rowoff[s] + r;
      int64_t v = *p;
      *p = run;
      run += v;
    }
    row_nnz[sefoff[i] + r] = run;
  }
}

// ------------------------------------------------------------------------------------
// per-pair set-up (one lane per neighbour)
// ------------------------------------------------------------------------------------
template <int W>
__device__ void pair_setup(const Params &P, int I, int J, PairInfo &pi, double *Kd) {
  int A = (J <= I) ? I : J, B = (J <= I) ? J : I;
  pi.A = A; pi.B = B; pi.swap = (J > I);
  pi.detA = P.detoff[A]; pi.detB = P.detoff[B];
  pi.colbase = P.sefoff[J];
  pi.nsefJ = (int)(P.sefoff[J + 1] - P.sefoff[J]);
  pi.nopenA = P.nopen[A]; pi.nopenB = P.nopen[B];
  pi.jsA = P.jsym[A]; pi.jsB = P.jsym[B];
  uint64_t e1A[W], e2A[W], e1B[W], e2B[W], im1[W], im2[W], jm1[W], jm2[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    e1A[w] = P.e1[(int64_t)A * W + w]; e2A[w] = P.e2[(int64_t)A * W + w];
    e1B[w] = P.e1[(int64_t)B * W + w]; e2B[w] = P.e2[(int64_t)B * W + w];
    im1[w] = e1A[w] & ~e1B[w]; im2[w] = e2A[w] & ~e2B[w];
    jm1[w] = e1B[w] & ~e1A[w]; jm2[w] = e2B[w] & ~e2A[w];
    pi.SA[w] = e1A[w] & ~e2A[w];
  }
  pi.v0 = 0.0; pi.v1 = 0.0;
  pi.iex0 = pi.iex1 = pi.jex0 = -1;
  int ni = popc_w<W>(im1) + popc_w<W>(im2);
  if (A == B) {
    pi.kind = K_DIAG;
    // processDiagExcitation (PsociHamiltonian.C:306-388)
    int sing[PSOCI_MAX_OPEN], ns = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t s = pi.SA[w];
      while (s && ns < PSOCI_MAX_OPEN) { sing[ns++] = 64 * w + __ffsll((long long)s) - 1; s &= s - 1; }
    }
    int mm = 1;
    for (int a = 1; a < ns; ++a)
      for (int b = 0; b < a; ++b) Kd[mm++] = g2(P, sing[a], sing[b], sing[b], sing[a]);
    double v = 0.0;
#pragma unroll
    for (int wi = 0; wi < W; ++wi) {
      uint64_t oi = e1A[wi];
      while (oi) {
        int ib = 64 * wi + __ffsll((long long)oi) - 1;
        oi &= oi - 1;
        int occi = 1 + (int)bit_at(e2A, ib);
        if (occi == 1) v += g1(P, ib, ib);
        else v += 2.0 * g1(P, ib, ib) + g2(P, ib, ib, ib, ib);
#pragma unroll
        for (int wj = 0; wj < W; ++wj) {
          uint64_t oj = e1A[wj];
          while (oj) {
            int jb = 64 * wj + __ffsll((long long)oj) - 1;
            oj &= oj - 1;
            if (jb >= ib) break;
            int ninj = occi * (1 + (int)bit_at(e2A, jb));
            if (ninj == 1) v += g2(P, ib, ib, jb, jb);
            else {
              double buf = 2.0 * g2(P, ib, ib, jb, jb);
              buf -= g2(P, ib, jb, ib, jb);
              if (ninj == 2) v += buf; else v += 2.0 * buf;
            }
          }
        }
      }
    }
    Kd[0] = v;
    pi.v0 = v;
    return;
  }
  if (ni == 1) {
    uint64_t im[W], jm[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { im[w] = im1[w] | im2[w]; jm[w] = jm1[w] | jm2[w]; }
    int ie = lowest_bit<W>(im), je = lowest_bit<W>(jm);
    pi.iex0 = ie; pi.jex0 = je;
    if (pi.jsA != pi.jsB) {
      // spin-orbit single (PsociHamiltonian.C:223-237): +-SO/2, sign flip if jex > iex
      double v = g1(P, ie, je);
      if (v != 0.0) {
        if (je > ie) v = -v;
        v = v / 2;
        pi.kind = K_SO;
        pi.v0 = v;
      } else {
        pi.kind = K_NONE;
      }
      return;
    }
    // same-symmetry single (PsociHamiltonian.C:239-258)
    double v = g1(P, ie, je) - g2(P, ie, je, ie, ie);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t o = e1A[w];
      while (o) {
        int p = 64 * w + __ffsll((long long)o) - 1;
        o &= o - 1;
        double buf = g2(P, ie, je, p, p);
        v += buf;
        bool dA = bit_at(e2A, p);
        if (dA) v += buf;
        if (dA && bit_at(e2B, p)) v -= g2(P, ie, p, p, je);
      }
    }
    if (v == 0.0) { pi.kind = K_NONE; return; }
    pi.kind = K_SINGLE;
    pi.v0 = v;
    int t = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t s = pi.SA[w];
      while (s && t < PSOCI_MAX_OPEN) {
        int p = 64 * w + __ffsll((long long)s) - 1;
        s &= s - 1;
        pi.X[t++] = g2(P, ie, p, p, je);
      }
    }
    return;
  }
  if (ni == 2) {
    // ascending with multiplicity: a position in both masks appears twice
    int ex[2], ney = 0, jy[2], nj = 0;
    for (int pass = 0; pass < 2; ++pass) {
      const uint64_t *m1 = pass == 0 ? im1 : jm1;
      const uint64_t *m2 = pass == 0 ? im2 : jm2;
      int *dst = pass == 0 ? ex : jy;
      int &nd = pass == 0 ? ney : nj;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        uint64_t u = m1[w] | m2[w];
        while (u && nd < 2) {
          int b = __ffsll((long long)u) - 1;
          u &= u - 1;
          int p = 64 * w + b;
          int mult = (int)((m1[w] >> b) & 1ull) + (int)((m2[w] >> b) & 1ull);
          for (int q = 0; q < mult && nd < 2; ++q) dst[nd++] = p;
        }
      }
    }
    pi.iex0 = ex[0]; pi.iex1 = ex[1]; pi.jex0 = jy[0];
    // processDoubleExcitation (PsociHamiltonian.C:180-184)
    double v0 = g2(P, ex[0], jy[0], ex[1], jy[1]);
    double v1 = g2(P, ex[0], jy[1], ex[1], jy[0]);
    if (v0 == 0.0 && v1 == 0.0) { pi.kind = K_NONE; return; }
    pi.kind = K_DOUBLE;
    pi.v0 = v0; pi.v1 = v1;
    return;
  }
  pi.kind = K_NONE;
}

// ------------------------------------------------------------------------------------
// determinant element <det a of A | H | det b of B>
// ------------------------------------------------------------------------------------
template <int W>
__device__ double det_elem(const Params &P, const PairInfo &pi, const double *Kd, int64_t da, int64_t db) {
  uint64_t aa[W], ba[W], ab[W], bb[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    aa[w] = __ldg(P.alpha + da * W + w); ba[w] = __ldg(P.beta + da * W + w);
    ab[w] = __ldg(P.alpha + db * W + w); bb[w] = __ldg(P.beta + db * W + w);
  }
  int pha = __ldg(P.phase + da), phb = __ldg(P.phase + db);
  int naa = __ldg(P.nalpha + da), nab = __ldg(P.nalpha + db);
  uint64_t ua[W], ub[W];
#pragma unroll
  for (int w = 0; w < W; ++w) { ua[w] = ab[w] & ~aa[w]; ub[w] = bb[w] & ~ba[w]; }
  int nmarka = popc_w<W>(ua);
  int nmarkb = nmarka + popc_w<W>(ub);
  const int ie = pi.iex0, je = pi.jex0;

  if (pi.kind == K_SO) {
    // socig (PsociHamiltonian.C:746-855): no spin-projection restriction
    if (nmarka > 1 || nmarkb > 1) return 0.0;
    int ncount = pha + phb;
    if (naa < nab) {
      ncount += popc_range<W>(ba, 0, ie - 1) + popc_range<W>(ab, je + 1, 64 * W - 1);
      if ((pi.jsA + pi.jsB) % 2 == 0) ++ncount;
      else if (pi.jsA % 2 == 1) ++ncount;
    } else if (naa > nab) {
      ncount += popc_range<W>(aa, ie + 1, 64 * W - 1) + popc_range<W>(bb, 0, je - 1);
      if ((pi.jsA + pi.jsB) % 2 != 0 && (pi.jsA % 2) == 1) ++ncount;
    } else {
      if (nmarka == 0) ++ncount;
      if (pi.jsA % 2 == 1) ++ncount;
      if (abs(ie - je) > 1) {
        int lo = min(ie, je) + 1, hi = max(ie, je) - 1;
        ncount += popc_range<W>(nmarka != 0 ? aa : ba, lo, hi);
      }
    }
    return (ncount & 1) ? -pi.v0 : pi.v0;
  }

  // generateSEFCIG (PsociHamiltonian.C:902-1113): equal spin projection only
  if (naa != nab) return 0.0;
  if (nmarka > 2 || nmarkb > 2) return 0.0;
  if (nmarkb == 0) {
    if (pi.kind != K_DIAG) return 0.0;  // identical determinants occur only on the diagonal
    double v = Kd[0];
    int sing[PSOCI_MAX_OPEN], ns = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t s = pi.SA[w];
      while (s && ns < PSOCI_MAX_OPEN) { sing[ns++] = 64 * w + __ffsll((long long)s) - 1; s &= s - 1; }
    }
    int mm = 0;
    for (int io = 1; io < ns; ++io) {
      bool si = bit_at(aa, sing[io]);
      for (int jo = 0; jo < io; ++jo) {
        ++mm;
        if (si == bit_at(aa, sing[jo])) v -= Kd[mm];
      }
    }
    return v;
  }
  if (nmarkb == 1) {
    // one spin-orbital excitation within spin (nmarka == 1: alpha, else beta)
    const uint64_t *sp = (nmarka != 0) ? aa : ba;
    int ncount = pha + phb;
    if (abs(ie - je) > 1) ncount += popc_range<W>(sp, min(ie, je) + 1, max(ie, je) - 1);
    double v = pi.v0;
    // exchange with the open shells of that spin in det a, except the excited orbitals
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t m = sp[w] & ~(aa[w] & ba[w]);
      if ((ie >> 6) == w) m &= ~(1ull << (ie & 63));
      if ((je >> 6) == w) m &= ~(1ull << (je & 63));
      while (m) {
        int b = __ffsll((long long)m) - 1;
        m &= m - 1;
        int p = 64 * w + b;
        int t = popc_range<W>(pi.SA, 0, p - 1);
        v -= pi.X[t];
      }
    }
    return (ncount & 1) ? -v : v;
  }
  if (nmarka == 1) {
    // alpha single times beta single
    uint64_t xa[W], xb[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { xa[w] = aa[w] & ~ab[w]; xb[w] = ba[w] & ~bb[w]; }
    int iex2 = lowest_bit<W>(ua), jex2 = lowest_bit<W>(ub);
    int iex3 = lowest_bit<W>(xa), jex3 = lowest_bit<W>(xb);
    int ncount = pha + phb;
    if (abs(iex2 - iex3) > 1) ncount += popc_range<W>(aa, min(iex2, iex3) + 1, max(iex2, iex3) - 1);
    if (abs(jex2 - jex3) > 1) ncount += popc_range<W>(ba, min(jex2, jex3) + 1, max(jex2, jex3) - 1);
    double v = g2(P, jex2, jex3, iex2, iex3);
    return (ncount & 1) ? -v : v;
  }
  // same-spin double (nmarka == 2: alpha, nmarka == 0: beta)
  if (pi.kind != K_DOUBLE) return 0.0;
  const uint64_t *spb = (nmarka == 2) ? ab : bb;
  const uint64_t *u = (nmarka == 2) ? ua : ub;
  int u0 = lowest_bit<W>(u), u1 = second_bit<W>(u);
  int ncount = pha + phb + popc_range<W>(spb, u0 + 1, u1 - 1);
  if (pi.iex1 - pi.iex0 > 1) ncount += popc_range<W>((nmarka != 0) ? aa : ba, pi.iex0 + 1, pi.iex1 - 1);
  double v = pi.v0 - pi.v1;
  return (ncount & 1) ? -v : v;
}

// SEF element (a, b) of the reference block (A, B): ciout / transformCDCt
template <int W>
__device__ double sef_elem(const Params &P, const PairInfo &pi, const double *Kd, int a, int b) {
  if (pi.kind == K_NONE) return 0.0;
  if (P.nelec & 1) return det_elem<W>(P, pi, Kd, pi.detA + a, pi.detB + b);
  const double r = sqrt(0.5);
  const bool oa = pi.nopenA != 0, ob = pi.nopenB != 0;
  const double mA = (pi.jsA % 2 != P.ksym % 2) ? -1.0 : 1.0;
  const double mB = (pi.jsB % 2 != P.ksym % 2) ? -1.0 : 1.0;
  int64_t a0 = pi.detA + (oa ? 2 * a : 0), a1 = a0 + 1;
  int64_t b0 = pi.detB + (ob ? 2 * b : 0), b1 = b0 + 1;
  double ds0, ds1 = 0.0;
  if (ob) {
    double t = det_elem<W>(P, pi, Kd, a0, b0);
    t += mB * det_elem<W>(P, pi, Kd, a0, b1);
    ds0 = t * r;
    if (oa) {
      double u = det_elem<W>(P, pi, Kd, a1, b0);
      u += mB * det_elem<W>(P, pi, Kd, a1, b1);
      ds1 = u * r;
    }
  } else {
    ds0 = det_elem<W>(P, pi, Kd, a0, b0);
    if (oa) ds1 = det_elem<W>(P, pi, Kd, a1, b0);
  }
  if (oa) {
    double t = r * ds0;
    t += (mA * r) * ds1;
    return t;
  }
  return ds0;
}

// ------------------------------------------------------------------------------------
// segment kernel: PASS 0 counts kept elements per row, PASS 1 writes them
// ------------------------------------------------------------------------------------
template <int W, int PASS>
__global__ void __launch_bounds__(WARPS_PER_CTA * 32) k_hbuild(Params P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem *ws = reinterpret_cast<WarpSmem *>(smem_raw) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t s = warp; s < P.nseg; s += nwarps) {
    const int I = P.seg_cfg[s];
    const int64_t k0 = P.seg_k0[s];
    const int n = P.seg_n[s];
    const int nsefI = (int)(P.sefoff[I + 1] - P.sefoff[I]);
    int myJ = -1, myn = 0;
    if (lane < n) {
      myJ = P.nbr[k0 + lane];
      pair_setup<W>(P, I, myJ, ws->pi[lane], ws->K);
      myn = ws->pi[lane].nsefJ;
    }
    // exclusive prefix of nsefJ over the segment
    int incl = myn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    ws->itemoff[lane + 1] = incl;
    if (lane == 0) ws->itemoff[0] = 0;
    __syncwarp();
    const int T = ws->itemoff[n];
    for (int r = 0; r < nsefI; ++r) {
      int64_t base = 0;
      if (PASS == 1) base = P.rowptr[P.sefoff[I] + r] + P.seg_cnt[P.seg_rowoff[s] + r];
      int64_t cnt = 0;
      for (int q0 = 0; q0 < T; q0 += 32) {
        const int q = q0 + lane;
        bool keep = false;
        double v = 0.0;
        int k = 0, t = 0;
        if (q < T) {
          // neighbour k with itemoff[k] <= q < itemoff[k+1]
          int lo = 0, hi = n - 1;
          while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (ws->itemoff[mid] <= q) lo = mid; else hi = mid - 1;
          }
          k = lo;
          t = q - ws->itemoff[k];
          const PairInfo &pi = ws->pi[k];
          bool diag_blk = (pi.kind == K_DIAG);
          if (diag_blk) {
            // lower half as computed by the reference, upper half mirrored
            v = (t <= r) ? sef_elem<W>(P, pi, ws->K, r, t) : sef_elem<W>(P, pi, ws->K, t, r);
            keep = (fabs(v) >= PSOCI_MIN_VALUE) || (t == r);
          } else {
            v = pi.swap ? sef_elem<W>(P, pi, ws->K, t, r) : sef_elem<W>(P, pi, ws->K, r, t);
            keep = fabs(v) >= PSOCI_MIN_VALUE;
          }
        }
        unsigned b = __ballot_sync(0xffffffffu, keep);
        if (PASS == 1 && keep) {
          int64_t pos = base + cnt + __popc(b & ((1u << lane) - 1u));
          const PairInfo &pi = ws->pi[k];
          P.col[pos] = (int32_t)(pi.colbase + t);
          P.val[pos] = v;
          if (P.val32) P.val32[pos] = (float)v;
          if (pi.kind == K_DIAG && t == r) P.diag[P.sefoff[I] + r] = v;
        }
        cnt += __popc(b);
      }
      if (PASS == 0 && lane == 0) P.seg_cnt[P.seg_rowoff[s] + r] = cnt;
    }
    __syncwarp();
  }
}

template <int W>
psoci_status run_build(psoci_ctx *c, psoci_hmode mode, int64_t *nnz_out) {
  cudaStream_t st = c->stream;
  const int n = c->nconf;
  Params P = {};
  P.nconf = n; P.nbf = c->nbf; P.nelec = c->nelec; P.ksym = c->ksym;
  P.e1 = c->d_e1; P.e2 = c->d_e2; P.jsym = c->d_jsym; P.nopen = c->d_nopen;
  P.sefoff = c->d_sefoff; P.detoff = c->d_detoff;
  P.alpha = c->d_alpha; P.beta = c->d_beta; P.phase = c->d_phase; P.nalpha = c->d_nalpha;
  P.one = c->d_one; P.eri = c->d_eri;

  psoci_status s;
  int64_t *d_cnt = nullptr, *d_nbroff = nullptr, *d_nseg = nullptr, *d_nrow = nullptr, *d_segoff = nullptr,
          *d_rowslot = nullptr, *d_segk0 = nullptr, *d_segrow = nullptr, *d_segcnt = nullptr, *d_rownnz = nullptr;
  int32_t *d_nbr = nullptr, *d_segcfg = nullptr, *d_segn = nullptr;
  auto cleanup = [&]() {
    psoci_free(d_cnt); psoci_free(d_nbroff); psoci_free(d_nseg); psoci_free(d_nrow); psoci_free(d_segoff);
    psoci_free(d_rowslot); psoci_free(d_segk0); psoci_free(d_segrow); psoci_free(d_segcnt); psoci_free(d_rownnz);
    psoci_free(d_nbr); psoci_free(d_segcfg); psoci_free(d_segn);
  };
#define TRY(x)                 \
  do {                         \
    s = (x);                   \
    if (s != PSOCI_OK) {       \
      cleanup();               \
      return s;                \
    }                          \
  } while (0)
#define TRYC(x)                                  \
  do {                                          \
    cudaError_t _e = (x);                       \
    if (_e != cudaSuccess) {                    \
      s = psoci_cuda_fail(c, _e, #x);           \
      cleanup();                                \
      return s;                                 \
    }                                           \
  } while (0)

  const int warp_threads = 256;
  const int blocks_cfg = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n * 32 + warp_threads - 1) / warp_threads, 152 * 32));
  // 1. screen
  TRY(psoci_alloc(c, &d_cnt, n + 1));
  TRY(psoci_alloc(c, &d_nbroff, n + 1));
  k_screen<W, 0><<<blocks_cfg, warp_threads, 0, st>>>(P, d_cnt);
  TRYC(cudaGetLastError());
  int64_t npairs = 0;
  TRY(psoci_scan_i64(c, d_cnt, d_nbroff, n, &npairs));
  TRY(psoci_alloc(c, &d_nbr, npairs));
  P.nbroff = d_nbroff; P.nbr = d_nbr;
  k_screen<W, 1><<<blocks_cfg, warp_threads, 0, st>>>(P, nullptr);
  TRYC(cudaGetLastError());
  c->npairs = npairs;

  // 2. segments
  TRY(psoci_alloc(c, &d_nseg, n + 1));
  TRY(psoci_alloc(c, &d_nrow, n + 1));
  TRY(psoci_alloc(c, &d_segoff, n + 1));
  TRY(psoci_alloc(c, &d_rowslot, n + 1));
  k_seg_counts<<<(n + 255) / 256, 256, 0, st>>>(n, d_nbroff, c->d_sefoff, d_nseg, d_nrow);
  TRYC(cudaGetLastError());
  int64_t nseg = 0, nslots = 0;
  TRY(psoci_scan_i64(c, d_nseg, d_segoff, n, &nseg));
  TRY(psoci_scan_i64(c, d_nrow, d_rowslot, n, &nslots));
  TRY(psoci_alloc(c, &d_segcfg, nseg));
  TRY(psoci_alloc(c, &d_segk0, nseg));
  TRY(psoci_alloc(c, &d_segn, nseg));
  TRY(psoci_alloc(c, &d_segrow, nseg));
  TRY(psoci_alloc(c, &d_segcnt, nslots));
  k_seg_init<<<(n + 255) / 256, 256, 0, st>>>(n, d_nbroff, c->d_sefoff, d_segoff, d_rowslot, d_segcfg, d_segk0, d_segn,
                                              d_segrow);
  TRYC(cudaGetLastError());
  c->nseg = nseg;
  P.nseg = nseg; P.seg_cfg = d_segcfg; P.seg_k0 = d_segk0; P.seg_n = d_segn; P.seg_rowoff = d_segrow;
  P.seg_cnt = d_segcnt;

  // 3. count
  const size_t smem = sizeof(WarpSmem) * WARPS_PER_CTA;
  TRYC(cudaFuncSetAttribute(k_hbuild<W, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  TRYC(cudaFuncSetAttribute(k_hbuild<W, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int hb_blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nseg + WARPS_PER_CTA - 1) / WARPS_PER_CTA, 152 * 16));
  k_hbuild<W, 0><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
  TRYC(cudaGetLastError());

  // 4. offsets
  const int64_t N = c->nsef_total;
  TRY(psoci_alloc(c, &d_rownnz, N + 1));
  k_seg_rowscan<<<(n + 127) / 128, 128, 0, st>>>(n, c->d_sefoff, d_segoff, d_segrow, d_segcnt, d_rownnz);
  TRYC(cudaGetLastError());
  TRY(psoci_alloc(c, &c->d_rowptr, N + 1));
  int64_t nnz = 0;
  TRY(psoci_scan_i64(c, d_rownnz, c->d_rowptr, N, &nnz));
  TRY(psoci_alloc(c, &c->d_col, nnz));
  TRY(psoci_alloc(c, &c->d_val, nnz));
  if (mode == PSOCI_HMODE_CSR_BOTH) TRY(psoci_alloc(c, &c->d_val32, nnz));
  TRY(psoci_alloc(c, &c->d_diag, N));
  P.rowptr = c->d_rowptr; P.col = c->d_col; P.val = c->d_val; P.val32 = c->d_val32; P.diag = c->d_diag;

  // 5. fill
  k_hbuild<W, 1><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
  TRYC(cudaGetLastError());
  TRYC(cudaStreamSynchronize(st));
  cleanup();
  c->nnz = nnz;
  *nnz_out = nnz;
  return PSOCI_OK;
#undef TRY
#undef TRYC
}

}  // namespace

void psoci_h_release(psoci_ctx *c) {
  psoci_free(c->d_rowptr);
  psoci_free(c->d_col);
  psoci_free(c->d_val);
  psoci_free(c->d_val32);
  psoci_free(c->d_diag);
  c->have_h = false;
  c->nnz = 0;
}

psoci_status psoci_h_build(psoci_ctx *c, psoci_hmode mode, int64_t *nnz) {
  if (!c->have_ints) return psoci_fail(c, PSOCI_ERR_STATE, "psoci_build_hamiltonian: no integrals set");
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "psoci_build_hamiltonian: determinants not built");
  if (c->nbf != 0 && c->n1 != (int64_t)c->nbf * (c->nbf + 1) / 2)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "integral and configuration orbital counts differ");
  psoci_h_release(c);
  auto t0 = std::chrono::steady_clock::now();
  psoci_status s = (c->words == 1) ? run_build<1>(c, mode, nnz) : run_build<2>(c, mode, nnz);
  if (s != PSOCI_OK) {
    psoci_h_release(c);
    return s;
  }
  c->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  c->have_h = true;
  if (c->verbose)
    fprintf(stderr, "psoci: H build N=%lld nnz=%lld pairs=%lld segments=%lld %.3f s\n", (long long)c->nsef_total,
            (long long)c->nnz, (long long)c->npairs, (long long)c->nseg, c->build_seconds);
  return PSOCI_OK;
}
