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
// lower-triangle value: only the blocks (I, J <= I) are evaluated, as the reference does,
// and the upper half of the matrix is their mirror image.  Rows are written in ascending
// column order, deterministically:
//
//   1. screen:   per configuration, the sorted list of configurations within two
//                excitations (XOR + popcount on occupancy bit-planes), then the blocks
//                that the integrals alone make zero are dropped;
//   2. segments: the lower neighbours (J <= I) of each row configuration in groups of <= 32,
//                one warp each;
//   3. evaluate: each warp marks the SEF elements that determinant connectivity allows and
//                evaluates them; kept values go to slab slots, per (pair, row SEF) a mask of
//                kept columns (fast path, <= 32 determinants per configuration);
//   4. rows:     full row lengths = lower counts + the mirrored columns of upper neighbours;
//   5. assemble: columns and values in order, the FP32 copy and the diagonal.
//
// Configurations with more than 32 determinants (7-11 open shells) take the generic path:
// every block (I, J) of the full neighbour list is evaluated in a count pass and again in
// a fill pass (a block with J > I as the reference's block (J, I), transposed).
//
// Floating point follows the reference's operation order; this file is compiled with
// --fmad=false so products and sums round as the reference's do.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <functional>
#include <queue>
#include <vector>

#include "psoci_internal.cuh"

namespace {

enum { K_NONE = 0, K_DIAG = 1, K_SINGLE = 2, K_DOUBLE = 3, K_SO = 4 };

constexpr int WARPS_PER_CTA = 4;
constexpr int MAXK = 1 + PSOCI_MAX_OPEN * (PSOCI_MAX_OPEN - 1) / 2;  // diagonal vnt list

struct PairInfo {
  int64_t detA, detB;   // first determinant of A, B
  int64_t colbase;      // first SEF of the neighbour J
  int kind, swap;       // swap: J > I, element (t, r) of block (J, I)
  int iex0, jex0;       // single excitations: the orbital A -> B
  int nopenA, nopenB, jsA, jsB, nsefJ;
  double v0, v1;
  double X[PSOCI_MAX_OPEN];  // single: (iex0 s|s jex0) over the open shells s of A
  uint64_t SA[PSOCI_MAX_WORDS];  // open shells of A
  // orbital ranges the determinant phases count electrons over, fixed for the pair:
  //   K_DOUBLE: 0-3 strictly between ex_i and jy_j (index 2i + j), 4 between ex0 and ex1,
  //             5 between jy0 and jy1;
  //   K_SINGLE, K_SO: 0 strictly between ie and je, 1 below ie, 2 above je, 3 below je,
  //             4 above ie
  uint64_t bm[6][PSOCI_MAX_WORDS];
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
  int64_t nbr_len;         // entries of nbr
  // segments
  int64_t nseg;
  const int32_t *seg_cfg;
  const int64_t *seg_k0;
  const int32_t *seg_n;
  const int64_t *seg_rowoff;
  int64_t *seg_cnt;        // count pass output / fill pass row offsets (local)
  // single-pass fast build over the lower pairs (J <= I): kept values are appended to slab
  // slots; per (pair, row SEF) a mask of kept columns and the pair's offset in the slot
  const int64_t *segoff;   // first segment of each configuration
  const int64_t *nlow;     // neighbours J <= I
  const int64_t *pr_off;   // first (pair, row) mask of each configuration
  uint64_t *prm;           // bits 0-15: kept column SEFs t; bits 16-63: slab position of the first
                           // of them (the pair's values in the row run follow one another)
  unsigned long long *slab_counter;
  int64_t slab_cap;
  double *slab_val;
  uint64_t *cg;            // connectivity masks C[r] per (pair, row SEF), as prm (two-launch evaluation)
  const int64_t *rowptr;
  int32_t *col;
  double *val;
  float *val32;
  double *diag;
  // direct sigma (PASS 2): Y[:, 0:kvec] += H X[:, 0:kvec]; with dx32 (the inputs in FP32,
  // 8 per row) the products are FP32 element x FP32 input with compensated FP32 sums
  const float *dx32;
  const double *dx;
  double *dy;
  int ldx, ldy, kvec;
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
// bits lo..hi inclusive (none when lo > hi) over W words
template <int W>
__device__ __forceinline__ void range_mask(int lo, int hi, uint64_t *m) {
#pragma unroll
  for (int w = 0; w < W; ++w) {
    int l = lo - 64 * w, h = hi - 64 * w;
    if (lo > hi || h < 0 || l > 63) { m[w] = 0ull; continue; }
    if (l < 0) l = 0;
    if (h > 63) h = 63;
    m[w] = (h == 63 ? ~0ull : ((1ull << (h + 1)) - 1ull)) & (~0ull << l);
  }
}
// orbitals strictly between a and b
template <int W>
__device__ __forceinline__ void between_mask(int a, int b, uint64_t *m) {
  range_mask<W>(min(a, b) + 1, max(a, b) - 1, m);
}
template <int W>
__device__ __forceinline__ int popc_and(const uint64_t *x, const uint64_t *m) {
  int c = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) c += __popcll(x[w] & m[w]);
  return c;
}

// register-array forms: word selection by value, so that the arrays stay in registers
template <int W>
__device__ __forceinline__ bool bit_w(const uint64_t (&x)[W], int p) {
  uint64_t v = x[0];
#pragma unroll
  for (int w = 1; w < W; ++w)
    if ((p >> 6) == w) v = x[w];
  return (v >> (p & 63)) & 1ull;
}
template <int W>
__device__ __forceinline__ void sel_w(uint64_t (&d)[W], bool c, const uint64_t (&a)[W], const uint64_t (&b)[W]) {
#pragma unroll
  for (int w = 0; w < W; ++w) d[w] = c ? a[w] : b[w];
}

__device__ __forceinline__ double g2(const Params &P, int i, int j, int k, int l) { return __ldg(P.eri + canon4(i, j, k, l)); }
__device__ __forceinline__ double g1(const Params &P, int i, int j) { return __ldg(P.one + tri64(i, j)); }

// ------------------------------------------------------------------------------------
// excitation screen
// ------------------------------------------------------------------------------------
// Excitation orbitals between occupations A and B, ascending with multiplicity:
// A has more electrons than B in iex, fewer in jex (generateSOCIblocks, PsociHamiltonian.C:496-512).
template <int W>
__device__ __forceinline__ int excitation(const uint64_t *e1A, const uint64_t *e2A, const uint64_t *e1B,
                                          const uint64_t *e2B, int *ex, int *jy) {
  int ni = 0, nj = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    uint64_t i1 = e1A[w] & ~e1B[w], i2 = e2A[w] & ~e2B[w];
    uint64_t j1 = e1B[w] & ~e1A[w], j2 = e2B[w] & ~e2A[w];
    uint64_t u = i1 | i2;
    while (u) {
      int b = __ffsll((long long)u) - 1;
      u &= u - 1;
      int mult = (int)((i1 >> b) & 1ull) + (int)((i2 >> b) & 1ull);
      for (int q = 0; q < mult; ++q) { if (ni < 2) ex[ni] = 64 * w + b; ++ni; }
    }
    u = j1 | j2;
    while (u) {
      int b = __ffsll((long long)u) - 1;
      u &= u - 1;
      int mult = (int)((j1 >> b) & 1ull) + (int)((j2 >> b) & 1ull);
      for (int q = 0; q < mult; ++q) { if (nj < 2) jy[nj] = 64 * w + b; ++nj; }
    }
  }
  return ni;
}

// The same, with the first two positions of each side returned in registers (no local
// arrays): ex0 <= ex1 removed from A, jy0 <= jy1 added in B, -1 where absent.
template <int W>
__device__ __forceinline__ int excitation_r(const uint64_t *e1A, const uint64_t *e2A, const uint64_t *e1B,
                                            const uint64_t *e2B, int &ex0, int &ex1, int &jy0, int &jy1) {
  int ni = 0, nj = 0;
  ex0 = ex1 = jy0 = jy1 = -1;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const uint64_t i1 = e1A[w] & ~e1B[w], i2 = e2A[w] & ~e2B[w];
    const uint64_t j1 = e1B[w] & ~e1A[w], j2 = e2B[w] & ~e2A[w];
    uint64_t u = i1 | i2;
    while (u) {
      const int b = __ffsll((long long)u) - 1;
      u &= u - 1;
      const int p = 64 * w + b;
      const int both = (int)((i1 >> b) & (i2 >> b) & 1ull);
      if (ni == 0) { ex0 = p; if (both) ex1 = p; }
      else if (ni == 1) ex1 = p;
      ni += 1 + both;
    }
    u = j1 | j2;
    while (u) {
      const int b = __ffsll((long long)u) - 1;
      u &= u - 1;
      const int p = 64 * w + b;
      const int both = (int)((j1 >> b) & (j2 >> b) & 1ull);
      if (nj == 0) { jy0 = p; if (both) jy1 = p; }
      else if (nj == 1) jy1 = p;
      nj += 1 + both;
    }
  }
  return ni;
}

// Screen, stage 1: configurations within two excitations of i (sum |occ_i - occ_j| <= 4,
// the orbmap test of PsociGADeterminants.C:2249-2277).  One thread per row configuration;
// tiles of column configurations are staged in shared memory and read by broadcast, so each
// thread's candidate list comes out sorted.  blockIdx.y selects a contiguous range of
// column configurations [y*chunk, (y+1)*chunk) so small problems still fill the GPU; MODE 0
// counts per (range, row), MODE 1 writes each range's candidates after the earlier ranges'.
constexpr int SCR_THREADS = 256;
constexpr int SCR_TILE = 512;
constexpr int SCR_ROWS = 4;  // row configurations per thread: one shared-memory load serves four tests

template <int W, int MODE>
__global__ void __launch_bounds__(SCR_THREADS) k_screen(Params P, int64_t *cnt, const int64_t *soff, int64_t chunk,
                                                        const int64_t *candoff, int32_t *cand) {
  __shared__ uint64_t t1[SCR_TILE * W], t2[SCR_TILE * W];
  uint64_t a1[SCR_ROWS][W], a2[SCR_ROWS][W];
  int64_t n[SCR_ROWS], out[SCR_ROWS];
  bool act[SCR_ROWS];
#pragma unroll
  for (int q = 0; q < SCR_ROWS; ++q) {
    const int64_t i = (int64_t)blockIdx.x * (SCR_THREADS * SCR_ROWS) + q * SCR_THREADS + threadIdx.x;
    act[q] = i < P.nconf;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      a1[q][w] = act[q] ? P.e1[i * W + w] : ~0ull;  // inactive rows match nothing
      a2[q][w] = act[q] ? P.e2[i * W + w] : ~0ull;
    }
    n[q] = 0;
    out[q] = (MODE == 1 && act[q]) ? candoff[i] + soff[(int64_t)blockIdx.y * P.nconf + i] : 0;
  }
  const int64_t jbeg = (int64_t)blockIdx.y * chunk;
  const int64_t jend = min((int64_t)P.nconf, jbeg + chunk);
  for (int64_t j0 = jbeg; j0 < jend; j0 += SCR_TILE) {
    const int nt = (int)min((int64_t)SCR_TILE, jend - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt * W; e += SCR_THREADS) {
      t1[e] = P.e1[j0 * W + e];
      t2[e] = P.e2[j0 * W + e];
    }
    __syncthreads();
    for (int jj = 0; jj < nt; ++jj) {
      uint64_t b1[W], b2[W];
#pragma unroll
      for (int w = 0; w < W; ++w) { b1[w] = t1[jj * W + w]; b2[w] = t2[jj * W + w]; }
#pragma unroll
      for (int q = 0; q < SCR_ROWS; ++q) {
        int d = __popcll(a1[q][0] ^ b1[0]) + __popcll(a2[q][0] ^ b2[0]);
#pragma unroll
        for (int w = 1; w < W; ++w)
          if (d <= 4) d += __popcll(a1[q][w] ^ b1[w]) + __popcll(a2[q][w] ^ b2[w]);
        if (d <= 4 && act[q]) {
          if (MODE == 1) cand[out[q] + n[q]] = (int32_t)(j0 + jj);
          ++n[q];
        }
      }
    }
  }
  if (MODE == 0) {
#pragma unroll
    for (int q = 0; q < SCR_ROWS; ++q) {
      const int64_t i = (int64_t)blockIdx.x * (SCR_THREADS * SCR_ROWS) + q * SCR_THREADS + threadIdx.x;
      if (act[q]) cnt[(int64_t)blockIdx.y * P.nconf + i] = n[q];
    }
  }
}

// A double-excitation block (PsociHamiltonian.C:180-185) has determinant elements +-v0,
// +-v1 or +-(v0 - v1) with v0 = (i0 j0|i1 j1), v1 = (i0 j1|i1 j0), and each SEF element
// combines at most four of them with weights +-1/2, so |element| <= 2 (|v0| + |v1|) (plus
// rounding of a few ulps).  With |v0| + |v1| < 4e-9 every element is below the 1e-8 that
// packSefsef stores (PsociGAhamiltonian.C:4077-4136): the block adds nothing to H and is
// not evaluated.  This includes the blocks the reference skips outright (v0 = v1 = 0).
__device__ __forceinline__ bool double_block_kept(double v0, double v1) { return fabs(v0) + fabs(v1) >= 4e-9; }

// Screen, stage 2: drop candidates whose block stores nothing, judged from its integral
// prefactors alone — double excitations as above and spin-orbit singles with SO_ij = 0
// (PsociHamiltonian.C:227); both tests are symmetric in (i, j).  One warp per row configuration, candidates in order, ballot
// compaction; MODE 0 counts, MODE 1 writes.
template <int W, int MODE>
__global__ void k_prune(Params P, const int64_t *candoff, const int32_t *cand, int64_t *cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < P.nconf; i += nwarps) {
    uint64_t a1[W], a2[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { a1[w] = P.e1[i * W + w]; a2[w] = P.e2[i * W + w]; }
    const int js_i = P.jsym[i];
    const int64_t c0 = candoff[i], c1 = candoff[i + 1];
    int64_t n = 0;
    const int64_t out = (MODE == 1) ? P.nbroff[i] : 0;
    for (int64_t t0 = c0; t0 < c1; t0 += 32) {
      const int64_t t = t0 + lane;
      bool keep = false;
      int32_t j = 0;
      if (t < c1) {
        j = cand[t];
        keep = true;
        if (j != i) {
          uint64_t b1[W], b2[W];
#pragma unroll
          for (int w = 0; w < W; ++w) { b1[w] = __ldg(P.e1 + (int64_t)j * W + w); b2[w] = __ldg(P.e2 + (int64_t)j * W + w); }
          int ex[2], jy[2];
          int ni = (j <= i) ? excitation<W>(a1, a2, b1, b2, ex, jy) : excitation<W>(b1, b2, a1, a2, ex, jy);
          if (ni == 2) {
            keep = double_block_kept(__ldg(P.eri + canon4(ex[0], jy[0], ex[1], jy[1])),
                                     __ldg(P.eri + canon4(ex[0], jy[1], ex[1], jy[0])));
          } else if (ni == 1 && __ldg(P.jsym + j) != js_i) {
            keep = __ldg(P.one + tri64(ex[0], jy[0])) != 0.0;
          }
        }
      }
      const unsigned b = __ballot_sync(0xffffffffu, keep);
      if (MODE == 1 && keep) P.nbr[out + n + __popc(b & ((1u << lane) - 1u))] = j;
      n += __popc(b);
    }
    if (MODE == 0 && lane == 0) cnt[i] = n;
  }
}

// ------------------------------------------------------------------------------------
// Screen by lookup ("split join").  With the orbitals split at s so that every
// configuration holds at most two electrons in the orbitals >= s, a configuration is a
// (hi pattern g, lo pattern l) pair and its distance to another is d_hi + d_lo.  Any two
// hi patterns of <= 2 electrons are within 4, so the neighbours of i are, for every hi
// pattern h, the configurations T[h][l'] with d_lo(l_i, l') <= 4 - d_hi(g_i, h): one lookup
// when the hi patterns are disjoint, a short list otherwise — work in proportion to the
// neighbours instead of to all pairs.  Configurations are numbered in (g, l) order (checked
// when the tables are built), so scanning h and then l' in ascending order yields sorted
// lists.  The integral-based pruning of k_prune is applied to each candidate on the spot.
// One warp per row configuration, one lane per hi pattern; MODE 0 counts (kept and all
// candidates), MODE 1 writes the kept neighbours at off[i].
// ------------------------------------------------------------------------------------
struct JoinTabs {
  int s, G, L;
  const int32_t *gid, *lid, *T, *lnoff, *ln, *hdec;
  const uint32_t *lokey;
  const int64_t *goff;    // per hi pattern g: its list of hi patterns h to visit ...
  const uint32_t *glist;  // ... h | d_hi(g, h) << 28, ascending h
  const uint32_t *dkept;  // double_block_kept of (ex0 <= ex1) -> (jy0 <= jy1), bit tri(ex)*NT + tri(jy)
  int64_t nt;             // NT = nbf(nbf+1)/2
};

// The pruning decision of every double excitation, as bits: word q holds the pairs
// (a, b), a = tri(ex0, ex1), b = tri(jy0, jy1), with a * NT + b in [32q, 32q + 32).  The
// same integrals and test as the per-candidate form, so the same decisions.
__global__ void k_double_kept(int64_t nt, const int2 *__restrict__ pairs, const double *__restrict__ eri,
                              uint32_t *bits) {
  const int64_t nwords = (nt * nt + 31) / 32;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nwords; q += (int64_t)gridDim.x * blockDim.x) {
    uint32_t w = 0u;
    for (int u = 0; u < 32; ++u) {
      const int64_t e = q * 32 + u;
      if (e >= nt * nt) break;
      const int2 x = pairs[e / nt], y = pairs[e % nt];  // (ex0, ex1), (jy0, jy1), ascending
      const bool k = double_block_kept(__ldg(eri + canon4(x.x, y.x, x.y, y.y)), __ldg(eri + canon4(x.x, y.y, x.y, y.x)));
      w |= (uint32_t)k << u;
    }
    bits[q] = w;
  }
}

template <int W>
__device__ __forceinline__ void set_bit_w(uint64_t (&x)[W], int p) {
#pragma unroll
  for (int w = 0; w < W; ++w)
    if ((p >> 6) == w) x[w] |= 1ull << (p & 63);
}

// occupancy bit-planes of hi pattern code (kind 0: empty, 1: one electron in a, 2: one
// each in a < b, 3: two in a; positions relative to s)
template <int W>
__device__ __forceinline__ void hi_bits(int code, int s, uint64_t (&e1)[W], uint64_t (&e2)[W]) {
#pragma unroll
  for (int w = 0; w < W; ++w) e1[w] = e2[w] = 0ull;
  const int kind = code & 3, a = (code >> 8) & 0xfff, b = (code >> 20) & 0xfff;
  if (kind != 0) set_bit_w<W>(e1, s + a);
  if (kind == 3) set_bit_w<W>(e2, s + a);
  if (kind == 2) set_bit_w<W>(e1, s + b);
}

// electrons of hi pattern code: 0, 1, 2, 2 for kinds 0-3
__device__ __forceinline__ int hi_electrons(int code) { return min(code & 3, 2); }

// Hi-pattern lists.  For d_hi(g, h) = 4 the lo patterns must be equal, so the pair is a
// double excitation between the hi orbitals alone and whether its block survives the
// integral test (double_block_kept) depends on (g, h) only — it is decided here once
// instead of once per configuration pair.  The list of g keeps every h with d_hi < 4 and
// the h with d_hi = 4 whose block survives.  One warp per g, lanes over h; MODE 0 counts,
// MODE 1 writes (ascending h).
template <int W, int MODE>
__global__ void k_group_lists(JoinTabs J, const double *__restrict__ eri, int64_t *gcnt, uint32_t *glist) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = warp; g < J.G; g += nwarps) {
    uint64_t g1[W], g2[W];
    hi_bits<W>(J.hdec[g], J.s, g1, g2);
    int64_t n = 0;
    const int64_t out = (MODE == 1) ? J.goff[g] : 0;
    for (int h0 = 0; h0 < J.G; h0 += 32) {
      const int h = h0 + lane;
      bool take = false;
      int d = 0;
      if (h < J.G) {
        uint64_t b1[W], b2[W];
        hi_bits<W>(J.hdec[h], J.s, b1, b2);
#pragma unroll
        for (int w = 0; w < W; ++w) d += __popcll(g1[w] ^ b1[w]) + __popcll(g2[w] ^ b2[w]);
        take = true;
        if (d == 4) {
          int ex[2], jy[2];
          const int ni = excitation<W>(g1, g2, b1, b2, ex, jy);
          take = (ni == 2) && double_block_kept(__ldg(eri + canon4(ex[0], jy[0], ex[1], jy[1])),
                                                __ldg(eri + canon4(ex[0], jy[1], ex[1], jy[0])));
        }
      }
      const unsigned b = __ballot_sync(0xffffffffu, take);
      if (MODE == 1 && take) glist[out + n + __popc(b & ((1u << lane) - 1u))] = (uint32_t)h | ((uint32_t)d << 28);
      n += __popc(b);
    }
    if (MODE == 0 && lane == 0) gcnt[g] = n;
  }
}

// Slab of the single-pass join (MODE 2): each warp appends the neighbour lists of its
// configurations to chunks it takes from a shared counter; a configuration's list stays
// contiguous (a list outgrowing its chunk moves to a fresh one).  Positions at or beyond
// cap are not touched; the host sees the counter and falls back to count + write passes.
struct JoinSlab {
  int32_t *list;
  unsigned long long *counter;
  int64_t cap;
  int64_t *start;  // [nconf] slab position of each configuration's list
};
constexpr int JOIN_CHUNK = 4096;

template <int W, int MODE>
__global__ void __launch_bounds__(256) k_join(Params P, JoinTabs J, int64_t *cnt, int64_t *ncand, const int64_t *off,
                                              JoinSlab S) {
  __shared__ int s_pre[8][33], s_q0[8][32], s_lp[8][32], s_h[8][32];
  __shared__ uint32_t s_hx[8][32];  // per hi pattern: its part of the excitation from i (see below)
  __shared__ int s_hn[8][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t lomask = (1u << J.s) - 1u;
  unsigned long long cursor = 0, chunk_end = 0;  // MODE 2: this warp's slab chunk
  for (int64_t i = warp; i < P.nconf; i += nwarps) {
    const int li = J.lid[i], js_i = P.jsym[i], gi = J.gid[i];
    const int ne_i = hi_electrons(J.hdec[gi]);
    // the excitation i -> j splits into its lo part (orbitals < s, from the two lo keys) and
    // its hi part (from the two hi patterns, once per hi pattern); orbitals ascend, so the lo
    // orbitals come first in each list
    uint64_t g1[W], g2[W];
    hi_bits<W>(J.hdec[gi], J.s, g1, g2);
    const uint32_t keyi = J.lokey[li], e1i = keyi & lomask, e2i = keyi >> J.s;
    int64_t nk = 0, nc = 0;
    int64_t base = (MODE == 1) ? off[i] : 0;
    unsigned long long lstart = cursor;  // MODE 2: where this configuration's list begins
    const int64_t gl0 = J.goff[gi], gl1 = J.goff[gi + 1];
    for (int64_t h0 = gl0; h0 < gl1; h0 += 32) {
      // this lane's hi pattern h: the lo patterns l' with d_lo <= 4 - d_hi and the electron
      // count that h leaves, as a range of the neighbour list of l_i (or l_i alone when the
      // hi patterns are disjoint: those blocks passed the integral test when the list was
      // built)
      int h = 0;
      int len = 0, q0 = 0, lp0 = li;
      if (h0 + lane < gl1) {
        const uint32_t ent = J.glist[h0 + lane];
        h = (int)(ent & 0x0fffffffu);
        const int d = (int)(ent >> 28);
        const int tau = 4 - d;
        const int code = J.hdec[h];
        const int k = ne_i - hi_electrons(code) + 2;  // lo electrons of l' minus l_i's, + 2
        if (tau <= 0) { len = (k == 2); q0 = -1; }
        else {
          const int64_t at = (int64_t)(tau - 1) * (5 * (int64_t)J.L + 1) + 5 * (int64_t)li + k;
          q0 = J.lnoff[at];
          len = J.lnoff[at + 1] - q0;
          // hi part: the electrons leaving g_i (the first two, ascending, with multiplicity)
          // and their count, the first two arriving in h; 8 bits per orbital
          uint64_t b1[W], b2[W];
          hi_bits<W>(code, J.s, b1, b2);
          int x0, x1, y0, y1;
          s_hn[wib][lane] = excitation_r<W>(g1, g2, b1, b2, x0, x1, y0, y1);
          s_hx[wib][lane] = (uint32_t)(x0 & 0xff) | ((uint32_t)(x1 & 0xff) << 8) | ((uint32_t)(y0 & 0xff) << 16) |
                            ((uint32_t)(y1 & 0xff) << 24);
        }
      }
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int tot = __shfl_sync(0xffffffffu, incl, 31);
      s_pre[wib][lane] = incl - len;
      s_q0[wib][lane] = q0;
      s_lp[wib][lane] = lp0;
      s_h[wib][lane] = h;
      __syncwarp();
      // the chunk's lookups, spread evenly over the lanes in (h, l') order
      for (int e0 = 0; e0 < tot; e0 += 32) {
        const int e = e0 + lane;
        bool found = false, keep = false;
        int j = -1;
        if (e < tot) {
          int o = 0;
#pragma unroll
          for (int st = 16; st > 0; st >>= 1)
            if (s_pre[wib][o + st] <= e) o += st;
          const int qo = s_q0[wib][o], ho = s_h[wib][o];
          const int lp = (qo < 0) ? s_lp[wib][o] : J.ln[qo + (e - s_pre[wib][o])];
          j = J.T[(int64_t)lp * J.G + ho];
          if (j >= 0) {
            found = true;
            keep = true;
            if (j != (int)i && qo >= 0) {
              // lo part from the keys (bit q: orbital q occupied; bit s + q: doubly)
              const uint32_t key = J.lokey[lp], e1j = key & lomask, e2j = key >> J.s;
              const uint32_t i1 = e1i & ~e1j, i2 = e2i & ~e2j, j1 = e1j & ~e1i, j2 = e2j & ~e2i;
              const int lni = __popc(i1) + __popc(i2), lnj = __popc(j1) + __popc(j2);
              const int ni = lni + s_hn[wib][o];
              const uint32_t hx = s_hx[wib][o];
              const int hx0 = (int)(hx & 0xffu), hx1 = (int)((hx >> 8) & 0xffu);
              const int hy0 = (int)((hx >> 16) & 0xffu), hy1 = (int)(hx >> 24);
              // first two orbitals of each list: lo ones (a doubly emptied / filled orbital
              // twice), then hi ones
              const int la0 = __ffs(i1 | i2) - 1, lb0 = __ffs(j1 | j2) - 1;
              const int la1 = (lni < 2) ? -1 : ((i1 & i2) >> la0) & 1u ? la0 : __ffs((i1 | i2) & ~(1u << la0)) - 1;
              const int lb1 = (lnj < 2) ? -1 : ((j1 & j2) >> lb0) & 1u ? lb0 : __ffs((j1 | j2) & ~(1u << lb0)) - 1;
              const int ex0 = (lni >= 1) ? la0 : hx0, jy0 = (lnj >= 1) ? lb0 : hy0;
              const int ex1 = (lni >= 2) ? la1 : (lni == 1) ? hx0 : hx1;
              const int jy1 = (lnj >= 2) ? lb1 : (lnj == 1) ? hy0 : hy1;
              // the tests below are symmetric in the two configurations' roles
              if (ni == 2) {
                const int64_t e = ((int64_t)ex1 * (ex1 + 1) / 2 + ex0) * J.nt + (int64_t)jy1 * (jy1 + 1) / 2 + jy0;
                keep = (__ldg(J.dkept + (e >> 5)) >> (e & 31)) & 1u;
              } else if (ni == 1 && __ldg(P.jsym + j) != js_i) {
                keep = __ldg(P.one + tri64(ex0, jy0)) != 0.0;
              }
            }
          }
        }
        const unsigned kb = __ballot_sync(0xffffffffu, keep);
        if (MODE == 0) {
          nc += __popc(__ballot_sync(0xffffffffu, found));
          nk += __popc(kb);
        } else if (MODE == 1) {
          if (keep) P.nbr[base + __popc(kb & ((1u << lane) - 1u))] = j;
          base += __popc(kb);
        } else {
          nc += __popc(__ballot_sync(0xffffffffu, found));
          if (cursor + 32 > chunk_end) {
            // a fresh chunk; the list written so far moves along
            const unsigned long long len = (unsigned long long)max((int64_t)JOIN_CHUNK, 2 * (nk + 32));
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(S.counter, len);
            b = __shfl_sync(0xffffffffu, b, 0);
            __syncwarp();  // the list's earlier entries were written by other lanes
            for (int64_t t = lane; t < nk; t += 32) {
              const unsigned long long from = lstart + t, to = b + t;
              if ((int64_t)from < S.cap && (int64_t)to < S.cap) S.list[to] = S.list[from];
            }
            lstart = b;
            cursor = b + nk;
            chunk_end = b + len;
          }
          const unsigned long long pos = cursor + __popc(kb & ((1u << lane) - 1u));
          if (keep && (int64_t)pos < S.cap) S.list[pos] = j;
          cursor += __popc(kb);
          nk += __popc(kb);
        }
      }
      __syncwarp();
    }
    if (MODE != 1 && lane == 0) { cnt[i] = nk; ncand[i] = nc; }
    if (MODE == 2 && lane == 0) S.start[i] = (int64_t)lstart;
  }
}

// neighbour lists from the join slab to their final, contiguous places
__global__ void k_join_compact(int nconf, const int32_t *__restrict__ slab, const int64_t *__restrict__ start,
                               const int64_t *__restrict__ nbroff, int32_t *__restrict__ nbr) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < nconf; i += nwarps) {
    const int64_t o = nbroff[i], len = nbroff[i + 1] - o, st = start[i];
    for (int64_t t = lane; t < len; t += 32) nbr[o + t] = slab[st + t];
  }
}

// per row configuration: exclusive offsets of its column ranges and its total
__global__ void k_screen_offsets(int nconf, int nsplit, const int64_t *cnt, int64_t *soff, int64_t *tot) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t run = 0;
  for (int sp = 0; sp < nsplit; ++sp) {
    int64_t v = cnt[(int64_t)sp * nconf + i];
    soff[(int64_t)sp * nconf + i] = run;
    run += v;
  }
  tot[i] = run;
}

// per configuration: number of segments and segment-row slots over its first nlen[i]
// neighbours (all of them when nlen is null)
__global__ void k_seg_counts(int nconf, const int64_t *nbroff, const int64_t *nlen, const int64_t *sefoff,
                             int64_t *nseg_i, int64_t *nrow_i) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t nn = nlen ? nlen[i] : nbroff[i + 1] - nbroff[i];
  int64_t ns = (nn + PSOCI_SEG - 1) / PSOCI_SEG;
  nseg_i[i] = ns;
  nrow_i[i] = ns * (sefoff[i + 1] - sefoff[i]);
}

__global__ void k_seg_init(int nconf, const int64_t *nbroff, const int64_t *nlen, const int64_t *sefoff,
                           const int64_t *segoff, const int64_t *rowslot, int32_t *seg_cfg, int64_t *seg_k0,
                           int32_t *seg_n, int64_t *seg_rowoff) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t nn = nlen ? nlen[i] : nbroff[i + 1] - nbroff[i];
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

// per configuration: nlow = neighbours J <= i (the lists are sorted ascending) and the
// number of (lower pair, row SEF) mask slots, nlow * nsef_i
__global__ void k_lower_counts(int nconf, const int64_t *nbroff, const int32_t *nbr, const int64_t *sefoff,
                               int64_t *nlow, int64_t *prrows) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nconf) return;
  int64_t lo = nbroff[i], hi = nbroff[i + 1];
  while (lo < hi) {  // first entry > i
    int64_t mid = (lo + hi) >> 1;
    if (nbr[mid] <= (int32_t)i) lo = mid + 1; else hi = mid;
  }
  nlow[i] = lo - nbroff[i];
  prrows[i] = nlow[i] * (sefoff[i + 1] - sefoff[i]);
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
// The first two positions of the multiset m1 + m2 (a position in both counts twice),
// ascending.
template <int W>
__device__ __forceinline__ void two_positions(const uint64_t (&m1)[W], const uint64_t (&m2)[W], int &p0, int &p1) {
  int nd = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    uint64_t u = m1[w] | m2[w];
    while (u && nd < 2) {
      const int b = __ffsll((long long)u) - 1;
      u &= u - 1;
      const int p = 64 * w + b;
      const int mult = (int)((m1[w] >> b) & 1ull) + (int)((m2[w] >> b) & 1ull);
      if (nd == 0) { p0 = p; nd = 1; if (mult == 2) { p1 = p; nd = 2; } }
      else { p1 = p; nd = 2; }
    }
  }
}

// Set up the pair (A, B) in the reference's roles (A = "iconf" of generateSOCIblocks);
// J is the configuration whose SEFs are the CSR columns.
template <int W>
__device__ void pair_setup_ab(const Params &P, int A, int B, int J, int swap, PairInfo &pi, double *Kd) {
  pi.swap = swap;
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
  pi.iex0 = pi.jex0 = -1;
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
        int occi = 1 + (int)bit_w<W>(e2A, ib);
        if (occi == 1) v += g1(P, ib, ib);
        else v += 2.0 * g1(P, ib, ib) + g2(P, ib, ib, ib, ib);
#pragma unroll
        for (int wj = 0; wj < W; ++wj) {
          uint64_t oj = e1A[wj];
          while (oj) {
            int jb = 64 * wj + __ffsll((long long)oj) - 1;
            oj &= oj - 1;
            if (jb >= ib) break;
            int ninj = occi * (1 + (int)bit_w<W>(e2A, jb));
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
    between_mask<W>(ie, je, pi.bm[0]);
    range_mask<W>(0, ie - 1, pi.bm[1]);
    range_mask<W>(je + 1, 64 * W - 1, pi.bm[2]);
    range_mask<W>(0, je - 1, pi.bm[3]);
    range_mask<W>(ie + 1, 64 * W - 1, pi.bm[4]);
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
        bool dA = bit_w<W>(e2A, p);
        if (dA) v += buf;
        if (dA && bit_w<W>(e2B, p)) v -= g2(P, ie, p, p, je);
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
    int ex0 = -1, ex1 = -1, jy0 = -1, jy1 = -1;
    two_positions<W>(im1, im2, ex0, ex1);
    two_positions<W>(jm1, jm2, jy0, jy1);
    const int ex[2] = {ex0, ex1}, jy[2] = {jy0, jy1};
    pi.iex0 = ex0; pi.jex0 = jy0;
    between_mask<W>(ex0, jy0, pi.bm[0]);
    between_mask<W>(ex0, jy1, pi.bm[1]);
    between_mask<W>(ex1, jy0, pi.bm[2]);
    between_mask<W>(ex1, jy1, pi.bm[3]);
    between_mask<W>(ex0, ex1, pi.bm[4]);
    between_mask<W>(jy0, jy1, pi.bm[5]);
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

template <int W>
__device__ void pair_setup(const Params &P, int I, int J, PairInfo &pi, double *Kd) {
  if (J <= I) pair_setup_ab<W>(P, I, J, J, 0, pi, Kd);
  else pair_setup_ab<W>(P, J, I, J, 1, pi, Kd);
}

// ------------------------------------------------------------------------------------
// determinant element <det a of A | H | det b of B>
// ------------------------------------------------------------------------------------
// One determinant: alpha and beta bit-strings, phase, alpha count.
template <int W>
struct DetBits {
  uint64_t al[W], be[W];
  int ph, na;
};

template <int W>
__device__ __forceinline__ void load_det(DetBits<W> &d, const uint64_t *alpha, const uint64_t *beta,
                                         const uint8_t *phase, const uint8_t *nalpha, int64_t i) {
#pragma unroll
  for (int w = 0; w < W; ++w) { d.al[w] = alpha[i * W + w]; d.be[w] = beta[i * W + w]; }
  d.ph = phase[i];
  d.na = nalpha[i];
}

// Diagonal element of a determinant (processDiagExcitation's vnt list): Kd[0] minus the
// exchange integral of every pair of open shells (io > jo, in the reference's order) whose
// spins agree.  Out of line: it runs for the diagonal blocks only, and keeping its loops out
// of the element code keeps that code compact.
template <int W>
__device__ __noinline__ double diag_det_elem(const uint64_t *SA, const double *Kd, const uint64_t (&aa)[W]) {
  double v = Kd[0];
  int mm = 0, io = 0;
#pragma unroll
  for (int wi = 0; wi < W; ++wi) {
    uint64_t si_bits = SA[wi];
    while (si_bits) {
      const uint64_t lo_i = si_bits & (~si_bits + 1);
      si_bits ^= lo_i;
      const bool si = (aa[wi] & lo_i) != 0ull;
      // open shells below this one, ascending
      int jo = 0;
#pragma unroll
      for (int wj = 0; wj < W; ++wj) {
        uint64_t sj = SA[wj];
        while (sj && jo < io) {
          const uint64_t lo_j = sj & (~sj + 1);
          sj ^= lo_j;
          ++mm;
          if (si == ((aa[wj] & lo_j) != 0ull)) v -= Kd[mm];
          ++jo;
        }
      }
      ++io;
    }
  }
  return v;
}

// <det a of A | H | det b of B> from the loaded determinants.  sef_elem calls it from a
// single site (a loop over the determinant pairs of an SEF element), so the kernels hold
// one copy of this body: several inlined copies overflow their instruction cache.
template <int W>
__device__ __forceinline__ double det_elem(const double *eri, const PairInfo &pi, const double *Kd,
                                           const DetBits<W> &A, const DetBits<W> &B) {
  const uint64_t(&aa)[W] = A.al;
  const uint64_t(&ba)[W] = A.be;
  const uint64_t(&ab)[W] = B.al;
  const uint64_t(&bb)[W] = B.be;
  const int pha = A.ph, phb = B.ph, naa = A.na, nab = B.na;
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
      ncount += popc_and<W>(ba, pi.bm[1]) + popc_and<W>(ab, pi.bm[2]);
      if ((pi.jsA + pi.jsB) % 2 == 0) ++ncount;
      else if (pi.jsA % 2 == 1) ++ncount;
    } else if (naa > nab) {
      ncount += popc_and<W>(aa, pi.bm[4]) + popc_and<W>(bb, pi.bm[3]);
      if ((pi.jsA + pi.jsB) % 2 != 0 && (pi.jsA % 2) == 1) ++ncount;
    } else {
      if (nmarka == 0) ++ncount;
      if (pi.jsA % 2 == 1) ++ncount;
      uint64_t sp[W];
      sel_w<W>(sp, nmarka != 0, aa, ba);
      ncount += popc_and<W>(sp, pi.bm[0]);  // empty unless |ie - je| > 1
    }
    return (ncount & 1) ? -pi.v0 : pi.v0;
  }

  // generateSEFCIG (PsociHamiltonian.C:902-1113): equal spin projection only
  if (naa != nab) return 0.0;
  if (nmarka > 2 || nmarkb > 2) return 0.0;
  if (nmarkb == 0) {
    if (pi.kind != K_DIAG) return 0.0;  // identical determinants occur only on the diagonal
    return diag_det_elem<W>(pi.SA, Kd, aa);
  }
  if (nmarkb == 1) {
    // one spin-orbital excitation within spin (nmarka == 1: alpha, else beta)
    uint64_t sp[W];
    sel_w<W>(sp, nmarka != 0, aa, ba);
    int ncount = pha + phb + popc_and<W>(sp, pi.bm[0]);  // empty unless |ie - je| > 1
    double v = pi.v0;
    // exchange with the open shells of that spin in det a, except the excited orbitals, in
    // ascending orbital order; X is indexed by the rank among A's open shells
    int t = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t m = sp[w] & ~(aa[w] & ba[w]);
      if ((ie >> 6) == w) m &= ~(1ull << (ie & 63));
      if ((je >> 6) == w) m &= ~(1ull << (je & 63));
      uint64_t sa = pi.SA[w];
      while (sa) {
        const uint64_t low = sa & (~sa + 1);
        if (m & low) v -= pi.X[t];
        ++t;
        sa ^= low;
      }
    }
    return (ncount & 1) ? -v : v;
  }
  if (nmarka == 1) {
    // alpha single times beta single
    uint64_t xa[W], xb[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { xa[w] = aa[w] & ~ab[w]; xb[w] = ba[w] & ~bb[w]; }
    if (pi.kind == K_DOUBLE) {
      // the alpha electron moves ex_ia -> jy_ja, the beta one the other two orbitals (the
      // same one when a doubly occupied orbital empties or fills); the integral
      // (beta move | alpha move) is then the table entry of v0 (ia == ja) or v1
      const int ia = bit_w<W>(xa, pi.iex0) ? 0 : 1, ja = bit_w<W>(ua, pi.jex0) ? 0 : 1;
      const int ncount = pha + phb + popc_and<W>(aa, pi.bm[2 * ia + ja]) + popc_and<W>(ba, pi.bm[3 - 2 * ia - ja]);
      const double v = (ia == ja) ? pi.v0 : pi.v1;
      return (ncount & 1) ? -v : v;
    }
    int iex2 = lowest_bit<W>(ua), jex2 = lowest_bit<W>(ub);
    int iex3 = lowest_bit<W>(xa), jex3 = lowest_bit<W>(xb);
    int ncount = pha + phb;
    if (abs(iex2 - iex3) > 1) ncount += popc_range<W>(aa, min(iex2, iex3) + 1, max(iex2, iex3) - 1);
    if (abs(jex2 - jex3) > 1) ncount += popc_range<W>(ba, min(jex2, jex3) + 1, max(jex2, jex3) - 1);
    double v = __ldg(eri + canon4(jex2, jex3, iex2, iex3));
    return (ncount & 1) ? -v : v;
  }
  // same-spin double (nmarka == 2: alpha, nmarka == 0: beta)
  if (pi.kind != K_DOUBLE) return 0.0;
  // both electrons of one spin move ex0, ex1 -> jy0, jy1 (distinct orbitals)
  uint64_t spb[W], sa[W];
  sel_w<W>(spb, nmarka == 2, ab, bb);
  sel_w<W>(sa, nmarka != 0, aa, ba);
  int ncount = pha + phb + popc_and<W>(spb, pi.bm[5]) + popc_and<W>(sa, pi.bm[4]);
  double v = pi.v0 - pi.v1;
  return (ncount & 1) ? -v : v;
}

// Where sef_elem finds the determinants of A: the global tables, or a copy of A's own
// determinants in shared memory (rows indexed from A's first determinant).
struct RowDets {
  const uint64_t *al, *be;
  const uint8_t *ph, *na;
};

// SEF element (a, b) of the reference block (A, B): ciout / transformCDCt.  conn bit
// (x << 1 | y) says whether determinant x of SEF a and determinant y of SEF b can couple;
// a determinant element that cannot is exactly zero and is not evaluated (adding the zero
// it would return leaves every partial sum unchanged).  The determinant elements are
// added in the reference's order: t = d00 + mB d01, u = d10 + mB d11, r (r t) + mA r (r u).
template <int W>
__device__ double sef_elem(const Params &PP, const PairInfo &pi, const double *Kd, int a, int b,
                           unsigned conn = 0xFu, const RowDets *rowA = nullptr) {
  if (pi.kind == K_NONE) return 0.0;
  const bool odd = PP.nelec & 1;
  const bool oa = !odd && pi.nopenA != 0, ob = !odd && pi.nopenB != 0;
  const int64_t a0 = odd ? a : (oa ? 2 * a : 0), b0 = pi.detB + (odd ? b : (ob ? 2 * b : 0));
  if (!ob) conn &= 0x5u;
  if (!oa) conn &= 0x3u;
  DetBits<W> A[2] = {}, B[2] = {};
#pragma unroll
  for (int x = 0; x < 2; ++x) {
    if (x == 1 && !oa) break;
    if (rowA) load_det<W>(A[x], rowA->al, rowA->be, rowA->ph, rowA->na, a0 + x);
    else load_det<W>(A[x], PP.alpha, PP.beta, PP.phase, PP.nalpha, pi.detA + a0 + x);
  }
#pragma unroll
  for (int y = 0; y < 2; ++y) {
    if (y == 1 && !ob) break;
    load_det<W>(B[y], PP.alpha, PP.beta, PP.phase, PP.nalpha, b0 + y);
  }
  const double mA = (pi.jsA % 2 != PP.ksym % 2) ? -1.0 : 1.0;
  const double mB = (pi.jsB % 2 != PP.ksym % 2) ? -1.0 : 1.0;
  double t = 0.0, u = 0.0;
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    if (!((conn >> q) & 1u)) continue;
    const int x = q >> 1, y = q & 1;
    DetBits<W> Ax, By;  // selected by value: the arrays stay in registers
#pragma unroll
    for (int w = 0; w < W; ++w) {
      Ax.al[w] = x ? A[1].al[w] : A[0].al[w];
      Ax.be[w] = x ? A[1].be[w] : A[0].be[w];
      By.al[w] = y ? B[1].al[w] : B[0].al[w];
      By.be[w] = y ? B[1].be[w] : B[0].be[w];
    }
    Ax.ph = x ? A[1].ph : A[0].ph;
    Ax.na = x ? A[1].na : A[0].na;
    By.ph = y ? B[1].ph : B[0].ph;
    By.na = y ? B[1].na : B[0].na;
    const double d = det_elem<W>(PP.eri, pi, Kd, Ax, By);
    if (x == 0) t = (y == 0) ? d : t + mB * d;
    else u = (y == 0) ? d : u + mB * d;
  }
  if (odd) return t;
  const double r = sqrt(0.5);
  const double ds0 = ob ? t * r : t;
  const double ds1 = ob ? u * r : u;
  if (oa) {
    double v = r * ds0;
    v += (mA * r) * ds1;
    return v;
  }
  return ds0;
}

// FP64 sum over the warp of v[0..7], scattered: lanes 4q..4q+3 end with the total of q
__device__ __forceinline__ double reduce_scatter8_f64(const double (&v)[8], int lane) {
  double a[4], b[2];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool hi = lane & 16;
    a[i] = (hi ? v[i + 4] : v[i]) + __shfl_xor_sync(0xffffffffu, hi ? v[i] : v[i + 4], 16);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool hi = lane & 8;
    b[i] = (hi ? a[i + 2] : a[i]) + __shfl_xor_sync(0xffffffffu, hi ? a[i] : a[i + 2], 8);
  }
  const bool hi = lane & 4;
  double c = (hi ? b[1] : b[0]) + __shfl_xor_sync(0xffffffffu, hi ? b[0] : b[1], 4);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  return c;
}

// ------------------------------------------------------------------------------------
// segment kernel over full neighbour lists: PASS 0 counts kept elements per row, PASS 1
// writes them; direct mode: PASS 2 adds H X into Y (atomically: a configuration's rows
// may span several segments), PASS 3 writes the diagonal only
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
    // PASS 3: the diagonal block (J = I) is in exactly one segment of I
    if (PASS == 3 && lane < n && ws->pi[lane].kind == K_DIAG)
      for (int r = 0; r < nsefI; ++r) P.diag[P.sefoff[I] + r] = sef_elem<W>(P, ws->pi[lane], ws->K, r, r);
    for (int r = 0; r < (PASS == 3 ? 0 : nsefI); ++r) {
      double acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = 0.0;
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
          // lower half of a diagonal block as the reference computes it, upper half mirrored;
          // block (J, I) transposed for J > I
          const bool diag_blk = (pi.kind == K_DIAG);
          const bool flip = diag_blk ? (t > r) : (pi.swap != 0);
          v = sef_elem<W>(P, pi, ws->K, flip ? t : r, flip ? r : t);
          keep = (fabs(v) >= PSOCI_MIN_VALUE) || (diag_blk && t == r);
        }
        if (PASS == 2 && keep) {
          const double *xr = P.dx + (int64_t)(ws->pi[k].colbase + t) * P.ldx;
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (q < P.kvec) acc[q] = fma(v, xr[q], acc[q]);
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
      if (PASS == 2) {
        const double tot = reduce_scatter8_f64(acc, lane);
        const int q = lane >> 2;
        if ((lane & 3) == 0 && q < P.kvec && tot != 0.0) atomicAdd(P.dy + (P.sefoff[I] + r) * P.ldy + q, tot);
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------------
// Fast segment kernel for configurations of at most 32 determinants (<= 6 open shells with
// an even electron count, <= 5 with an odd one; at most 16 SEFs).  A SEF block is sparse:
// a determinant couples only to determinants within two spin-orbital substitutions with
// the same spin projection (one substitution, any spin, for spin-orbit pairs).  Each lane
// owns one neighbour J and first marks, per row SEF r of I, the column SEFs t whose
// determinants pass that test; only marked elements are then evaluated, with the same
// element function (and operation order) as the generic kernel.  An unmarked element is
// a combination of zero determinant elements and therefore exactly zero.
// ------------------------------------------------------------------------------------
constexpr int FAST_MAXDET = 32;
constexpr int FAST_MAXSEF = 16;
constexpr int FAST_MAXOPEN = 6;  // 2^(6-1) = 32 determinants
constexpr int SLAB_CHUNK = 4096; // slab slots a warp takes at a time
constexpr int FAST_ROWS = 4;     // rows of a configuration evaluated together
constexpr int FAST_MAXK = 1 + FAST_MAXOPEN * (FAST_MAXOPEN - 1) / 2;  // diagonal list, <= 6 open shells

__device__ __forceinline__ bool tbit(const uint64_t *x, int p) { return (x[p >> 6] >> (p & 63)) & 1ull; }

template <int W>
struct FastSmem {
  PairInfo pi[PSOCI_SEG];
  double K[FAST_MAXK];
  uint64_t ra[FAST_MAXDET * W], rb[FAST_MAXDET * W];
  uint8_t rna[FAST_MAXDET], rph[FAST_MAXDET];
  // phase 2, per row of a group: connectivity of the marked elements of each slot (see
  // below; the marked columns are its four 16-bit quarters or-ed), their exclusive prefix,
  // kept columns of each neighbour
  uint64_t cm[FAST_ROWS][PSOCI_SEG];
  int16_t pre[FAST_ROWS][PSOCI_SEG];
  uint32_t keep[FAST_ROWS][PSOCI_SEG];
  int8_t perm[PSOCI_SEG];  // evaluation order: slot -> neighbour lane, grouped by pair kind
};

// DIRECT (direct mode): segments over the full neighbour lists; instead of storing the kept
// elements, Y[row, 0:kvec] += element * X[column, 0:kvec], added atomically per row.
// PH: 0 both phases in one launch; 2 phase 2 alone, from the connectivity masks that
// k_hbuild_masks stored in P.cg (each launch then runs a smaller body).
template <int W, int DIRECT = 0, int PH = 0>
__global__ void __launch_bounds__(WARPS_PER_CTA * 32) k_hbuild_fast(Params P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FastSmem<W> *ws = reinterpret_cast<FastSmem<W> *>(smem_raw) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool odd = P.nelec & 1;
  unsigned long long cursor = 0, chunk_end = 0;  // this warp's slab chunk
  for (int64_t s = warp; s < P.nseg; s += nwarps) {
    const int I = P.seg_cfg[s];
    const int64_t k0 = P.seg_k0[s];
    const int n = P.seg_n[s];
    const int nsefI = (int)(P.sefoff[I + 1] - P.sefoff[I]);
    const int64_t d0I = P.detoff[I];
    const int ndI = (int)(P.detoff[I + 1] - d0I);
    const int nopI = P.nopen[I];
    if (lane < n) pair_setup<W>(P, I, P.nbr[k0 + lane], ws->pi[lane], ws->K);
    for (int d = lane; d < ndI; d += 32) {
#pragma unroll
      for (int w = 0; w < W; ++w) {
        ws->ra[d * W + w] = P.alpha[(d0I + d) * W + w];
        ws->rb[d * W + w] = P.beta[(d0I + d) * W + w];
      }
      ws->rna[d] = P.nalpha[d0I + d];
      ws->rph[d] = P.phase[d0I + d];
    }
    __syncwarp();
    // phase 1: connectivity masks C[r] for this lane's neighbour, bit-parallel over the
    // row determinants.  With m_a the alpha pattern of row det a on I's open shells, a column
    // det b (alpha ab, beta bb) differs from a in
    //   c(a) = F + #{p in x : p not in m_a} + #{p in y : p in m_a}
    // spin-orbitals of b, where x, y are b's alpha / beta patterns on I's open shells and F
    // counts b's electrons in orbitals empty in I.  Non-spin-orbit pairs need c(a) <= 2 and
    // equal alpha counts, spin-orbit pairs c(a) <= 1 (the tests det_elem starts with).  The sets
    // {a : p in m_a} and {a : |m_a| = k} are warp ballots; c(a) is kept as a saturating
    // bit-sliced counter over all row dets at once.
    uint32_t Ap[FAST_MAXOPEN], Nk[FAST_MAXOPEN + 1];
    int sI[FAST_MAXOPEN];
    uint64_t occI[W];
    if (PH != 2) {
      uint64_t SI[W];
#pragma unroll
      for (int w = 0; w < W; ++w) {
        occI[w] = P.e1[(int64_t)I * W + w];
        SI[w] = occI[w] & ~P.e2[(int64_t)I * W + w];
      }
      // open shells of I, ascending (fixed-size loops keep these arrays in registers)
#pragma unroll
      for (int p = 0; p < FAST_MAXOPEN; ++p) {
        sI[p] = lowest_bit<W>(SI);
        bool done = false;
#pragma unroll
        for (int w = 0; w < W; ++w)
          if (!done && SI[w]) { SI[w] &= SI[w] - 1; done = true; }
      }
      uint32_t ma = 0u;
      if (lane < ndI)
#pragma unroll
        for (int p = 0; p < FAST_MAXOPEN; ++p)
          if (p < nopI) ma |= (uint32_t)tbit(&ws->ra[lane * W], sI[p]) << p;
#pragma unroll
      for (int p = 0; p < FAST_MAXOPEN; ++p) Ap[p] = __ballot_sync(0xffffffffu, (lane < ndI) && ((ma >> p) & 1u));
#pragma unroll
      for (int k = 0; k <= FAST_MAXOPEN; ++k) Nk[k] = __ballot_sync(0xffffffffu, (lane < ndI) && __popc(ma) == k);
    }
    const int ndblI = P.nelec - nopI;  // electrons in I's doubly occupied orbitals
    // C[r]: for row SEF r and column SEF t, bit t + 16 (x << 1 | y) says that determinant x
    // of SEF r and determinant y of SEF t can couple; the SEF element is marked when any can.
    uint64_t C[FAST_MAXSEF];
    for (int r = 0; r < FAST_MAXSEF; ++r) C[r] = 0ull;
    if (PH != 2 && lane < n) {
      const PairInfo &pi = ws->pi[lane];
      if (pi.kind != K_NONE) {
        const bool so = (pi.kind == K_SO);
        const int64_t d0J = pi.swap ? pi.detA : pi.detB;
        const int nopJ = pi.swap ? pi.nopenA : pi.nopenB;
        const int ndJ = 1 << (nopJ > 1 ? nopJ - 1 : 0);
        const int thr = so ? 1 : 2;
        const uint32_t rows_valid = (ndI >= 32) ? 0xffffffffu : ((1u << ndI) - 1u);
        for (int b = 0; b < ndJ; ++b) {
          uint64_t ja[W], jb[W];
#pragma unroll
          for (int w = 0; w < W; ++w) { ja[w] = __ldg(P.alpha + (d0J + b) * W + w); jb[w] = __ldg(P.beta + (d0J + b) * W + w); }
          int F = 0;
#pragma unroll
          for (int w = 0; w < W; ++w) F += __popcll(ja[w] & ~occI[w]) + __popcll(jb[w] & ~occI[w]);
          if (F > thr) continue;
          uint32_t ok = 0u;
          {
            // saturating counter over the row dets: S0 (c'=0), S1, S2, S3 (>= 3)
            uint32_t S0 = 0xffffffffu, S1 = 0u, S2 = 0u;
#pragma unroll
            for (int p = 0; p < FAST_MAXOPEN; ++p) {
              if (p >= nopI) break;
              const bool xa = bit_w<W>(ja, sI[p]), yb = bit_w<W>(jb, sI[p]);
              if (xa) {  // mismatch where row det has beta on p
                const uint32_t T = ~Ap[p];
                S2 = (S2 & ~T) | (S1 & T);
                S1 = (S1 & ~T) | (S0 & T);
                S0 &= ~T;
              }
              if (yb) {  // mismatch where row det has alpha on p
                const uint32_t T = Ap[p];
                S2 = (S2 & ~T) | (S1 & T);
                S1 = (S1 & ~T) | (S0 & T);
                S0 &= ~T;
              }
            }
            ok = (thr - F >= 2) ? (S0 | S1 | S2) : (thr - F == 1) ? (S0 | S1) : S0;
          }
          int na = 0;
#pragma unroll
          for (int w = 0; w < W; ++w) na += __popcll(ja[w]);
          const int need = na - (ndblI / 2);  // alpha open shells a row det needs for equal counts
          ok &= rows_valid;
          if (!so) {
            uint32_t nk = 0u;
#pragma unroll
            for (int k = 0; k <= FAST_MAXOPEN; ++k)
              if (k == need) nk = Nk[k];
            ok &= (need >= 0 && need <= nopI) ? nk : 0u;
          }
          const int t = odd ? b : (nopJ ? (b >> 1) : 0);
          const int y = (!odd && nopJ) ? (b & 1) : 0;
          while (ok) {
            const int a = __ffs(ok) - 1;
            ok &= ok - 1;
            const int x = (!odd && nopI) ? (a & 1) : 0;
            C[odd ? a : (nopI ? (a >> 1) : 0)] |= 1ull << (t + 16 * ((x << 1) | y));
          }
        }
      }
    }
    const int64_t prbase = DIRECT ? 0 : P.pr_off[I] + (k0 - P.nbroff[I]) * nsefI;
    // phase 2, FAST_ROWS rows at a time (one row in the direct modes, whose sums are per
    // row): the marked elements of the group's rows, in (row, neighbour, column) order, are
    // numbered e = 0..T-1 and lane e % 32 evaluates element e, so the lanes share the work
    // whatever the spread of marks over the neighbours and rows (a row holds about one
    // warp's worth of marks: taken alone, its last pass would run on few lanes).  Kept values
    // are compacted in the same order, so each row's values form one run in ascending column
    // order and the runs of a group follow one another.  Each warp takes slab space in chunks
    // and advances through a chunk by the kept count of each group.
    const RowDets rowA = {ws->ra, ws->rb, ws->rph, ws->rna};  // I's determinants (A = I)
    // evaluation order of the neighbours: grouped by pair kind (doubles, singles, spin-orbit,
    // diagonal), ascending within a kind, so that neighbouring lanes mostly run the same
    // branch of the element code.  Values of a row are stored in this order; each pair's
    // offset in its row run goes to prm, which is all the assembly needs.
    {
      const int kd = (lane < n) ? ws->pi[lane].kind : -1;
      const int key = (kd == K_DOUBLE) ? 0 : (kd == K_SINGLE) ? 1 : (kd == K_SO) ? 2 : (kd == K_DIAG) ? 3
                                                                                         : (kd == K_NONE) ? 4 : 5;
      int rank = 0, base = 0;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, key == k);
        if (key == k) rank = base + __popc(m & ((1u << lane) - 1u));
        base += __popc(m);
      }
      ws->perm[rank] = (int8_t)lane;
      __syncwarp();
    }
    const int src = ws->perm[lane];  // the neighbour lane at evaluation slot `lane`
    constexpr int R = DIRECT ? 1 : FAST_ROWS;
    for (int r0 = 0; r0 < nsefI; r0 += R) {
      const int nr = min(R, nsefI - r0);
      // per row g of the group: marked columns of each slot, their exclusive prefix counted
      // from the group's first element, and rs[g], the row's first element
      int T = 0, rs[R];
#pragma unroll
      for (int g = 0; g < R; ++g) {
        rs[g] = T;
        if (g < nr) {
          const uint64_t cr = (PH == 2) ? ((src < n) ? __ldg(P.cg + prbase + (int64_t)src * nsefI + r0 + g) : 0ull)
                                        : __shfl_sync(0xffffffffu, (lane < n) ? C[r0 + g] : 0ull, src);
          const uint32_t mr = (uint32_t)((cr | (cr >> 16) | (cr >> 32) | (cr >> 48)) & 0xffffull);
          const int cm = __popc(mr);
          int inclm = cm;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inclm, o);
            if (lane >= o) inclm += v;
          }
          ws->pre[g][lane] = (int16_t)(T + inclm - cm);
          ws->cm[g][lane] = cr;
          ws->keep[g][lane] = 0u;
          T += __shfl_sync(0xffffffffu, inclm, 31);
        }
      }
      if (!DIRECT && cursor + T > chunk_end) {  // room for every marked element of the group
        const unsigned long long len = (unsigned long long)max(T, SLAB_CHUNK);
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(P.slab_counter, len);
        cursor = __shfl_sync(0xffffffffu, b, 0);
        chunk_end = cursor + len;
      }
      double acc[8];
      float accs[8], accc[8];  // DIRECT == 2: compensated FP32 sums of FP32 products
#pragma unroll
      for (int q = 0; q < 8; ++q) { acc[q] = 0.0; accs[q] = 0.f; accc[q] = 0.f; }
      const unsigned long long base = cursor;
      // chunks beyond the slab capacity are counted but not written; the host sees the
      // final counter, enlarges the slab and evaluates again
      const bool fits = (int64_t)chunk_end <= P.slab_cap;
      __syncwarp();
      int kc = 0;
      for (int e0 = 0; e0 < T; e0 += 32) {
        const int e = e0 + lane;
        bool keep = false;
        double v = 0.0;
        if (e < T) {
          int g = 0;  // the row of element e: last row whose first element is <= e
#pragma unroll
          for (int k = 1; k < R; ++k) g += (rs[k] <= e);
          const int r = r0 + g;
          int o = 0;  // the slot owning element e: last slot whose prefix is <= e
#pragma unroll
          for (int step = 16; step > 0; step >>= 1)
            if (ws->pre[g][o + step] <= e) o += step;
          const uint64_t cw = ws->cm[g][o];
          uint32_t m = (uint32_t)((cw | (cw >> 16) | (cw >> 32) | (cw >> 48)) & 0xffffull);
          for (int q = e - ws->pre[g][o]; q > 0; --q) m &= m - 1;
          const int t = __ffs(m) - 1;
          const int pl = ws->perm[o];  // its neighbour lane
          const PairInfo &pi = ws->pi[pl];
          // reference roles: the lower half of a diagonal block, block (J, I) for J > I
          const bool diag_blk = (pi.kind == K_DIAG);
          const bool flip = diag_blk ? (t > r) : (pi.swap != 0);
          const uint64_t co = cw >> t;
          unsigned conn = (unsigned)((co & 1ull) | ((co >> 15) & 2ull) | ((co >> 30) & 4ull) | ((co >> 45) & 8ull));
          // a diagonal block is symmetric: the transposed element swaps the determinant roles
          if (flip) conn = (conn & 9u) | ((conn & 2u) << 1) | ((conn & 4u) >> 1);
          // A's determinants come from shared memory when A = I (every lower pair; a pair
          // J > I of the direct mode has A = J, read from the tables)
          v = sef_elem<W>(P, pi, ws->K, flip ? t : r, flip ? r : t, conn, (DIRECT && pi.swap) ? nullptr : &rowA);
          keep = (fabs(v) >= PSOCI_MIN_VALUE) || (diag_blk && t == r);
          if (DIRECT) {
            if (DIRECT == 2 && keep) {
              const float vf = (float)v;
              const float4 *xr = reinterpret_cast<const float4 *>(P.dx32 + (pi.colbase + t) * 8);
              const float4 xa = __ldg(xr), xb = __ldg(xr + 1);
              const float xv[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
#pragma unroll
              for (int q = 0; q < 8; ++q) {
                // Kahan: the rounding error of each addition is carried in accc and fed back
                const float yv = __fsub_rn(__fmul_rn(vf, xv[q]), accc[q]);
                const float tt = __fadd_rn(accs[q], yv);
                accc[q] = __fsub_rn(__fsub_rn(tt, accs[q]), yv);
                accs[q] = tt;
              }
            } else if (keep) {
              const double *xr = P.dx + (pi.colbase + t) * P.ldx;
#pragma unroll
              for (int q = 0; q < 8; ++q)
                if (q < P.kvec) acc[q] = fma(v, xr[q], acc[q]);
            }
          } else if (keep) {
            atomicOr(&ws->keep[g][pl], 1u << t);
          }
        }
        if (!DIRECT) {
          const unsigned kb = __ballot_sync(0xffffffffu, keep);
          if (keep && fits) P.slab_val[(int64_t)base + kc + __popc(kb & ((1u << lane) - 1u))] = v;
          kc += __popc(kb);
        }
      }
      if (DIRECT) {  // one row per group
        if (DIRECT == 2) {
#pragma unroll
          for (int q = 0; q < 8; ++q) acc[q] = (double)accs[q] - (double)accc[q];
        }
        const double tot = reduce_scatter8_f64(acc, lane);
        const int q = lane >> 2;
        if ((lane & 3) == 0 && q < P.kvec && tot != 0.0) atomicAdd(P.dy + (P.sefoff[I] + r0) * P.ldy + q, tot);
        __syncwarp();
        continue;
      }
      __syncwarp();
      // per row of the group: its kept count, its run's place in the slab, and each pair's
      // offset in the run (kept columns before it, in the evaluation order)
      unsigned long long run = base;
      for (int g = 0; g < nr; ++g) {
        const uint32_t keepm = (lane < n) ? ws->keep[g][lane] : 0u;
        const int cs = __popc(__shfl_sync(0xffffffffu, keepm, src));
        int incl = cs;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int kg = __shfl_sync(0xffffffffu, incl, 31);
        ws->pre[g][src] = (int16_t)(incl - cs);  // the element loop is done with pre
        __syncwarp();
        if (lane == 0) P.seg_cnt[P.seg_rowoff[s] + r0 + g] = kg;
        if (lane < n)
          P.prm[prbase + (int64_t)lane * nsefI + r0 + g] =
              (uint64_t)keepm | ((uint64_t)(run + (unsigned long long)ws->pre[g][lane]) << 16);
        run += (unsigned long long)kg;
      }
      cursor += (unsigned long long)kc;
      __syncwarp();
    }
    __syncwarp();
  }
}

// Connectivity masks of the lower pairs for the two-launch evaluation: for every (pair, row
// SEF r) the word C[r] of k_hbuild_fast's phase 1 (bit t + 16 (x << 1 | y): determinant x of
// row SEF r and determinant y of column SEF t can couple), stored in P.cg at the pair's prm
// index.  Pair kinds come from the excitation level and the symmetries alone, without the
// integrals: a pair whose integrals vanish is marked all the same, and its elements then
// evaluate to exactly zero and are not kept.  The work items, (neighbour, column SEF t), are
// spread evenly over the lanes; an item tests t's one or two column determinants against all
// row determinants at once (the bit-sliced counter of k_hbuild_fast) and ors the result into
// the neighbour's words in shared memory.
constexpr int MASK_WARPS = 8;
struct MaskSmem {
  uint64_t C[PSOCI_SEG][FAST_MAXSEF];
  int64_t d0J[PSOCI_SEG];
  int8_t nopJ[PSOCI_SEG], so[PSOCI_SEG];
  int16_t ipre[PSOCI_SEG];
};

template <int W>
__global__ void __launch_bounds__(MASK_WARPS * 32) k_hbuild_masks(Params P) {
  __shared__ MaskSmem smem_masks[MASK_WARPS];
  MaskSmem &ws = smem_masks[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const bool odd = P.nelec & 1;
  for (int64_t s = warp; s < P.nseg; s += nwarps) {
    const int I = P.seg_cfg[s];
    const int64_t k0 = P.seg_k0[s];
    const int n = P.seg_n[s];
    const int nsefI = (int)(P.sefoff[I + 1] - P.sefoff[I]);
    const int64_t d0I = P.detoff[I];
    const int ndI = (int)(P.detoff[I + 1] - d0I);
    const int nopI = P.nopen[I];
    uint64_t occI[W], dblI[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { occI[w] = P.e1[(int64_t)I * W + w]; dblI[w] = P.e2[(int64_t)I * W + w]; }
    // this lane's neighbour J <= I: diagonal, single (spin-orbit when the symmetries differ)
    // or double by the excitation level I -> J
    int nit = 0;
    if (lane < n) {
      const int J = P.nbr[k0 + lane];
      int ni = 0;
#pragma unroll
      for (int w = 0; w < W; ++w)
        ni += __popcll(occI[w] & ~P.e1[(int64_t)J * W + w]) + __popcll(dblI[w] & ~P.e2[(int64_t)J * W + w]);
      const bool diag = (J == I);
      ws.so[lane] = (int8_t)(!diag && ni == 1 && P.jsym[I] != P.jsym[J]);
      ws.d0J[lane] = P.detoff[J];
      ws.nopJ[lane] = (int8_t)P.nopen[J];
      nit = (diag || ni == 1 || ni == 2) ? (int)(P.sefoff[J + 1] - P.sefoff[J]) : 0;
    }
    for (int q = lane; q < PSOCI_SEG * FAST_MAXSEF; q += 32) (&ws.C[0][0])[q] = 0ull;
    int incl = nit;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    ws.ipre[lane] = (int16_t)(incl - nit);
    const int NIT = __shfl_sync(0xffffffffu, incl, 31);
    // I's open shells and, over the row determinants, the ballots of the counter
    uint32_t Ap[FAST_MAXOPEN], Nk[FAST_MAXOPEN + 1];
    int sI[FAST_MAXOPEN];
    {
      uint64_t SI[W];
#pragma unroll
      for (int w = 0; w < W; ++w) SI[w] = occI[w] & ~dblI[w];
#pragma unroll
      for (int p = 0; p < FAST_MAXOPEN; ++p) {
        sI[p] = lowest_bit<W>(SI);
        bool done = false;
#pragma unroll
        for (int w = 0; w < W; ++w)
          if (!done && SI[w]) { SI[w] &= SI[w] - 1; done = true; }
      }
      uint32_t ma = 0u;
      if (lane < ndI) {
        uint64_t ra[W];
#pragma unroll
        for (int w = 0; w < W; ++w) ra[w] = P.alpha[(d0I + lane) * W + w];
#pragma unroll
        for (int p = 0; p < FAST_MAXOPEN; ++p)
          if (p < nopI) ma |= (uint32_t)bit_w<W>(ra, sI[p]) << p;
      }
#pragma unroll
      for (int p = 0; p < FAST_MAXOPEN; ++p) Ap[p] = __ballot_sync(0xffffffffu, (lane < ndI) && ((ma >> p) & 1u));
#pragma unroll
      for (int k = 0; k <= FAST_MAXOPEN; ++k) Nk[k] = __ballot_sync(0xffffffffu, (lane < ndI) && __popc(ma) == k);
    }
    const int ndblI = P.nelec - nopI;
    const uint32_t rows_valid = (ndI >= 32) ? 0xffffffffu : ((1u << ndI) - 1u);
    __syncwarp();
    for (int i0 = 0; i0 < NIT; i0 += 32) {
      const int it = i0 + lane;
      if (it >= NIT) break;
      int p = 0;  // the neighbour owning item it: last lane whose first item is <= it
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (ws.ipre[p + step] <= it) p += step;
      const int t = it - ws.ipre[p];
      const bool so = ws.so[p] != 0;
      const int nopJ = ws.nopJ[p];
      const int thr = so ? 1 : 2;
      // column SEF t: determinant t (odd electron count), 2t and 2t + 1 (even, open shells)
      // or the configuration's one determinant
      const bool two = !odd && nopJ;
      const int64_t b0 = ws.d0J[p] + (two ? 2 * t : t);
      uint32_t okv[2] = {0u, 0u};
#pragma unroll
      for (int y = 0; y < 2; ++y) {
        if (y == 1 && !two) break;
        uint64_t ja[W], jb[W];
#pragma unroll
        for (int w = 0; w < W; ++w) { ja[w] = __ldg(P.alpha + (b0 + y) * W + w); jb[w] = __ldg(P.beta + (b0 + y) * W + w); }
        int F = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) F += __popcll(ja[w] & ~occI[w]) + __popcll(jb[w] & ~occI[w]);
        if (F > thr) continue;
        // saturating counter over the row dets: S0 (c'=0), S1, S2, S3 (>= 3)
        uint32_t S0 = 0xffffffffu, S1 = 0u, S2 = 0u;
#pragma unroll
        for (int q = 0; q < FAST_MAXOPEN; ++q) {
          if (q >= nopI) break;
          const bool xa = bit_w<W>(ja, sI[q]), yb = bit_w<W>(jb, sI[q]);
          if (xa) {  // mismatch where row det has beta on q
            const uint32_t T = ~Ap[q];
            S2 = (S2 & ~T) | (S1 & T);
            S1 = (S1 & ~T) | (S0 & T);
            S0 &= ~T;
          }
          if (yb) {  // mismatch where row det has alpha on q
            const uint32_t T = Ap[q];
            S2 = (S2 & ~T) | (S1 & T);
            S1 = (S1 & ~T) | (S0 & T);
            S0 &= ~T;
          }
        }
        uint32_t ok = (thr - F >= 2) ? (S0 | S1 | S2) : (thr - F == 1) ? (S0 | S1) : S0;
        ok &= rows_valid;
        if (!so) {
          int na = 0;
#pragma unroll
          for (int w = 0; w < W; ++w) na += __popcll(ja[w]);
          const int need = na - (ndblI / 2);  // alpha open shells a row det needs for equal counts
          uint32_t nk = 0u;
#pragma unroll
          for (int k = 0; k <= FAST_MAXOPEN; ++k)
            if (k == need) nk = Nk[k];
          ok &= (need >= 0 && need <= nopI) ? nk : 0u;
        }
        okv[y] = ok;
      }
      if (odd) {  // row SEF r = row det r, column SEF t = column det t
        uint32_t rows = okv[0];
        while (rows) {
          const int r = __ffs(rows) - 1;
          rows &= rows - 1;
          atomicOr(reinterpret_cast<unsigned long long *>(&ws.C[p][r]), 1ull << t);
        }
      } else {  // row SEF r holds row dets 2r (x = 0) and 2r + 1 (x = 1)
        uint32_t rows = (okv[0] | okv[1]);
        rows = (rows | (rows >> 1)) & 0x55555555u;
        while (rows) {
          const int a = __ffs(rows) - 1;  // 2r
          rows &= rows - 1;
          const uint64_t wd = ((uint64_t)((okv[0] >> a) & 1u) << t) | ((uint64_t)((okv[1] >> a) & 1u) << (t + 16)) |
                              ((uint64_t)((okv[0] >> (a + 1)) & 1u) << (t + 32)) |
                              ((uint64_t)((okv[1] >> (a + 1)) & 1u) << (t + 48));
          atomicOr(reinterpret_cast<unsigned long long *>(&ws.C[p][a >> 1]), (unsigned long long)wd);
        }
      }
    }
    __syncwarp();
    // the words at the pairs' prm positions (pair-major, then row)
    const int64_t prbase = P.pr_off[I] + (k0 - P.nbroff[I]) * nsefI;
    for (int q = lane; q < n * nsefI; q += 32) P.cg[prbase + q] = ws.C[q / nsefI][q % nsefI];
    __syncwarp();
  }
}

// Full rows from the lower pairs.  Row r of configuration I holds, in ascending column order,
// the kept entries of its lower pairs (J <= I, evaluated above; the diagonal block in full)
// and, for every neighbour J > I, column r of the lower block (J, I): the entries whose
// mask bit r is set in the (J, I) pair's rows t.  mk[k] is the position of I in J's list.
//
// One warp per configuration: row lengths, and I's position in each upper neighbour's list.
constexpr int NBR_SKIP = 16;  // one skip-table entry per 16 neighbour-list entries

// skip[q] = nbr[16 q]: the first entry of every 64-byte block of the neighbour lists
__global__ void k_nbr_skip(int64_t nq, const int32_t *__restrict__ nbr, int32_t *__restrict__ skip) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x)
    skip[q] = nbr[q * NBR_SKIP];
}

__global__ void k_mirror_count(Params P, const int32_t *__restrict__ skip, int64_t *row_nnz, int32_t *mk, int *err) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t I = warp; I < P.nconf; I += nwarps) {
    const int64_t b0 = P.nbroff[I], nl = P.nlow[I], nn = P.nbroff[I + 1] - b0;
    const int nsefI = (int)(P.sefoff[I + 1] - P.sefoff[I]);
    int64_t low = 0;
    if (lane < nsefI)
      for (int64_t sg = P.segoff[I]; sg < P.segoff[I + 1]; ++sg) low += P.seg_cnt[P.seg_rowoff[sg] + lane];
    int up[FAST_MAXSEF];
#pragma unroll
    for (int r = 0; r < FAST_MAXSEF; ++r) up[r] = 0;
    for (int64_t k = nl + lane; k < nn; k += 32) {
      const int J = P.nbr[b0 + k];
      const int64_t jb = P.nbroff[J], je = jb + P.nlow[J];
      // I in J's lower list [jb, je) (ascending): the last 16-entry block starting inside
      // the list whose first entry is <= I, by binary search over the skip table (small
      // enough to stay in L2), then a scan of that block (64 bytes)
      int64_t qa = jb / NBR_SKIP, qb = (je - 1) / NBR_SKIP;  // blocks qa + 1 .. qb start inside
      while (qa < qb) {
        const int64_t mid = (qa + qb + 1) >> 1;
        if (__ldg(skip + mid) <= (int32_t)I) qa = mid; else qb = mid - 1;
      }
      int64_t lo = -1;
      const int64_t b16 = qa * NBR_SKIP;
      if (b16 + NBR_SKIP <= P.nbr_len) {  // the block as four 16-byte loads, compared in registers
        const int4 *blk = reinterpret_cast<const int4 *>(P.nbr + b16);
        int4 v[NBR_SKIP / 4];
#pragma unroll
        for (int u = 0; u < NBR_SKIP / 4; ++u) v[u] = __ldg(blk + u);
#pragma unroll
        for (int u = 0; u < NBR_SKIP / 4; ++u) {
          const int64_t p = b16 + 4 * u;
          if (v[u].x == (int32_t)I && p >= jb && p < je) lo = p;
          if (v[u].y == (int32_t)I && p + 1 >= jb && p + 1 < je) lo = p + 1;
          if (v[u].z == (int32_t)I && p + 2 >= jb && p + 2 < je) lo = p + 2;
          if (v[u].w == (int32_t)I && p + 3 >= jb && p + 3 < je) lo = p + 3;
        }
      } else {  // the last, partial block of the lists
        for (int64_t p = max(jb, b16); p < je && p < b16 + NBR_SKIP; ++p)
          if (P.nbr[p] == (int32_t)I) lo = p;
      }
      if (lo < 0) {
        atomicExch(err, 1);
        mk[b0 + k] = -1;
        continue;
      }
      mk[b0 + k] = (int32_t)(lo - jb);
      const int nsefJ = (int)(P.sefoff[J + 1] - P.sefoff[J]);
      const uint64_t *pm = P.prm + P.pr_off[J] + (lo - jb) * nsefJ;
      for (int t = 0; t < nsefJ; ++t) {
        const uint32_t m = (uint32_t)pm[t];
#pragma unroll
        for (int r = 0; r < FAST_MAXSEF; ++r) up[r] += (int)((m >> r) & 1u);
      }
    }
    int mine = 0;
#pragma unroll
    for (int r = 0; r < FAST_MAXSEF; ++r) {
      int v = up[r];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == r) mine = v;
    }
    if (lane < nsefI) row_nnz[P.sefoff[I] + lane] = low + mine;
  }
}

// One warp per configuration: columns, values (and the FP32 copy and the diagonal) of its
// rows; lane r carries the write position of row r.  Entries are spread over the lanes one
// per lane (e = lane, lane + 32, ...), so consecutive lanes write consecutive positions:
// the lane that owns entry e is found by binary search over the per-pair offsets.
constexpr int ASM_THREADS = 256;
__global__ void __launch_bounds__(ASM_THREADS) k_assemble(Params P, const int32_t *mk) {
  __shared__ int s_off[ASM_THREADS / 32][33];     // per lane: first entry of the lane in the row
  __shared__ int s_soff[ASM_THREADS / 32][32];    // lower part: per row, its first entry in the segment
  __shared__ uint32_t s_msk[ASM_THREADS / 32][32];  // per lane: columns t of the run, as bits
  __shared__ int32_t s_J[ASM_THREADS / 32][32];
  __shared__ int64_t s_col[ASM_THREADS / 32][32];
  __shared__ uint64_t s_mm[ASM_THREADS / 32][32][FAST_MAXSEF];  // mask words (prm)
  __shared__ int16_t s_ro[ASM_THREADS / 32][FAST_MAXSEF][32];  // lower part: per row, first entry of each slot
  __shared__ int64_t s_dst[ASM_THREADS / 32][FAST_MAXSEF];      // lower part: per row, its write position
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t I = warp; I < P.nconf; I += nwarps) {
    const int64_t row0 = P.sefoff[I];
    const int nsefI = (int)(P.sefoff[I + 1] - row0);
    const int64_t b0 = P.nbroff[I], nl = P.nlow[I], nn = P.nbroff[I + 1] - b0;
    int64_t mypos = (lane < nsefI) ? P.rowptr[row0 + lane] : 0;
    // lower pairs, segment by segment: the run of (segment, row r) is contiguous in the slab
    // and in row r, in the same order.  The segment's runs and mask words are loaded first;
    // then its entries, all rows together, are numbered in (row, neighbour, column) order
    // and spread evenly over the lanes.
    for (int64_t sg = P.segoff[I]; sg < P.segoff[I + 1]; ++sg) {
      const int64_t k0 = P.seg_k0[sg];
      const int ns = P.seg_n[sg];
      if (lane < ns) {
        const int J = P.nbr[k0 + lane];
        s_J[wib][lane] = J;
        s_col[wib][lane] = P.sefoff[J];
      }
      // mask words of (neighbour o, row r): contiguous in prm, pair-major
      const uint64_t *pm = P.prm + P.pr_off[I] + (k0 - b0) * nsefI;
      for (int q = lane; q < ns * nsefI; q += 32) s_mm[wib][q / nsefI][q % nsefI] = pm[q];
      // row r (lane r): its entry count and its first entry in the segment
      int cnt = 0;
      if (lane < nsefI) {
        cnt = (int)P.seg_cnt[P.seg_rowoff[sg] + lane];
        s_dst[wib][lane] = mypos;
      }
      int rincl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, rincl, o);
        if (lane >= o) rincl += v;
      }
      const int T = __shfl_sync(0xffffffffu, rincl, 31);
      s_soff[wib][lane] = rincl - cnt;
      __syncwarp();
      // per row, the first entry of each neighbour: the row takes the pairs in neighbour
      // order; the slab run holds them in the evaluation order, each where its prm word says
      for (int r = 0; r < nsefI; ++r) {
        const int cl = (lane < ns) ? __popc(s_mm[wib][lane][r] & 0xffffu) : 0;
        int incl = cl;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        s_ro[wib][r][lane] = (int16_t)(incl - cl);
      }
      __syncwarp();
      for (int e = lane; e < T; e += 32) {
        int r = 0;  // the row of entry e: last row whose first entry is <= e
#pragma unroll
        for (int st = 8; st > 0; st >>= 1)
          if (r + st < nsefI && s_soff[wib][r + st] <= e) r += st;
        const int el = e - s_soff[wib][r];
        int o = 0;  // its neighbour: last slot whose first entry in the row is <= el
#pragma unroll
        for (int st = 16; st > 0; st >>= 1)
          if (o + st < 32 && s_ro[wib][r][o + st] <= el) o += st;
        const uint64_t w = s_mm[wib][o][r];
        const int k = el - s_ro[wib][r][o];
        uint32_t m = (uint32_t)w & 0xffffu;
        for (int q = k; q > 0; --q) m &= m - 1;
        const int t = __ffs(m) - 1;
        const double v = P.slab_val[(int64_t)(w >> 16) + k];
        const int64_t dst = s_dst[wib][r] + el;
        P.col[dst] = (int32_t)(s_col[wib][o] + t);
        P.val[dst] = v;
        if (P.val32) P.val32[dst] = (float)v;
        if (s_J[wib][o] == (int)I && t == r) P.diag[row0 + r] = v;
      }
      __syncwarp();
      mypos += cnt;
    }
    // upper neighbours, 32 at a time: column r of their lower block (J, I)
    for (int64_t kc = nl; kc < nn; kc += 32) {
      const int64_t k = kc + lane;
      uint32_t mm[FAST_MAXSEF];  // kept-column masks of the block's rows t
#pragma unroll
      for (int t = 0; t < FAST_MAXSEF; ++t) mm[t] = 0u;
      int64_t colJ = 0;
      if (k < nn) {
        const int J = P.nbr[b0 + k];
        const int kk = mk[b0 + k];
        if (kk >= 0) {
          const int nsefJ = (int)(P.sefoff[J + 1] - P.sefoff[J]);
          colJ = P.sefoff[J];
          const uint64_t *pm = P.prm + P.pr_off[J] + (int64_t)kk * nsefJ;
#pragma unroll
          for (int t = 0; t < FAST_MAXSEF; ++t)
            if (t < nsefJ) {
              const uint64_t w = pm[t];
              s_mm[wib][lane][t] = w;
              mm[t] = (uint32_t)w & 0xffffu;
            }
        }
      }
      s_col[wib][lane] = colJ;
      for (int r = 0; r < nsefI; ++r) {
        uint32_t cm = 0u;  // columns t of this lane's block whose row t keeps column r
#pragma unroll
        for (int t = 0; t < FAST_MAXSEF; ++t) cm |= ((mm[t] >> r) & 1u) << t;
        const int cnt = __popc(cm);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int tot = __shfl_sync(0xffffffffu, incl, 31);
        const int64_t dst = __shfl_sync(0xffffffffu, mypos, r);
        s_off[wib][lane] = incl - cnt;
        s_msk[wib][lane] = cm;
        __syncwarp();
        const uint32_t below = (1u << r) - 1u;
        for (int e = lane; e < tot; e += 32) {
          int o = 0;
#pragma unroll
          for (int st = 16; st > 0; st >>= 1)
            if (o + st < 32 && s_off[wib][o + st] <= e) o += st;
          uint32_t m = s_msk[wib][o];
          for (int q = e - s_off[wib][o]; q > 0; --q) m &= m - 1;
          const int t = __ffs(m) - 1;
          const uint64_t wt = s_mm[wib][o][t];
          const double v = P.slab_val[(int64_t)(wt >> 16) + __popc((uint32_t)wt & below)];
          P.col[dst + e] = (int32_t)(s_col[wib][o] + t);
          P.val[dst + e] = v;
          if (P.val32) P.val32[dst + e] = (float)v;
        }
        __syncwarp();
        if (lane == r) mypos += tot;
      }
      __syncwarp();
    }
  }
}

// generateSOCIblocks for an explicit list of (A, B) pairs: the full nsef_A x nsef_B block,
// row-major, at out + outoff[p] (reference roles, no transposition or mirroring)
template <int W>
__global__ void __launch_bounds__(WARPS_PER_CTA * 32) k_blocks(Params P, int npairs, const int32_t *pa,
                                                               const int32_t *pb, const int64_t *outoff,
                                                               double *out) {
  __shared__ PairInfo spi[WARPS_PER_CTA];
  __shared__ double sK[WARPS_PER_CTA][MAXK];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t q = warp; q < npairs; q += nwarps) {
    const int A = pa[q], B = pb[q];
    if (lane == 0) pair_setup_ab<W>(P, A, B, B, 0, spi[wib], sK[wib]);
    __syncwarp();
    const int na = (int)(P.sefoff[A + 1] - P.sefoff[A]), nb = (int)(P.sefoff[B + 1] - P.sefoff[B]);
    for (int e = lane; e < na * nb; e += 32) {
      int a = e / nb, b = e - a * nb;
      out[outoff[q] + e] = sef_elem<W>(P, spi[wib], sK[wib], a, b);
    }
    __syncwarp();
  }
}

template <int W>
psoci_status run_blocks(psoci_ctx *c, int npairs, const int32_t *hA, const int32_t *hB, double *hout) {
  std::vector<int64_t> off(npairs + 1, 0);
  for (int q = 0; q < npairs; ++q) {
    if (hA[q] < 0 || hA[q] >= c->nconf || hB[q] < 0 || hB[q] >= c->nconf)
      return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "blocks: configuration index out of range");
    int64_t na = c->h_sefoff[hA[q] + 1] - c->h_sefoff[hA[q]], nb = c->h_sefoff[hB[q] + 1] - c->h_sefoff[hB[q]];
    off[q + 1] = off[q] + na * nb;
  }
  Params P = {};
  P.nconf = c->nconf; P.nbf = c->nbf; P.nelec = c->nelec; P.ksym = c->ksym;
  P.e1 = c->d_e1; P.e2 = c->d_e2; P.jsym = c->d_jsym; P.nopen = c->d_nopen;
  P.sefoff = c->d_sefoff; P.detoff = c->d_detoff;
  P.alpha = c->d_alpha; P.beta = c->d_beta; P.phase = c->d_phase; P.nalpha = c->d_nalpha;
  P.one = c->d_one; P.eri = c->d_eri;
  int32_t *dA = nullptr, *dB = nullptr;
  int64_t *doff = nullptr;
  double *dout = nullptr;
  psoci_status s;
  if ((s = psoci_alloc(c, &dA, npairs)) || (s = psoci_alloc(c, &dB, npairs)) || (s = psoci_alloc(c, &doff, npairs + 1)) ||
      (s = psoci_alloc(c, &dout, off[npairs]))) {
    psoci_free(dA); psoci_free(dB); psoci_free(doff); psoci_free(dout);
    return s;
  }
  cudaStream_t st = c->stream;
  cudaMemcpyAsync(dA, hA, sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dB, hB, sizeof(int32_t) * npairs, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * (npairs + 1), cudaMemcpyHostToDevice, st);
  int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((npairs + WARPS_PER_CTA - 1) / WARPS_PER_CTA, 152 * 16));
  psoci_note_launch();
  k_blocks<W><<<blocks, WARPS_PER_CTA * 32, 0, st>>>(P, npairs, dA, dB, doff, dout);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(hout, dout, sizeof(double) * off[npairs], cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  psoci_free(dA); psoci_free(dB); psoci_free(doff); psoci_free(dout);
  if (e != cudaSuccess) return psoci_cuda_fail(c, e, "blocks");
  return PSOCI_OK;
}

// Neighbour lists of every configuration: the configurations within two excitations (sorted),
// less the pairs whose block the integral tables prune_one / prune_eri make zero (the build
// passes the Hamiltonian's own tables; a table of ones keeps every pair).  Lookup screen for
// MRCI-type spaces, all-pairs test otherwise.  d_nbroff [nconf+1] and d_nbr [npairs] are
// allocated here and owned by the caller.
template <int W>
psoci_status screen_pairs(psoci_ctx *c, const Params &P0, const double *prune_one, const double *prune_eri,
                          int64_t *&d_nbroff, int32_t *&d_nbr, int64_t &ncand, int64_t &npairs, int &nsplit) {
  cudaStream_t st = c->stream;
  const int n = c->nconf;
  Params P = P0;
  P.one = prune_one;
  P.eri = prune_eri;
  psoci_status s;
  int64_t *d_cnt = nullptr, *d_soff = nullptr, *d_tot = nullptr, *d_candoff = nullptr;
  int32_t *d_cand = nullptr;
  int64_t *d_gcnt = nullptr, *d_goff = nullptr;
  uint32_t *d_glist = nullptr;
  unsigned long long *d_counter = nullptr;
  int32_t *d_jslab = nullptr;
  int64_t *d_jstart = nullptr;
  int2 *d_tpairs = nullptr;
  uint32_t *d_dkept = nullptr;
  ncand = npairs = 0;
  nsplit = 0;
  auto cleanup = [&]() {
    psoci_free(d_cnt); psoci_free(d_soff); psoci_free(d_tot); psoci_free(d_candoff); psoci_free(d_cand);
    psoci_free(d_gcnt); psoci_free(d_goff); psoci_free(d_glist); psoci_free(d_counter); psoci_free(d_jslab);
    psoci_free(d_jstart); psoci_free(d_tpairs); psoci_free(d_dkept);
  };
  auto fail = [&]() {
    cleanup();
    psoci_free(d_nbroff);
    psoci_free(d_nbr);
  };
#define TRY(x)                 \
  do {                         \
    s = (x);                   \
    if (s != PSOCI_OK) {       \
      fail();                  \
      return s;                \
    }                          \
  } while (0)
#define TRYC(x)                                  \
  do {                                          \
    cudaError_t _e = (x);                       \
    if (_e != cudaSuccess) {                    \
      s = psoci_cuda_fail(c, _e, #x);           \
      fail();                                   \
      return s;                                 \
    }                                           \
  } while (0)
  if (c->join_ok) {
    // by lookup, with the integral pruning fused
    JoinTabs J = {c->join_s, c->join_G, c->join_L, c->d_jgid, c->d_jlid, c->d_jT, c->d_jlnoff, c->d_jln,
                  c->d_jhdec, c->d_jlokey, nullptr, nullptr, nullptr, 0};
    // hi-pattern lists (depend on the integrals, so built here)
    const int G = c->join_G;
    TRY(psoci_alloc(c, &d_gcnt, G + 1));
    TRY(psoci_alloc(c, &d_goff, G + 1));
    const int gblocks = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)G * 32 + 255) / 256, 152 * 32));
    psoci_note_launch();
    k_group_lists<W, 0><<<gblocks, 256, 0, st>>>(J, prune_eri, d_gcnt, nullptr);
    TRYC(cudaGetLastError());
    int64_t nglist = 0;
    TRY(psoci_scan_i64(c, d_gcnt, d_goff, G, &nglist));
    TRY(psoci_alloc(c, &d_glist, nglist));
    J.goff = d_goff;
    psoci_note_launch();
    k_group_lists<W, 1><<<gblocks, 256, 0, st>>>(J, prune_eri, nullptr, d_glist);
    TRYC(cudaGetLastError());
    J.glist = d_glist;
    {
      // pruning bits of all double excitations (depend on the integrals)
      const int64_t nt = (int64_t)c->nbf * (c->nbf + 1) / 2;
      std::vector<int2> pairs((size_t)nt);
      for (int a = 0; a < c->nbf; ++a)
        for (int b = 0; b <= a; ++b) pairs[(size_t)a * (a + 1) / 2 + b] = make_int2(b, a);  // (low, high)
      TRY(psoci_alloc(c, &d_tpairs, nt));
      TRY(psoci_alloc(c, &d_dkept, (nt * nt + 31) / 32));
      TRYC(cudaMemcpyAsync(d_tpairs, pairs.data(), sizeof(int2) * nt, cudaMemcpyHostToDevice, st));
      psoci_note_launch();
      k_double_kept<<<152 * 8, 256, 0, st>>>(nt, d_tpairs, prune_eri, d_dkept);
      TRYC(cudaGetLastError());
      TRYC(cudaStreamSynchronize(st));  // pairs is a host buffer
      J.dkept = d_dkept;
      J.nt = nt;
    }
    TRY(psoci_alloc(c, &d_cnt, n + 1));
    TRY(psoci_alloc(c, &d_tot, n + 1));
    TRY(psoci_alloc(c, &d_candoff, n + 1));
    TRY(psoci_alloc(c, &d_nbroff, n + 1));
    const int jblocks = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n * 32 + 255) / 256, 152 * 32));
    // single pass into a slab sized from the last build of this space (or 1024 neighbours
    // a configuration plus the warps' chunk tails), then a compaction copy; the count and
    // write passes remain for a slab that turns out too small
    JoinSlab S = {};
    bool single = false;
    {
      size_t freeb = 0, totb = 0;
      TRYC(cudaMemGetInfo(&freeb, &totb));
      const int64_t tails = (int64_t)jblocks * 8 * 2 * JOIN_CHUNK;
      int64_t cap = std::max<int64_t>(c->join_hint + c->join_hint / 8, 1024 * (int64_t)n) + tails;
      cap = std::min<int64_t>(cap, (int64_t)(freeb * 0.4) / 4);
      if (psoci_alloc(c, &d_jslab, cap) == PSOCI_OK && psoci_alloc(c, &d_jstart, n + 1) == PSOCI_OK &&
          psoci_alloc(c, &d_counter, 1) == PSOCI_OK) {
        TRYC(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st));
        S = {d_jslab, d_counter, cap, d_jstart};
        psoci_note_launch();
        k_join<W, 2><<<jblocks, 256, 0, st>>>(P, J, d_cnt, d_tot, nullptr, S);
        TRYC(cudaGetLastError());
        unsigned long long used = 0;
        TRYC(cudaMemcpyAsync(&used, d_counter, sizeof(used), cudaMemcpyDeviceToHost, st));
        TRYC(cudaStreamSynchronize(st));
        if ((int64_t)used <= cap) {
          TRY(psoci_scan_i64(c, d_tot, d_candoff, n, &ncand));
          TRY(psoci_scan_i64(c, d_cnt, d_nbroff, n, &npairs));
          TRY(psoci_alloc(c, &d_nbr, npairs));
          psoci_note_launch();
          k_join_compact<<<jblocks, 256, 0, st>>>(n, d_jslab, d_jstart, d_nbroff, d_nbr);
          TRYC(cudaGetLastError());
          single = true;
        }
        c->join_hint = (int64_t)used;
      } else {
        cudaGetLastError();  // no room for the slab: the two passes below
      }
      TRYC(cudaStreamSynchronize(st));
      psoci_free(d_jslab);
      psoci_free(d_jstart);
      psoci_free(d_counter);
    }
    if (!single) {
      psoci_note_launch();
      k_join<W, 0><<<jblocks, 256, 0, st>>>(P, J, d_cnt, d_tot, nullptr, S);
      TRYC(cudaGetLastError());
      TRY(psoci_scan_i64(c, d_tot, d_candoff, n, &ncand));
      TRY(psoci_scan_i64(c, d_cnt, d_nbroff, n, &npairs));
      TRY(psoci_alloc(c, &d_nbr, npairs));
      P.nbroff = d_nbroff; P.nbr = d_nbr;
      psoci_note_launch();
      k_join<W, 1><<<jblocks, 256, 0, st>>>(P, J, nullptr, nullptr, d_nbroff, S);
      TRYC(cudaGetLastError());
    }
    P.nbroff = d_nbroff; P.nbr = d_nbr;
  } else {
  const int scr_rows = (n + SCR_THREADS * SCR_ROWS - 1) / (SCR_THREADS * SCR_ROWS);
  nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(64, (152 * 8 + scr_rows - 1) / scr_rows));
  int64_t chunk = ((int64_t)n + nsplit - 1) / nsplit;
  chunk = std::max<int64_t>(chunk, SCR_TILE);
  nsplit = (int)((n + chunk - 1) / chunk);
  TRY(psoci_alloc(c, &d_cnt, (size_t)nsplit * n + 1));
  TRY(psoci_alloc(c, &d_soff, (size_t)nsplit * n + 1));
  TRY(psoci_alloc(c, &d_tot, n + 1));
  TRY(psoci_alloc(c, &d_candoff, n + 1));
  TRY(psoci_alloc(c, &d_nbroff, n + 1));
  dim3 scr_grid(scr_rows, nsplit);
  psoci_note_launch();
  k_screen<W, 0><<<scr_grid, SCR_THREADS, 0, st>>>(P, d_cnt, nullptr, chunk, nullptr, nullptr);
  TRYC(cudaGetLastError());
  psoci_note_launch();
  k_screen_offsets<<<(n + 255) / 256, 256, 0, st>>>(n, nsplit, d_cnt, d_soff, d_tot);
  TRYC(cudaGetLastError());
  TRY(psoci_scan_i64(c, d_tot, d_candoff, n, &ncand));
  TRY(psoci_alloc(c, &d_cand, ncand));
  psoci_note_launch();
  k_screen<W, 1><<<scr_grid, SCR_THREADS, 0, st>>>(P, nullptr, d_soff, chunk, d_candoff, d_cand);
  TRYC(cudaGetLastError());
  const int prune_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n * 32 + 255) / 256, 152 * 32));
  psoci_note_launch();
  k_prune<W, 0><<<prune_blocks, 256, 0, st>>>(P, d_candoff, d_cand, d_tot);
  TRYC(cudaGetLastError());
  TRY(psoci_scan_i64(c, d_tot, d_nbroff, n, &npairs));
  TRY(psoci_alloc(c, &d_nbr, npairs));
  P.nbroff = d_nbroff; P.nbr = d_nbr;
  psoci_note_launch();
  k_prune<W, 1><<<prune_blocks, 256, 0, st>>>(P, d_candoff, d_cand, nullptr);
  TRYC(cudaGetLastError());
  psoci_free(d_cand);
  }
  cleanup();
  return PSOCI_OK;
#undef TRY
#undef TRYC
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
  int64_t *d_soff = nullptr, *d_tot = nullptr, *d_candoff = nullptr;
  int64_t *d_nlow = nullptr, *d_prrows = nullptr, *d_proff = nullptr;
  int32_t *d_cand = nullptr, *d_mk = nullptr, *d_skip = nullptr;
  int64_t *d_gcnt = nullptr, *d_goff = nullptr;
  uint32_t *d_glist = nullptr;
  uint64_t *d_prm = nullptr;
  uint64_t *d_cg = nullptr;
  int *d_err = nullptr;
  unsigned long long *d_counter = nullptr;
  double *d_slabval = nullptr;
  int32_t *d_jslab = nullptr;
  int64_t *d_jstart = nullptr;
  int2 *d_tpairs = nullptr;
  uint32_t *d_dkept = nullptr;
  cudaEvent_t ev[6] = {};
  auto cleanup = [&]() {
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    psoci_free(d_soff); psoci_free(d_tot); psoci_free(d_counter);
    psoci_free(d_candoff); psoci_free(d_cand); psoci_free(d_skip);
    psoci_free(d_nlow); psoci_free(d_prrows); psoci_free(d_proff); psoci_free(d_mk); psoci_free(d_prm); psoci_free(d_cg);
    psoci_free(d_err); psoci_free(d_slabval); psoci_free(d_jslab); psoci_free(d_jstart);
    psoci_free(d_tpairs); psoci_free(d_dkept);
    psoci_free(d_gcnt); psoci_free(d_goff); psoci_free(d_glist);
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

  auto tnow = [&]() {
    if (c->verbose) cudaStreamSynchronize(st);
    return std::chrono::steady_clock::now();
  };
  for (auto &e : ev) TRYC(cudaEventCreate(&e));
  TRYC(cudaEventRecord(ev[0], st));
  auto t_a = tnow();
  // 1. screen
  int64_t ncand = 0, npairs = 0;
  int nsplit = 0;
  TRY(screen_pairs<W>(c, P, c->d_one, c->d_eri, d_nbroff, d_nbr, ncand, npairs, nsplit));
  P.nbroff = d_nbroff; P.nbr = d_nbr;
  c->ncand = ncand;
  c->npairs = npairs;
  TRYC(cudaEventRecord(ev[1], st));
  auto t_b = tnow();

  // fast path: only the lower pairs (J <= I) are evaluated; the rest are mirrored
  const bool direct = (mode == PSOCI_HMODE_DIRECT);
  const bool fast = !direct && c->max_ndet <= FAST_MAXDET;
  int64_t nprm = 0;
  bool split = false;  // fast path: masks and elements in two launches
  if (fast) {
    TRY(psoci_alloc(c, &d_nlow, n + 1));
    TRY(psoci_alloc(c, &d_prrows, n + 1));
    TRY(psoci_alloc(c, &d_proff, n + 1));
    psoci_note_launch();
    k_lower_counts<<<(n + 255) / 256, 256, 0, st>>>(n, d_nbroff, d_nbr, c->d_sefoff, d_nlow, d_prrows);
    TRYC(cudaGetLastError());
    TRY(psoci_scan_i64(c, d_prrows, d_proff, n, &nprm));
    TRY(psoci_alloc(c, &d_prm, nprm));
    P.nlow = d_nlow; P.pr_off = d_proff; P.prm = d_prm;
  }

  // 2. segments
  TRY(psoci_alloc(c, &d_nseg, n + 1));
  TRY(psoci_alloc(c, &d_nrow, n + 1));
  TRY(psoci_alloc(c, &d_segoff, n + 1));
  TRY(psoci_alloc(c, &d_rowslot, n + 1));
  psoci_note_launch();
  k_seg_counts<<<(n + 255) / 256, 256, 0, st>>>(n, d_nbroff, d_nlow, c->d_sefoff, d_nseg, d_nrow);
  TRYC(cudaGetLastError());
  int64_t nseg = 0, nslots = 0;
  TRY(psoci_scan_i64(c, d_nseg, d_segoff, n, &nseg));
  TRY(psoci_scan_i64(c, d_nrow, d_rowslot, n, &nslots));
  TRY(psoci_alloc(c, &d_segcfg, nseg));
  TRY(psoci_alloc(c, &d_segk0, nseg));
  TRY(psoci_alloc(c, &d_segn, nseg));
  TRY(psoci_alloc(c, &d_segrow, nseg));
  TRY(psoci_alloc(c, &d_segcnt, nslots));
  psoci_note_launch();
  k_seg_init<<<(n + 255) / 256, 256, 0, st>>>(n, d_nbroff, d_nlow, c->d_sefoff, d_segoff, d_rowslot, d_segcfg, d_segk0,
                                              d_segn, d_segrow);
  TRYC(cudaGetLastError());
  c->nseg = nseg;
  P.nseg = nseg; P.seg_cfg = d_segcfg; P.seg_k0 = d_segk0; P.seg_n = d_segn; P.seg_rowoff = d_segrow;
  P.seg_cnt = d_segcnt; P.segoff = d_segoff;

  // 3. evaluate
  int hb_blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nseg + WARPS_PER_CTA - 1) / WARPS_PER_CTA, 152 * 16));
  const int64_t N = c->nsef_total;
  int64_t nnz = 0, slab_used = 0;
  int evaluations = 0;
  auto t_c = tnow();
  auto t_d = t_c, t_e = t_c;
  if (direct) {
    // direct mode: the diagonal now, the other elements in every sigma; the neighbour lists
    // and segments move to the context
    TRY(psoci_alloc(c, &c->d_diag, N));
    P.diag = c->d_diag;
    const size_t smem = sizeof(WarpSmem) * WARPS_PER_CTA;
    TRYC(cudaFuncSetAttribute(k_hbuild<W, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    TRYC(cudaEventRecord(ev[2], st));
    psoci_note_launch();
    k_hbuild<W, 3><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
    TRYC(cudaGetLastError());
    TRYC(cudaEventRecord(ev[3], st));
    TRYC(cudaEventRecord(ev[4], st));
    TRYC(cudaEventRecord(ev[5], st));
    TRYC(cudaStreamSynchronize(st));
    c->dir_nbroff = d_nbroff; d_nbroff = nullptr;
    c->dir_nbr = d_nbr; d_nbr = nullptr;
    c->dir_segcfg = d_segcfg; d_segcfg = nullptr;
    c->dir_segk0 = d_segk0; d_segk0 = nullptr;
    c->dir_segn = d_segn; d_segn = nullptr;
    c->direct = true;
  } else if (fast) {
    // 3. evaluate the lower pairs once: kept values go to slab slots, masks to prm
    const size_t smem = sizeof(FastSmem<W>) * WARPS_PER_CTA;
    TRYC(cudaFuncSetAttribute(k_hbuild_fast<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // two launches when the masks fit (8 bytes per (pair, row SEF), a quarter of the free
    // memory at most): the connectivity masks (k_hbuild_masks), then the elements from them;
    // otherwise both phases in one launch
    size_t freeb = 0, totb = 0;
    TRYC(cudaMemGetInfo(&freeb, &totb));
    split = c->eval_launches != 1 && (double)nprm * 8.0 <= 0.25 * (double)freeb;
    if (split) {
      TRYC(cudaFuncSetAttribute(k_hbuild_fast<W, 0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      TRY(psoci_alloc(c, &d_cg, nprm));
      P.cg = d_cg;
    }
    TRY(psoci_alloc(c, &d_counter, 1));
    TRYC(cudaMemGetInfo(&freeb, &totb));
    // slots hold the kept elements of the lower pairs plus the unused tails of the warps'
    // chunks; first guess from the pair count (observed up to 7 kept elements per lower
    // pair; (npairs + nconf) / 2 lower pairs) or from the previous build of the same space;
    // an overflow is detected by the kernel's counter and the evaluation repeats with the
    // exact size
    const int64_t tails = (int64_t)hb_blocks * WARPS_PER_CTA * SLAB_CHUNK;
    int64_t cap = std::max<int64_t>(4 * npairs + 4 * (int64_t)n, c->slab_hint) + tails;
    cap = std::min<int64_t>((int64_t)(freeb * 0.5) / 8, cap);
    int64_t nlower = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
      auto t_al = std::chrono::steady_clock::now();
      TRY(psoci_alloc(c, &d_slabval, cap));
      if (c->verbose)
        fprintf(stderr, "psoci: H build slab allocation %.4f s (%lld slots)\n",
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t_al).count(), (long long)cap);
      TRYC(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), st));
      P.slab_counter = d_counter; P.slab_cap = cap; P.slab_val = d_slabval;
      TRYC(cudaEventRecord(ev[2], st));
      if (split && attempt == 0) {
        const int mblocks = (int)std::max<int64_t>(1, std::min<int64_t>((nseg + MASK_WARPS - 1) / MASK_WARPS, 152 * 8));
        psoci_note_launch();
        k_hbuild_masks<W><<<mblocks, MASK_WARPS * 32, 0, st>>>(P);
        TRYC(cudaGetLastError());
      }
      psoci_note_launch();
      if (split) k_hbuild_fast<W, 0, 2><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
      else k_hbuild_fast<W><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
      TRYC(cudaGetLastError());
      TRYC(cudaEventRecord(ev[3], st));
      ++evaluations;
      unsigned long long used = 0;
      TRYC(cudaMemcpyAsync(&used, d_counter, sizeof(used), cudaMemcpyDeviceToHost, st));
      TRYC(cudaStreamSynchronize(st));
      nlower = (int64_t)used;
      if (c->verbose)
        fprintf(stderr, "psoci: H build slab %lld of %lld slots used\n", (long long)nlower, (long long)cap);
      if (nlower <= cap) break;
      psoci_free(d_slabval);
      cap = nlower + tails;  // chunk tails differ from run to run
      if (attempt == 1) TRY(psoci_fail(c, PSOCI_ERR_NOMEM, "H build: element slab overflow"));
    }
    psoci_free(d_cg);  // the masks are done with
    t_d = tnow();
    // 4. full row lengths (lower counts + mirrored columns) and offsets
    TRY(psoci_alloc(c, &d_rownnz, N + 1));
    TRY(psoci_alloc(c, &d_mk, npairs));
    TRY(psoci_alloc(c, &d_err, 1));
    TRYC(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    const int cfg_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n * 32 + 255) / 256, 152 * 32));
    const int64_t nq = (npairs + NBR_SKIP - 1) / NBR_SKIP;
    P.nbr_len = npairs;
    TRY(psoci_alloc(c, &d_skip, nq));
    psoci_note_launch();
    k_nbr_skip<<<(int)std::min<int64_t>((nq + 255) / 256, 152 * 16), 256, 0, st>>>(nq, d_nbr, d_skip);
    TRYC(cudaGetLastError());
    psoci_note_launch();
    k_mirror_count<<<cfg_blocks, 256, 0, st>>>(P, d_skip, d_rownnz, d_mk, d_err);
    TRYC(cudaGetLastError());
    int herr = 0;
    TRYC(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TRY(psoci_alloc(c, &c->d_rowptr, N + 1));
    TRY(psoci_scan_i64(c, d_rownnz, c->d_rowptr, N, &nnz));
    if (herr) TRY(psoci_fail(c, PSOCI_ERR_CUDA, "H build: neighbour lists are not symmetric"));
    TRYC(cudaEventRecord(ev[4], st));
    slab_used = nlower;
    c->slab_hint = nlower;
    if (nnz < N) TRY(psoci_fail(c, PSOCI_ERR_CUDA, "H build: rows without their diagonal element"));
    TRY(psoci_alloc(c, &c->d_col, nnz));
    TRY(psoci_alloc(c, &c->d_val, nnz));
    if (mode == PSOCI_HMODE_CSR_BOTH) TRY(psoci_alloc(c, &c->d_val32, nnz));
    TRY(psoci_alloc(c, &c->d_diag, N));
    P.rowptr = c->d_rowptr; P.col = c->d_col; P.val = c->d_val; P.val32 = c->d_val32; P.diag = c->d_diag;
    t_e = tnow();
    // 5. ordered assembly
    psoci_note_launch();
    k_assemble<<<cfg_blocks, ASM_THREADS, 0, st>>>(P, d_mk);
    TRYC(cudaGetLastError());
    TRYC(cudaEventRecord(ev[5], st));
    TRYC(cudaStreamSynchronize(st));
  } else {
    const size_t smem = sizeof(WarpSmem) * WARPS_PER_CTA;
    TRYC(cudaFuncSetAttribute(k_hbuild<W, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    TRYC(cudaFuncSetAttribute(k_hbuild<W, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // 3. count
    TRYC(cudaEventRecord(ev[2], st));
    psoci_note_launch();
    k_hbuild<W, 0><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
    TRYC(cudaGetLastError());
    TRYC(cudaEventRecord(ev[3], st));
    ++evaluations;
    t_d = tnow();
    // 4. offsets
    TRY(psoci_alloc(c, &d_rownnz, N + 1));
    psoci_note_launch();
    k_seg_rowscan<<<(n + 127) / 128, 128, 0, st>>>(n, c->d_sefoff, d_segoff, d_segrow, d_segcnt, d_rownnz);
    TRYC(cudaGetLastError());
    TRY(psoci_alloc(c, &c->d_rowptr, N + 1));
    TRY(psoci_scan_i64(c, d_rownnz, c->d_rowptr, N, &nnz));
    TRYC(cudaEventRecord(ev[4], st));
    TRY(psoci_alloc(c, &c->d_col, nnz));
    TRY(psoci_alloc(c, &c->d_val, nnz));
    if (mode == PSOCI_HMODE_CSR_BOTH) TRY(psoci_alloc(c, &c->d_val32, nnz));
    TRY(psoci_alloc(c, &c->d_diag, N));
    P.rowptr = c->d_rowptr; P.col = c->d_col; P.val = c->d_val; P.val32 = c->d_val32; P.diag = c->d_diag;
    t_e = tnow();
    // 5. fill
    psoci_note_launch();
    k_hbuild<W, 1><<<hb_blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
    TRYC(cudaGetLastError());
    TRYC(cudaEventRecord(ev[5], st));
    TRYC(cudaStreamSynchronize(st));
  }
  auto t_f = std::chrono::steady_clock::now();
  if (c->verbose) {
    auto d = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count(); };
    fprintf(stderr,
            "psoci: H build phases (%s kernel%s, %s screen): screen %.4f s, segments %.4f s, evaluate %.4f s, "
            "offsets %.4f s, fill/copy %.4f s\n",
            fast ? "fast" : "generic", split ? ", masks launched apart" : "", nsplit ? "all-pairs" : "lookup",
            d(t_a, t_b), d(t_b, t_c), d(t_c, t_d),
            d(t_d, t_e), d(t_e, t_f));
  }
  {
    psoci_build_info &b = c->binfo;
    b = psoci_build_info{};
    b.candidates = ncand; b.pairs = npairs; b.segments = nseg; b.nnz = nnz; b.nnz_lower = direct ? 0 : (nnz + N) / 2;
    b.slab_slots = slab_used; b.evaluations = evaluations; b.fast = fast ? 1 : 0;
    b.lookup_screen = c->join_ok ? 1 : 0;
    b.eval_launches = fast ? (split ? 2 : 1) : 0;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess) b.screen_ms = ms;
    if (cudaEventElapsedTime(&ms, ev[2], ev[3]) == cudaSuccess) b.evaluate_ms = ms;
    if (cudaEventElapsedTime(&ms, ev[3], ev[4]) == cudaSuccess) b.rows_ms = ms;
    if (cudaEventElapsedTime(&ms, ev[4], ev[5]) == cudaSuccess) b.assemble_ms = ms;
    if (cudaEventElapsedTime(&ms, ev[0], ev[5]) == cudaSuccess) b.total_ms = ms;
  }
  cleanup();
  c->nnz = nnz;
  *nnz_out = nnz;
  return PSOCI_OK;
#undef TRY
#undef TRYC
}

// X (FP64, leading dim ldx, k <= 8 columns) -> X32 (FP32, row stride 8, zero padded)
__global__ void k_direct_x32(int64_t n, int k, const double *__restrict__ x, int ldx, float *__restrict__ x32) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    float f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) f[q] = (q < k) ? (float)x[r * ldx + q] : 0.f;
    float4 *d = reinterpret_cast<float4 *>(x32 + r * 8);
    d[0] = make_float4(f[0], f[1], f[2], f[3]);
    d[1] = make_float4(f[4], f[5], f[6], f[7]);
  }
}

template <int W>
psoci_status run_direct_sigma(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy, psoci_prec prec,
                              float *x32) {
  cudaStream_t st = c->stream;
  Params P = {};
  P.nconf = c->nconf; P.nbf = c->nbf; P.nelec = c->nelec; P.ksym = c->ksym;
  P.e1 = c->d_e1; P.e2 = c->d_e2; P.jsym = c->d_jsym; P.nopen = c->d_nopen;
  P.sefoff = c->d_sefoff; P.detoff = c->d_detoff;
  P.alpha = c->d_alpha; P.beta = c->d_beta; P.phase = c->d_phase; P.nalpha = c->d_nalpha;
  P.one = c->d_one; P.eri = c->d_eri;
  P.nbroff = c->dir_nbroff; P.nbr = c->dir_nbr;
  P.nseg = c->nseg; P.seg_cfg = c->dir_segcfg; P.seg_k0 = c->dir_segk0; P.seg_n = c->dir_segn;
  const int64_t N = c->nsef_total;
  PSOCI_CUDA(c, cudaMemset2DAsync(dY, sizeof(double) * ldy, 0, sizeof(double) * k, N, st));
  if (P.nseg == 0) return PSOCI_OK;
  // configurations of at most 32 determinants: the connectivity-marking kernel, evaluating
  // only the elements that can be non-zero; otherwise the generic one
  const bool fast = c->max_ndet <= FAST_MAXDET;
  const size_t smem = fast ? sizeof(FastSmem<W>) * WARPS_PER_CTA : sizeof(WarpSmem) * WARPS_PER_CTA;
  if (fast) {
    PSOCI_CUDA(c, cudaFuncSetAttribute(k_hbuild_fast<W, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    PSOCI_CUDA(c, cudaFuncSetAttribute(k_hbuild_fast<W, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  } else
    PSOCI_CUDA(c, cudaFuncSetAttribute(k_hbuild<W, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((P.nseg + WARPS_PER_CTA - 1) / WARPS_PER_CTA, 152 * 16));
  // MIXED (connectivity-marking kernel only): FP32 element x FP32 input products
  const bool mixed = fast && prec == PSOCI_PREC_MIXED && x32;
  for (int q0 = 0; q0 < k; q0 += 8) {
    P.dx = dX + q0; P.dy = dY + q0; P.ldx = ldx; P.ldy = ldy; P.kvec = std::min(8, k - q0);
    P.dx32 = nullptr;
    if (mixed) {
      psoci_note_launch();
      k_direct_x32<<<(unsigned)std::min<int64_t>((N + 255) / 256, 152 * 16), 256, 0, st>>>(N, P.kvec, P.dx, ldx, x32);
      P.dx32 = x32;
    }
    psoci_note_launch();
    if (fast && mixed)
      k_hbuild_fast<W, 2><<<blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
    else if (fast)
      k_hbuild_fast<W, 1><<<blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
    else
      k_hbuild<W, 2><<<blocks, WARPS_PER_CTA * 32, smem, st>>>(P);
    PSOCI_CUDA(c, cudaGetLastError());
  }
  return PSOCI_OK;
}

}  // namespace

psoci_status psoci_direct_sigma(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy, psoci_prec prec,
                                float *x32) {
  if (!c->direct) return psoci_fail(c, PSOCI_ERR_STATE, "direct sigma: no direct-mode build");
  return (c->words == 1) ? run_direct_sigma<1>(c, k, dX, ldx, dY, ldy, prec, x32)
                         : run_direct_sigma<2>(c, k, dX, ldx, dY, ldy, prec, x32);
}

void psoci_join_release(psoci_ctx *c) {
  psoci_free(c->d_jgid);
  psoci_free(c->d_jlid);
  psoci_free(c->d_jT);
  psoci_free(c->d_jlnoff);
  psoci_free(c->d_jln);
  psoci_free(c->d_jhdec);
  psoci_free(c->d_jlokey);
  c->join_ok = false;
}

// Tables of the lookup screen (see k_join).  The space qualifies when some split s <= 12
// leaves every configuration at most two electrons in the orbitals >= s, the
// configurations are numbered in ascending (hi pattern, lo pattern) order with lo patterns
// numbered by first appearance, and the tables stay small; otherwise the all-pairs screen
// is used.  Not qualifying is not an error.
namespace {
// the configuration of each (lo pattern, hi pattern) cell; the pairs are unique
__global__ void k_fill_T(int n, const int32_t *__restrict__ gid, const int32_t *__restrict__ lid, int64_t G,
                         int32_t *__restrict__ T) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    T[(int64_t)lid[i] * G + gid[i]] = i;
}
}  // namespace

psoci_status psoci_join_prepare(psoci_ctx *c) {
  psoci_join_release(c);
  const int n = c->nconf, nbf = c->nbf;
  const uint8_t *occ = c->h_occ.data();
  // split: orbitals >= s hold at most two electrons in every configuration
  // (the configuration loops run on the host's cores; only the numbering of lo patterns by
  // first appearance is sequential)
  std::vector<int> smax(std::max<unsigned>(1u, std::thread::hardware_concurrency()), 0);
  const int nthr = psoci_parallel_ranges(n, [&](int64_t lo, int64_t hi, int t) {
    int sm = 0;
    for (int64_t i = lo; i < hi; ++i) {
      const uint8_t *o = occ + (size_t)i * nbf;
      int e = 0, si = 0;
      for (int q = nbf - 1; q >= 0; --q) {
        e += o[q];
        if (e >= 3) { si = q + 1; break; }
      }
      sm = std::max(sm, si);
    }
    smax[t] = sm;
  });
  int s = 0;
  for (int t = 0; t < nthr; ++t) s = std::max(s, smax[t]);
  const int nh = nbf - s;
  if (s > 12 || nh < 1) return PSOCI_OK;
  const int64_t G = 1 + nh + (int64_t)nh * (nh + 1) / 2;
  std::vector<int32_t> gid(n), lid(n), keyid((size_t)1 << (2 * s), -1);
  std::vector<uint32_t> lokey, keys(n);
  psoci_parallel_ranges(n, [&](int64_t lo, int64_t hi, int) {
    for (int64_t i = lo; i < hi; ++i) {
      const uint8_t *o = occ + (size_t)i * nbf;
      uint32_t key = 0;
      for (int q = 0; q < s; ++q) {
        if (o[q] >= 1) key |= 1u << q;
        if (o[q] == 2) key |= 1u << (s + q);
      }
      int pa = -1, pb = -1, kind = 0;
      for (int q = s; q < nbf; ++q) {
        if (o[q] == 0) continue;
        if (o[q] == 2) { kind = 3; pa = q - s; }
        else if (pa < 0) { kind = 1; pa = q - s; }
        else { kind = 2; pb = q - s; }
      }
      gid[i] = (kind == 0) ? 0 : (kind == 1) ? 1 + pa
               : (int32_t)(1 + nh + (kind == 3 ? (int64_t)pa * (pa + 1) / 2 + pa : (int64_t)pb * (pb + 1) / 2 + pa));
      keys[i] = key;
    }
  });
  for (int i = 0; i < n; ++i) {
    const uint32_t key = keys[i];
    if (keyid[key] < 0) { keyid[key] = (int32_t)lokey.size(); lokey.push_back(key); }
    lid[i] = keyid[key];
    if (i > 0 && gid[i] < gid[i - 1]) return PSOCI_OK;  // hi patterns must ascend
  }
  const int64_t L = (int64_t)lokey.size();
  // Number the lo patterns so that they ascend inside every hi pattern: each group's order
  // is a chain of constraints; a topological order of all of them (ties broken by first
  // appearance) exists unless two groups order some patterns differently.
  {
    // constraint edges lid[i-1] -> lid[i] within a hi pattern, as a compressed adjacency
    std::vector<int32_t> indeg((size_t)L, 0), eoff((size_t)L + 1, 0), next;
    for (int i = 1; i < n; ++i)
      if (gid[i] == gid[i - 1]) {
        if (lid[i] == lid[i - 1]) return PSOCI_OK;  // repeated configuration
        ++eoff[lid[i - 1] + 1];
        ++indeg[lid[i]];
      }
    for (int64_t l = 0; l < L; ++l) eoff[l + 1] += eoff[l];
    next.resize((size_t)eoff[L]);
    {
      std::vector<int32_t> fill(eoff.begin(), eoff.end() - 1);
      for (int i = 1; i < n; ++i)
        if (gid[i] == gid[i - 1]) next[fill[lid[i - 1]]++] = lid[i];
    }
    std::vector<int32_t> order;
    order.reserve((size_t)L);
    std::priority_queue<int32_t, std::vector<int32_t>, std::greater<int32_t>> ready;
    for (int64_t l = 0; l < L; ++l)
      if (indeg[l] == 0) ready.push((int32_t)l);
    while (!ready.empty()) {
      const int32_t l = ready.top();
      ready.pop();
      order.push_back(l);
      for (int32_t e = eoff[l]; e < eoff[l + 1]; ++e)
        if (--indeg[next[e]] == 0) ready.push(next[e]);
    }
    if ((int64_t)order.size() != L) return PSOCI_OK;  // contradictory orders
    std::vector<int32_t> rank((size_t)L);
    std::vector<uint32_t> key2((size_t)L);
    for (int64_t r = 0; r < L; ++r) { rank[order[r]] = (int32_t)r; key2[r] = lokey[order[r]]; }
    for (int i = 0; i < n; ++i) lid[i] = rank[lid[i]];
    lokey.swap(key2);
    for (int i = 1; i < n; ++i)
      if (gid[i] == gid[i - 1] && lid[i] <= lid[i - 1]) return PSOCI_OK;
  }
  if (G * L > ((int64_t)1 << 26)) return PSOCI_OK;
  std::vector<int32_t> hdec((size_t)G);
  hdec[0] = 0;
  for (int a = 0; a < nh; ++a) hdec[1 + a] = 1 | (a << 8);
  for (int b = 0; b < nh; ++b)
    for (int a = 0; a <= b; ++a)
      hdec[1 + nh + (size_t)b * (b + 1) / 2 + a] = (a == b) ? (3 | (a << 8)) : (2 | (a << 8) | (b << 20));
  // lo patterns within tau = 1..4 of each lo pattern (itself included), ascending inside
  // each of five groups: the lo electron count minus l's, -2..2 (a hi pattern holds 0-2
  // electrons, so a partner lo pattern differs by at most 2; the others never make a
  // configuration and are left out).  Lists tau-major, then by pattern, then by group; one
  // distance per pair, counted then written in parallel.
  constexpr int NGRP = 5;
  std::vector<int32_t> lnoff(4 * (NGRP * L + 1)), ln, lcnt((size_t)4 * NGRP * L, 0);
  psoci_parallel_ranges(L, [&](int64_t lo, int64_t hi, int) {
    for (int64_t l = lo; l < hi; ++l) {
      const int nel = __builtin_popcount(lokey[l]);
      for (int64_t m = 0; m < L; ++m) {
        const int k = __builtin_popcount(lokey[m]) - nel + 2;
        if (k < 0 || k >= NGRP) continue;
        const int d = __builtin_popcount(lokey[l] ^ lokey[m]);
        for (int tau = std::max(d, 1); tau <= 4; ++tau) ++lcnt[((size_t)(tau - 1) * L + l) * NGRP + k];
      }
    }
  }, 64);
  {
    int64_t run = 0;
    for (int tau = 1; tau <= 4; ++tau) {
      for (int64_t g = 0; g < NGRP * L; ++g) {
        lnoff[(tau - 1) * (NGRP * L + 1) + g] = (int32_t)run;
        run += lcnt[(size_t)(tau - 1) * NGRP * L + g];
      }
      lnoff[(tau - 1) * (NGRP * L + 1) + NGRP * L] = (int32_t)run;
    }
    if (run > INT32_MAX) return PSOCI_OK;
    ln.resize((size_t)run);
  }
  psoci_parallel_ranges(L, [&](int64_t lo, int64_t hi, int) {
    for (int64_t l = lo; l < hi; ++l) {
      const int nel = __builtin_popcount(lokey[l]);
      int32_t pos[4][NGRP];
      for (int tau = 1; tau <= 4; ++tau)
        for (int k = 0; k < NGRP; ++k) pos[tau - 1][k] = lnoff[(tau - 1) * (NGRP * L + 1) + NGRP * l + k];
      for (int64_t m = 0; m < L; ++m) {
        const int k = __builtin_popcount(lokey[m]) - nel + 2;
        if (k < 0 || k >= NGRP) continue;
        const int d = __builtin_popcount(lokey[l] ^ lokey[m]);
        for (int tau = std::max(d, 1); tau <= 4; ++tau) ln[pos[tau - 1][k]++] = (int32_t)m;
      }
    }
  }, 64);
  psoci_status st;
  if ((st = psoci_alloc(c, &c->d_jgid, n)) || (st = psoci_alloc(c, &c->d_jlid, n)) ||
      (st = psoci_alloc(c, &c->d_jT, (size_t)(G * L))) || (st = psoci_alloc(c, &c->d_jlnoff, lnoff.size())) ||
      (st = psoci_alloc(c, &c->d_jln, ln.size())) || (st = psoci_alloc(c, &c->d_jhdec, hdec.size())) ||
      (st = psoci_alloc(c, &c->d_jlokey, lokey.size()))) {
    psoci_join_release(c);
    return st;
  }
  cudaStream_t q = c->stream;
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jgid, gid.data(), 4 * gid.size(), cudaMemcpyHostToDevice, q));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jlid, lid.data(), 4 * lid.size(), cudaMemcpyHostToDevice, q));
  // T[lo pattern][hi pattern] = configuration (or -1), filled on the device
  PSOCI_CUDA(c, cudaMemsetAsync(c->d_jT, 0xff, sizeof(int32_t) * (size_t)(G * L), q));
  psoci_note_launch();
  k_fill_T<<<(n + 255) / 256, 256, 0, q>>>(n, c->d_jgid, c->d_jlid, G, c->d_jT);
  PSOCI_CUDA(c, cudaGetLastError());
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jlnoff, lnoff.data(), 4 * lnoff.size(), cudaMemcpyHostToDevice, q));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jln, ln.data(), 4 * std::max<size_t>(ln.size(), 1), cudaMemcpyHostToDevice, q));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jhdec, hdec.data(), 4 * hdec.size(), cudaMemcpyHostToDevice, q));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_jlokey, lokey.data(), 4 * lokey.size(), cudaMemcpyHostToDevice, q));
  PSOCI_CUDA(c, cudaStreamSynchronize(q));
  c->join_s = s; c->join_nh = nh; c->join_G = (int)G; c->join_L = (int)L;
  c->join_ok = true;
  return PSOCI_OK;
}

void psoci_h_release(psoci_ctx *c) {
  psoci_grad_release(c);
  c->sigma_variant = PSOCI_SIGMA_DEFAULT;
  c->sigma_tuned = false;
  psoci_free(c->dir_nbroff);
  psoci_free(c->dir_nbr);
  psoci_free(c->dir_segcfg);
  psoci_free(c->dir_segk0);
  psoci_free(c->dir_segn);
  c->direct = false;
  psoci_free(c->d_rowptr);
  psoci_free(c->d_col);
  psoci_free(c->d_val);
  psoci_free(c->d_val32);
  psoci_free(c->d_diag);
  c->have_h = false;
  c->nnz = 0;
  c->binfo = psoci_build_info{};
}

psoci_status psoci_h_blocks(psoci_ctx *c, int npairs, const int32_t *A, const int32_t *B, double *out) {
  if (!c->have_ints) return psoci_fail(c, PSOCI_ERR_STATE, "blocks: no integrals set");
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "blocks: determinants not built");
  if (npairs < 0 || (npairs > 0 && (!A || !B || !out))) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "blocks: bad arguments");
  if (npairs == 0) return PSOCI_OK;
  return (c->words == 1) ? run_blocks<1>(c, npairs, A, B, out) : run_blocks<2>(c, npairs, A, B, out);
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
    fprintf(stderr, "psoci: H build N=%lld nnz=%lld candidates=%lld pairs=%lld segments=%lld %.3f s\n",
            (long long)c->nsef_total, (long long)c->nnz, (long long)c->ncand, (long long)c->npairs, (long long)c->nseg,
            c->build_seconds);
  return PSOCI_OK;
}

// ------------------------------------------------------------------------------------
// Energy gradient with respect to the integral tables: the adjoint of the element
// evaluation.  For a CI vector c, E = c^T H c and every element of H is a sum of entries of
// the packed tables with fixed coefficients (once the reference's zero-prefactor skips are
// left out), so dE / d table[t] is the transposed evaluation: every coupling of a
// determinant pair (x of I, y of J) adds its weight w_xy = cd_I[x] cd_J[y] (cd = the vector in
// the determinant basis, CDC^T's transpose) to the entries its element reads, with the
// element's sign and coefficient.  dE/d one[pq] is the spin-free 1-RDM (equal irreps) or the
// spin-orbit density (unequal irreps), dE/d eri[canon(pq,rs)] the 2-RDM in the reference's
// 8-fold packed layout (Hellmann-Feynman).
//
// Work: one warp per row configuration I over its lower neighbours J <= I (pairs J < I
// count twice, as H_JI = H_IJ^T), 32 pairs set up at a time (a lane each); lanes over the
// determinant pairs of one configuration pair classify each coupling (det_adj mirrors
// det_elem's branches) and add its weights to the pair's terms: v0, v1 (double, SO and
// single prefactors, or the diagonal's Kd[0]) in registers, the exchange terms X[t] /
// Kd[mm] in a per-warp shared array; the pair's terms are then scattered to the tables.
// ------------------------------------------------------------------------------------
namespace {

constexpr int ADJ_WARPS = 4;
constexpr int ADJ_MAXR = 8;                                        // roots per pass
constexpr int ADJ_NT = 2 + PSOCI_MAX_OPEN * (PSOCI_MAX_OPEN - 1) / 2;  // v0, v1, X[t] or Kd[mm]

enum { T_NONE = 0, T_V0, T_V1, T_V0MV1, T_SGL, T_X, T_DIAG, T_K, T_DIRECT };

template <int W>
struct AdjPair {
  int64_t detA, detB;
  int A, B, kind;
  int iex0, iex1, jex0, jex1;
  int jsA, jsB, nopenA, ndetA, ndetB;
  uint64_t SA[W];
  uint64_t bm[6][W];
};

// The structure of the pair (A, B) in the reference's roles, from the occupations and the
// symmetries alone: diagonal, same-symmetry single, spin-orbit single, double or none
// (more than two excitations).
template <int W>
__device__ void adj_pair_setup(const Params &P, int A, int B, AdjPair<W> &pi) {
  pi.A = A; pi.B = B;
  pi.detA = P.detoff[A]; pi.detB = P.detoff[B];
  pi.ndetA = (int)(P.detoff[A + 1] - P.detoff[A]);
  pi.ndetB = (int)(P.detoff[B + 1] - P.detoff[B]);
  pi.jsA = P.jsym[A]; pi.jsB = P.jsym[B];
  pi.nopenA = P.nopen[A];
  uint64_t e1A[W], e2A[W], e1B[W], e2B[W], im1[W], im2[W], jm1[W], jm2[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    e1A[w] = P.e1[(int64_t)A * W + w]; e2A[w] = P.e2[(int64_t)A * W + w];
    e1B[w] = P.e1[(int64_t)B * W + w]; e2B[w] = P.e2[(int64_t)B * W + w];
    im1[w] = e1A[w] & ~e1B[w]; im2[w] = e2A[w] & ~e2B[w];
    jm1[w] = e1B[w] & ~e1A[w]; jm2[w] = e2B[w] & ~e2A[w];
    pi.SA[w] = e1A[w] & ~e2A[w];
  }
  pi.iex0 = pi.iex1 = pi.jex0 = pi.jex1 = -1;
  const int ni = popc_w<W>(im1) + popc_w<W>(im2);
  const int nj = popc_w<W>(jm1) + popc_w<W>(jm2);
  if (A == B) { pi.kind = K_DIAG; return; }
  if (ni == 1 && nj == 1) {
    uint64_t im[W], jm[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { im[w] = im1[w] | im2[w]; jm[w] = jm1[w] | jm2[w]; }
    const int ie = lowest_bit<W>(im), je = lowest_bit<W>(jm);
    pi.iex0 = ie; pi.jex0 = je;
    between_mask<W>(ie, je, pi.bm[0]);
    range_mask<W>(0, ie - 1, pi.bm[1]);
    range_mask<W>(je + 1, 64 * W - 1, pi.bm[2]);
    range_mask<W>(0, je - 1, pi.bm[3]);
    range_mask<W>(ie + 1, 64 * W - 1, pi.bm[4]);
    pi.kind = (pi.jsA != pi.jsB) ? K_SO : K_SINGLE;
    return;
  }
  if (ni == 2 && nj == 2) {
    int ex0 = -1, ex1 = -1, jy0 = -1, jy1 = -1;
    two_positions<W>(im1, im2, ex0, ex1);
    two_positions<W>(jm1, jm2, jy0, jy1);
    pi.iex0 = ex0; pi.iex1 = ex1; pi.jex0 = jy0; pi.jex1 = jy1;
    between_mask<W>(ex0, jy0, pi.bm[0]);
    between_mask<W>(ex0, jy1, pi.bm[1]);
    between_mask<W>(ex1, jy0, pi.bm[2]);
    between_mask<W>(ex1, jy1, pi.bm[3]);
    between_mask<W>(ex0, ex1, pi.bm[4]);
    between_mask<W>(jy0, jy1, pi.bm[5]);
    pi.kind = K_DOUBLE;
    return;
  }
  pi.kind = K_NONE;
}

// rank of orbital p among the set bits of S (p must be set in S for a meaningful rank)
template <int W>
__device__ __forceinline__ int rank_in(const uint64_t (&S)[W], int p) {
  int r = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    if (64 * w + 63 < p) r += __popcll(S[w]);
    else if (64 * w <= p) r += __popcll(S[w] & ((1ull << (p & 63)) - 1ull));
  }
  return r;
}

// det_elem's branches, returning what the element is made of instead of its value:
// tag T_V0 / T_V1 / T_V0MV1 (+-v0, +-v1, +-(v0 - v1)); T_SGL: +-(v0 - sum of X[t] over the
// bits of mask); T_X: +-X[term]; T_DIAG: Kd[0] - sum of Kd[mm] over the bits mm of mask;
// T_K: +-Kd[term]; T_DIRECT: +-eri[direct]; T_NONE: zero.  sgn = +1 / -1.
template <int W>
__device__ __forceinline__ int det_adj(const AdjPair<W> &pi, const DetBits<W> &A, const DetBits<W> &B, int &sgn,
                                       uint64_t &mask, int &term, int64_t &direct) {
  const uint64_t(&aa)[W] = A.al;
  const uint64_t(&ba)[W] = A.be;
  const uint64_t(&ab)[W] = B.al;
  const uint64_t(&bb)[W] = B.be;
  const int pha = A.ph, phb = B.ph, naa = A.na, nab = B.na;
  uint64_t ua[W], ub[W];
#pragma unroll
  for (int w = 0; w < W; ++w) { ua[w] = ab[w] & ~aa[w]; ub[w] = bb[w] & ~ba[w]; }
  const int nmarka = popc_w<W>(ua);
  const int nmarkb = nmarka + popc_w<W>(ub);
  const int ie = pi.iex0, je = pi.jex0;
  sgn = 1;
  if (pi.kind == K_NONE) return T_NONE;
  if (pi.kind == K_SO) {
    if (nmarka > 1 || nmarkb > 1) return T_NONE;
    int ncount = pha + phb;
    if (naa < nab) {
      ncount += popc_and<W>(ba, pi.bm[1]) + popc_and<W>(ab, pi.bm[2]);
      if ((pi.jsA + pi.jsB) % 2 == 0) ++ncount;
      else if (pi.jsA % 2 == 1) ++ncount;
    } else if (naa > nab) {
      ncount += popc_and<W>(aa, pi.bm[4]) + popc_and<W>(bb, pi.bm[3]);
      if ((pi.jsA + pi.jsB) % 2 != 0 && (pi.jsA % 2) == 1) ++ncount;
    } else {
      if (nmarka == 0) ++ncount;
      if (pi.jsA % 2 == 1) ++ncount;
      uint64_t sp[W];
      sel_w<W>(sp, nmarka != 0, aa, ba);
      ncount += popc_and<W>(sp, pi.bm[0]);
    }
    sgn = (ncount & 1) ? -1 : 1;
    return T_V0;
  }
  if (naa != nab) return T_NONE;
  if (nmarka > 2 || nmarkb > 2) return T_NONE;
  if (nmarkb == 0) {
    if (pi.kind != K_DIAG) return T_NONE;
    // diag_det_elem: Kd[0] minus Kd[mm] for every pair of open shells with equal spins
    mask = 0ull;
    int mm = 0, io = 0;
#pragma unroll
    for (int wi = 0; wi < W; ++wi) {
      uint64_t si_bits = pi.SA[wi];
      while (si_bits) {
        const uint64_t lo_i = si_bits & (~si_bits + 1);
        si_bits ^= lo_i;
        const bool si = (aa[wi] & lo_i) != 0ull;
        int jo = 0;
#pragma unroll
        for (int wj = 0; wj < W; ++wj) {
          uint64_t sj = pi.SA[wj];
          while (sj && jo < io) {
            const uint64_t lo_j = sj & (~sj + 1);
            sj ^= lo_j;
            ++mm;
            if (si == ((aa[wj] & lo_j) != 0ull)) mask |= 1ull << (mm - 1);
            ++jo;
          }
        }
        ++io;
      }
    }
    return T_DIAG;
  }
  if (nmarkb == 1) {
    if (pi.kind != K_SINGLE) return T_NONE;
    uint64_t sp[W];
    sel_w<W>(sp, nmarka != 0, aa, ba);
    const int ncount = pha + phb + popc_and<W>(sp, pi.bm[0]);
    mask = 0ull;
    int t = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t m = sp[w] & ~(aa[w] & ba[w]);
      if ((ie >> 6) == w) m &= ~(1ull << (ie & 63));
      if ((je >> 6) == w) m &= ~(1ull << (je & 63));
      uint64_t sa = pi.SA[w];
      while (sa) {
        const uint64_t low = sa & (~sa + 1);
        if (m & low) mask |= 1ull << t;
        ++t;
        sa ^= low;
      }
    }
    sgn = (ncount & 1) ? -1 : 1;
    return T_SGL;
  }
  if (nmarka == 1) {
    uint64_t xa[W], xb[W];
#pragma unroll
    for (int w = 0; w < W; ++w) { xa[w] = aa[w] & ~ab[w]; xb[w] = ba[w] & ~bb[w]; }
    if (pi.kind == K_DOUBLE) {
      const int ia = bit_w<W>(xa, pi.iex0) ? 0 : 1, ja = bit_w<W>(ua, pi.jex0) ? 0 : 1;
      const int ncount = pha + phb + popc_and<W>(aa, pi.bm[2 * ia + ja]) + popc_and<W>(ba, pi.bm[3 - 2 * ia - ja]);
      sgn = (ncount & 1) ? -1 : 1;
      return (ia == ja) ? T_V0 : T_V1;
    }
    if (pi.kind != K_SINGLE && pi.kind != K_DIAG) return T_NONE;
    const int iex2 = lowest_bit<W>(ua), jex2 = lowest_bit<W>(ub);
    const int iex3 = lowest_bit<W>(xa), jex3 = lowest_bit<W>(xb);
    int ncount = pha + phb;
    if (abs(iex2 - iex3) > 1) ncount += popc_range<W>(aa, min(iex2, iex3) + 1, max(iex2, iex3) - 1);
    if (abs(jex2 - jex3) > 1) ncount += popc_range<W>(ba, min(jex2, jex3) + 1, max(jex2, jex3) - 1);
    sgn = (ncount & 1) ? -1 : 1;
    direct = canon4(jex2, jex3, iex2, iex3);
    if (pi.kind == K_SINGLE) {
      // alpha and beta moves through an open shell p of A: the integral is X[rank of p]
      const int p = (iex3 == ie || iex3 == je) ? iex2 : iex3;
      if (bit_w<W>(pi.SA, p) && canon4(ie, p, p, je) == direct) {
        term = rank_in<W>(pi.SA, p);
        return T_X;
      }
      return T_DIRECT;
    }
    // diagonal: a spin exchange between two open shells p and q, the integral Kd[mm(p, q)]
    const int p = iex3, q = iex2;
    if (bit_w<W>(pi.SA, p) && bit_w<W>(pi.SA, q) && canon4(p, q, q, p) == direct) {
      const int rp = rank_in<W>(pi.SA, p), rq = rank_in<W>(pi.SA, q);
      const int a = max(rp, rq), b = min(rp, rq);
      term = a * (a - 1) / 2 + b;  // Kd[1 + term] in diag_det_elem's order
      return T_K;
    }
    return T_DIRECT;
  }
  if (pi.kind != K_DOUBLE) return T_NONE;
  uint64_t spb[W], sa[W];
  sel_w<W>(spb, nmarka == 2, ab, bb);
  sel_w<W>(sa, nmarka != 0, aa, ba);
  const int ncount = pha + phb + popc_and<W>(spb, pi.bm[5]) + popc_and<W>(sa, pi.bm[4]);
  sgn = (ncount & 1) ? -1 : 1;
  return T_V0MV1;
}

// vectors (k per pass, root-major with stride ldv, FP64) in the determinant basis:
// CD[d * k + r], the transpose of ciout's transform (PsociHamiltonian.C:1457-1516)
template <typename CT>
__global__ void k_sef_to_det(int nconf, int nelec, int ksym, const int64_t *__restrict__ sefoff,
                             const int64_t *__restrict__ detoff, const int32_t *__restrict__ jsym,
                             const int32_t *__restrict__ nopen, const double *__restrict__ V, int64_t ldv, int k,
                             CT *__restrict__ CD) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t >> 5), lane = threadIdx.x & 31;
  if (i >= nconf) return;
  const int64_t s0 = sefoff[i], d0 = detoff[i];
  const int nsef = (int)(sefoff[i + 1] - s0);
  const bool odd = nelec & 1;
  const bool open = !odd && nopen[i] != 0;
  const double m = (jsym[i] % 2 != ksym % 2) ? -1.0 : 1.0;
  const double r = sqrt(0.5);
  for (int e = lane; e < nsef * k; e += 32) {
    const int a = e / k, q = e - a * k;
    const double c = V[(int64_t)q * ldv + s0 + a];
    if (open) {
      CD[(d0 + 2 * a) * k + q] = (CT)(r * c);
      CD[(d0 + 2 * a + 1) * k + q] = (CT)((m * r) * c);
    } else {
      CD[(d0 + a) * k + q] = (CT)c;
    }
  }
}

template <int W>
struct AdjSmem {
  AdjPair<W> pi[32];
  double acc[ADJ_NT][ADJ_MAXR];
};

// scatter of one pair's terms into the gradient tables G1 [k][n1], G2 [k][n2] (FP64 atomics);
// f = 2 for J < I, 1 on the diagonal.  Lanes split the roots and entries.
template <int W>
__device__ void adj_scatter(const Params &P, const AdjPair<W> &pi, const double (&acc)[ADJ_NT][ADJ_MAXR], int k,
                            double f, double *G1, int64_t n1, double *G2, int64_t n2, int lane) {
  const int A = pi.A;
  if (pi.kind == K_DOUBLE) {
    if (lane < k) {
      atomicAdd(G2 + lane * n2 + canon4(pi.iex0, pi.jex0, pi.iex1, pi.jex1), f * acc[0][lane]);
      atomicAdd(G2 + lane * n2 + canon4(pi.iex0, pi.jex1, pi.iex1, pi.jex0), f * acc[1][lane]);
    }
    return;
  }
  if (pi.kind == K_SO) {
    // v = +-SO(ie, je) / 2, negated when je > ie (processSingleExcitation, PsociHamiltonian.C:223-237)
    if (lane < k) atomicAdd(G1 + lane * n1 + tri64(pi.iex0, pi.jex0), f * (pi.jex0 > pi.iex0 ? -0.5 : 0.5) * acc[0][lane]);
    return;
  }
  uint64_t e1A[W], e2A[W], e2B[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    e1A[w] = P.e1[(int64_t)A * W + w]; e2A[w] = P.e2[(int64_t)A * W + w];
    e2B[w] = P.e2[(int64_t)pi.B * W + w];
  }
  if (pi.kind == K_SINGLE) {
    const int ie = pi.iex0, je = pi.jex0;
    // lanes over (root, entry): entry 0 one[ie, je], 1 (ie je|ie ie), 2.. the occupied p,
    // then the X[t] terms
    for (int r = 0; r < k; ++r) {
      const double a0 = f * acc[0][r];
      if (lane == 0) {
        atomicAdd(G1 + r * n1 + tri64(ie, je), a0);
        atomicAdd(G2 + r * n2 + canon4(ie, je, ie, ie), -a0);
      }
      // sum over the occupied orbitals p of A: (ie je|p p) x occ_A(p), and -(ie p|p je) where
      // p is doubly occupied in both
      int pidx = 0;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        uint64_t o = e1A[w];
        while (o) {
          const int p = 64 * w + __ffsll((long long)o) - 1;
          o &= o - 1;
          if ((pidx & 31) == lane) {
            const bool dA = bit_w<W>(e2A, p);
            atomicAdd(G2 + r * n2 + canon4(ie, je, p, p), dA ? 2.0 * a0 : a0);
            if (dA && bit_w<W>(e2B, p)) atomicAdd(G2 + r * n2 + canon4(ie, p, p, je), -a0);
          }
          ++pidx;
        }
      }
      int t = 0;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        uint64_t sa = pi.SA[w];
        while (sa) {
          const int p = 64 * w + __ffsll((long long)sa) - 1;
          sa &= sa - 1;
          if ((t & 31) == lane && acc[2 + t][r] != 0.0) atomicAdd(G2 + r * n2 + canon4(ie, p, p, je), f * acc[2 + t][r]);
          ++t;
        }
      }
    }
    return;
  }
  if (pi.kind == K_DIAG) {
    // Kd[0] = sum over occupied ib of occ h_ii (+ (ii|ii) if doubly) and over pairs jb < ib of
    // Coulomb and exchange terms (processDiagExcitation, PsociHamiltonian.C:306-388); lanes
    // over ib
    for (int r = 0; r < k; ++r) {
      const double a0 = f * acc[0][r];
      int iidx = 0;
#pragma unroll
      for (int wi = 0; wi < W; ++wi) {
        uint64_t oi = e1A[wi];
        while (oi) {
          const int ib = 64 * wi + __ffsll((long long)oi) - 1;
          oi &= oi - 1;
          if ((iidx & 31) == lane) {
            const int occi = 1 + (int)bit_w<W>(e2A, ib);
            if (occi == 1) atomicAdd(G1 + r * n1 + tri64(ib, ib), a0);
            else {
              atomicAdd(G1 + r * n1 + tri64(ib, ib), 2.0 * a0);
              atomicAdd(G2 + r * n2 + canon4(ib, ib, ib, ib), a0);
            }
#pragma unroll
            for (int wj = 0; wj < W; ++wj) {
              uint64_t oj = e1A[wj];
              while (oj) {
                const int jb = 64 * wj + __ffsll((long long)oj) - 1;
                oj &= oj - 1;
                if (jb >= ib) break;
                const int ninj = occi * (1 + (int)bit_w<W>(e2A, jb));
                if (ninj == 1) atomicAdd(G2 + r * n2 + canon4(ib, ib, jb, jb), a0);
                else {
                  const double m = (ninj == 2) ? 1.0 : 2.0;
                  atomicAdd(G2 + r * n2 + canon4(ib, ib, jb, jb), 2.0 * m * a0);
                  atomicAdd(G2 + r * n2 + canon4(ib, jb, ib, jb), -m * a0);
                }
              }
            }
          }
          ++iidx;
        }
      }
      // Kd[mm] = (s_a s_b|s_b s_a) over the open shells a > b, in that order
      int sing[PSOCI_MAX_OPEN], ns = 0;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        uint64_t sb = pi.SA[w];
        while (sb && ns < PSOCI_MAX_OPEN) { sing[ns++] = 64 * w + __ffsll((long long)sb) - 1; sb &= sb - 1; }
      }
      int mm = 0;
      for (int a = 1; a < ns; ++a)
        for (int b = 0; b < a; ++b, ++mm)
          if ((mm & 31) == lane && acc[2 + mm][r] != 0.0)
            atomicAdd(G2 + r * n2 + canon4(sing[a], sing[b], sing[b], sing[a]), f * acc[2 + mm][r]);
    }
  }
}

// Whether determinants A and B of the pair can couple (det_adj's early exits): a cheap
// first pass, so that the classification runs on the coupled pairs only.
template <int W>
__device__ __forceinline__ bool det_coupled(const AdjPair<W> &pi, const DetBits<W> &A, const DetBits<W> &B) {
  int na = 0, nb = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) { na += __popcll(B.al[w] & ~A.al[w]); nb += __popcll(B.be[w] & ~A.be[w]); }
  if (pi.kind == K_SO) return na <= 1 && na + nb <= 1;
  if (A.na != B.na || na + nb > 2) return false;
  if (na + nb == 0) return pi.kind == K_DIAG;
  if (na + nb == 1) return pi.kind == K_SINGLE;
  if (na == 1) return pi.kind != K_NONE;
  return pi.kind == K_DOUBLE;
}

constexpr int ADJ_RT = 15;    // exchange terms held in registers (Kd[mm] of <= 6 open shells)
constexpr int ADJ_CONN = 128; // coupled determinant pairs collected per round

// A coupled determinant pair of the pair being processed, classified: its determinants
// (x << 16 | y), the det_adj tag, sign and term, and the exchange-term mask.
struct AdjRec {
  uint64_t mask;
  uint32_t xy;
  int32_t info;  // tag | (sgn < 0) << 4 | term << 8
};

// One warp per row configuration I (grid-stride); its lower neighbours J <= I in chunks of
// 32 set up by the lanes.  Per pair: (1) lanes over the determinant pairs (x, y) test them for
// coupling and classify the coupled ones (det_adj), collecting the records in shared memory;
// (2) lanes = (slot, root) take the records, slots over the records and roots over the lanes
// of a slot, and add s * cd_I[x] * cd_J[y] to register accumulators of the pair's terms (v0,
// v1, and the exchange terms X[t] / Kd[mm]; terms beyond ADJ_RT, only on diagonals of 7+ open
// shells, go to shared-memory atomics); (3) the slots' sums are reduced by shuffles and the
// root lanes scatter the pair's terms to the tables.  CT/ACC: the type of the determinant-
// basis vectors and of the sums within a pair (FP64, or FP32 for the FP32-bulk variant).
template <int W, typename CT, typename ACC>
__global__ void __launch_bounds__(ADJ_WARPS * 32) k_energy_grad(Params P, const int64_t *__restrict__ nbroff,
                                                                const int32_t *__restrict__ nbr,
                                                                const CT *__restrict__ CD, int k, double *G1,
                                                                int64_t n1, double *G2, int64_t n2) {
  __shared__ AdjSmem<W> sm[ADJ_WARPS];
  __shared__ AdjRec recs[ADJ_WARPS][ADJ_CONN];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  AdjSmem<W> &S = sm[wib];
  AdjRec *rec = recs[wib];
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // lanes of one slot hold consecutive roots: kp (a power of two >= k) roots per slot
  const int kp = (k <= 1) ? 1 : (k <= 2) ? 2 : (k <= 4) ? 4 : 8;
  const int nslot = 32 / kp, slot = lane / kp, r = lane % kp;
  const bool rok = r < k;
  for (int e = lane; e < ADJ_NT * ADJ_MAXR; e += 32) (&S.acc[0][0])[e] = 0.0;
  __syncwarp();
  for (int64_t I = warp; I < P.nconf; I += nwarps) {
    const int64_t b0 = nbroff[I], b1 = nbroff[I + 1];
    for (int64_t c0 = b0; c0 < b1; c0 += 32) {
      const int64_t q = c0 + lane;
      const int J = (q < b1) ? nbr[q] : INT_MAX;
      const bool lower = J <= (int)I;
      if (lower) adj_pair_setup<W>(P, (int)I, J, S.pi[lane]);
      const unsigned lm = __ballot_sync(0xffffffffu, lower);
      __syncwarp();
      const int np = __popc(lm);  // lower pairs come first within the chunk
      for (int u = 0; u < np; ++u) {
        const AdjPair<W> &pi = S.pi[u];
        if (pi.kind == K_NONE) continue;
        const double fpair = (pi.A == pi.B) ? 1.0 : 2.0;
        const int nterm = (pi.kind == K_SINGLE) ? pi.nopenA
                          : (pi.kind == K_DIAG) ? min(ADJ_RT, pi.nopenA * (pi.nopenA - 1) / 2) : 0;
        ACC a0 = 0, a1 = 0, aT[ADJ_RT];
#pragma unroll
        for (int t = 0; t < ADJ_RT; ++t) aT[t] = 0;
        const int nd = pi.ndetA * pi.ndetB;
        for (int e0 = 0; e0 < nd;) {
          // (1) classify the determinant pairs, one a lane; keep the coupled ones
          int nc = 0;
          while (e0 < nd && nc + 32 <= ADJ_CONN) {
            const int e = e0 + lane;
            int tag = T_NONE, sgn = 1, term = 0, x = 0, y = 0;
            uint64_t mask = 0ull;
            if (e < nd) {
              x = e / pi.ndetB;
              y = e - x * pi.ndetB;
              DetBits<W> Ad, Bd;
              load_det<W>(Ad, P.alpha, P.beta, P.phase, P.nalpha, pi.detA + x);
              load_det<W>(Bd, P.alpha, P.beta, P.phase, P.nalpha, pi.detB + y);
              if (det_coupled<W>(pi, Ad, Bd)) {
                int64_t direct = 0;
                tag = det_adj<W>(pi, Ad, Bd, sgn, mask, term, direct);
                if (tag == T_DIRECT) {
                  // an integral outside the pair's terms (not met in practice): added here
                  for (int rr = 0; rr < k; ++rr)
                    atomicAdd(G2 + (int64_t)rr * n2 + direct,
                              fpair * sgn * (double)CD[(pi.detA + x) * k + rr] * (double)CD[(pi.detB + y) * k + rr]);
                  tag = T_NONE;
                }
              }
            }
            const bool keep = tag != T_NONE;
            const unsigned cb = __ballot_sync(0xffffffffu, keep);
            if (keep) {
              AdjRec &R = rec[nc + __popc(cb & ((1u << lane) - 1u))];
              R.mask = mask;
              R.xy = ((uint32_t)x << 16) | (uint32_t)y;
              R.info = tag | ((sgn < 0) ? 16 : 0) | (term << 8);
            }
            nc += __popc(cb);
            e0 += 32;
          }
          __syncwarp();
          // (2) accumulate, slots over the records, roots over the lanes of a slot
          if (rok) {
            for (int cq = slot; cq < nc; cq += nslot) {
              const AdjRec R = rec[cq];
              const int x = (int)(R.xy >> 16), y = (int)(R.xy & 0xffffu);
              const int tag = R.info & 15, term = R.info >> 8;
              ACC w = (ACC)__ldg(CD + (pi.detA + x) * k + r) * (ACC)__ldg(CD + (pi.detB + y) * k + r);
              if (R.info & 16) w = -w;
              if (tag == T_V0) a0 += w;
              else if (tag == T_V1) a1 += w;
              else if (tag == T_V0MV1) { a0 += w; a1 -= w; }
              else if (tag == T_SGL || tag == T_DIAG) {
                a0 += w;
#pragma unroll
                for (int t = 0; t < ADJ_RT; ++t) {
                  if (t >= nterm) break;  // uniform over the warp
                  if ((R.mask >> t) & 1ull) aT[t] -= w;
                }
                uint64_t m = R.mask >> ADJ_RT;
                while (m) {
                  const int t = ADJ_RT + __ffsll((long long)m) - 1;
                  m &= m - 1;
                  atomicAdd(&S.acc[2 + t][r], -(double)w);
                }
              } else {  // T_X, T_K
                if (term < ADJ_RT) {
#pragma unroll
                  for (int t = 0; t < ADJ_RT; ++t) {
                    if (t >= nterm) break;
                    if (t == term) aT[t] += w;
                  }
                } else {
                  atomicAdd(&S.acc[2 + term][r], (double)w);
                }
              }
            }
          }
          __syncwarp();
        }
        // (3) sums over the slots (lanes r, r + kp, r + 2kp, ...): lanes of slot 0 hold them
        double s0 = (double)a0, s1 = (double)a1, sT[ADJ_RT];
#pragma unroll
        for (int t = 0; t < ADJ_RT; ++t) sT[t] = (double)aT[t];
        for (int o = kp; o < 32; o <<= 1) {
          s0 += __shfl_xor_sync(0xffffffffu, s0, o);
          s1 += __shfl_xor_sync(0xffffffffu, s1, o);
#pragma unroll
          for (int t = 0; t < ADJ_RT; ++t)
            if (t < nterm) sT[t] += __shfl_xor_sync(0xffffffffu, sT[t], o);
        }
        __syncwarp();  // the shared-memory terms (spilled atomics) are complete
        if (lane < k) {
          S.acc[0][lane] = s0;
          S.acc[1][lane] = s1;
#pragma unroll
          for (int t = 0; t < ADJ_RT; ++t)
            if (t < nterm) S.acc[2 + t][lane] = sT[t];
        }
        __syncwarp();
        adj_scatter<W>(P, pi, S.acc, k, fpair, G1, n1, G2, n2, lane);
        __syncwarp();
        const int used = 2 + ((pi.kind == K_DIAG) ? pi.nopenA * (pi.nopenA - 1) / 2 : pi.nopenA);
        for (int e = lane; e < used * ADJ_MAXR; e += 32) (&S.acc[0][0])[e] = 0.0;
        __syncwarp();
      }
      __syncwarp();
      if (np < 32) break;  // past the diagonal
    }
  }
}

__global__ void k_fill(double *p, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_nonzero(const double *__restrict__ src, double *__restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (src[i] != 0.0) ? 1.0 : 0.0;
}
// entries of zero integrals reported as zero (mode: derivatives of the non-zero integrals)
__global__ void k_mask_zero(const double *__restrict__ tab, int64_t n, int k, double *G) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (tab[i] == 0.0)
      for (int r = 0; r < k; ++r) G[(int64_t)r * n + i] = 0.0;
}

template <int W>
psoci_status run_energy_grad(psoci_ctx *c, int k, const double *dV, int64_t ldv, int mode, psoci_prec prec,
                             double *dG1, double *dG2) {
  cudaStream_t st = c->stream;
  const int n = c->nconf;
  Params P = {};
  P.nconf = n; P.nbf = c->nbf; P.nelec = c->nelec; P.ksym = c->ksym;
  P.e1 = c->d_e1; P.e2 = c->d_e2; P.jsym = c->d_jsym; P.nopen = c->d_nopen;
  P.sefoff = c->d_sefoff; P.detoff = c->d_detoff;
  P.alpha = c->d_alpha; P.beta = c->d_beta; P.phase = c->d_phase; P.nalpha = c->d_nalpha;
  P.one = c->d_one; P.eri = c->d_eri;
  psoci_status s;
  const int64_t n1 = c->n1, n2 = c->n2;
  // neighbour lists: every pair within two excitations (mode 0), or those whose integral
  // prefactors are not all zero (mode 1); kept in the context for later calls
  if (!c->grad_nbroff || c->grad_mode != mode) {
    psoci_free(c->grad_nbroff);
    psoci_free(c->grad_nbr);
    double *t1 = nullptr, *t2 = nullptr;
    if ((s = psoci_alloc(c, &t1, n1)) || (s = psoci_alloc(c, &t2, n2))) {
      psoci_free(t1);
      psoci_free(t2);
      return s;
    }
    psoci_note_launch();
    if (mode == 0) k_fill<<<152 * 4, 256, 0, st>>>(t1, n1, 1.0);
    else k_nonzero<<<152 * 4, 256, 0, st>>>(c->d_one, t1, n1);
    psoci_note_launch();
    if (mode == 0) k_fill<<<152 * 8, 256, 0, st>>>(t2, n2, 1.0);
    else k_nonzero<<<152 * 8, 256, 0, st>>>(c->d_eri, t2, n2);
    int64_t ncand = 0, npairs = 0;
    int nsplit = 0;
    s = screen_pairs<W>(c, P, t1, t2, c->grad_nbroff, c->grad_nbr, ncand, npairs, nsplit);
    cudaStreamSynchronize(st);
    psoci_free(t1);
    psoci_free(t2);
    if (s) return s;
    c->grad_mode = mode;
    c->grad_npairs = npairs;
  }
  double *CD = nullptr;  // determinant-basis vectors (FP64, or FP32 for the FP32-bulk variant)
  if ((s = psoci_alloc(c, &CD, (size_t)c->ndet_total * std::min(k, ADJ_MAXR)))) return s;
  float *CD32 = reinterpret_cast<float *>(CD);
  PSOCI_CUDA(c, cudaMemsetAsync(dG1, 0, sizeof(double) * n1 * k, st));
  PSOCI_CUDA(c, cudaMemsetAsync(dG2, 0, sizeof(double) * n2 * k, st));
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)n + ADJ_WARPS - 1) / ADJ_WARPS, 152 * 16));
  for (int r0 = 0; r0 < k; r0 += ADJ_MAXR) {
    const int kk = std::min(ADJ_MAXR, k - r0);
    const unsigned sb = (unsigned)(((int64_t)n * 32 + 255) / 256);
    psoci_note_launch();
    if (prec == PSOCI_PREC_MIXED)
      k_sef_to_det<float><<<sb, 256, 0, st>>>(n, c->nelec, c->ksym, c->d_sefoff, c->d_detoff, c->d_jsym, c->d_nopen,
                                              dV + (int64_t)r0 * ldv, ldv, kk, CD32);
    else
      k_sef_to_det<double><<<sb, 256, 0, st>>>(n, c->nelec, c->ksym, c->d_sefoff, c->d_detoff, c->d_jsym, c->d_nopen,
                                               dV + (int64_t)r0 * ldv, ldv, kk, CD);
    psoci_note_launch();
    if (prec == PSOCI_PREC_MIXED)
      k_energy_grad<W, float, float><<<blocks, ADJ_WARPS * 32, 0, st>>>(P, c->grad_nbroff, c->grad_nbr, CD32, kk,
                                                                        dG1 + r0 * n1, n1, dG2 + r0 * n2, n2);
    else
      k_energy_grad<W, double, double><<<blocks, ADJ_WARPS * 32, 0, st>>>(P, c->grad_nbroff, c->grad_nbr, CD, kk,
                                                                          dG1 + r0 * n1, n1, dG2 + r0 * n2, n2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      psoci_free(CD);
      return psoci_cuda_fail(c, e, "energy_gradient");
    }
  }
  if (mode == 1) {
    psoci_note_launch();
    k_mask_zero<<<152 * 4, 256, 0, st>>>(c->d_one, n1, k, dG1);
    psoci_note_launch();
    k_mask_zero<<<152 * 8, 256, 0, st>>>(c->d_eri, n2, k, dG2);
  }
  cudaError_t e = cudaStreamSynchronize(st);
  psoci_free(CD);
  if (e != cudaSuccess) return psoci_cuda_fail(c, e, "energy_gradient");
  return PSOCI_OK;
}

}  // namespace

void psoci_grad_release(psoci_ctx *c) {
  psoci_free(c->grad_nbroff);
  psoci_free(c->grad_nbr);
  c->grad_mode = -1;
  c->grad_npairs = 0;
}

psoci_status psoci_energy_grad_run(psoci_ctx *c, int k, const double *dV, int64_t ldv, int mode, psoci_prec prec,
                                   double *dG1, double *dG2) {
  if (!c->have_ints) return psoci_fail(c, PSOCI_ERR_STATE, "energy_gradient: no integrals set");
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "energy_gradient: determinants not built");
  if (k < 1 || ldv < c->nsef_total || !dV || !dG1 || !dG2)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "energy_gradient: bad arguments");
  if (mode != 0 && mode != 1) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "energy_gradient: mode must be 0 or 1");
  if (prec != PSOCI_PREC_FP64 && prec != PSOCI_PREC_MIXED)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "energy_gradient: precision must be FP64 or MIXED");
  return (c->words == 1) ? run_energy_grad<1>(c, k, dV, ldv, mode, prec, dG1, dG2)
                         : run_energy_grad<2>(c, k, dV, ldv, mode, prec, dG1, dG2);
}
