// Davidson eigensolver on the device.
//
// Reference flow (psociRestart-Cori/): driver.PSOCI.splittest.C:1186-1311 with
//   PsociGAsubspace::generateIncrementalSubspace (PsociGAsubspace.C:273-366)  S, G columns
//   PsociGAsubspace::diagSubspaceGOP (:1088-1171) -> dsygv                     Rayleigh-Ritz
//   PsociGAsubspace::computeRnormSingle (:874-1000)                            residual
//   PsociGAbasis::precondition (PsociGAbasis.C:1860-1919)   t_i = r_i/(D_i-l) if |D_i-l| > 1e-3
//   PsociGAbasis::orthonormalizeAppendedVectors (:1371-1474)                   Gram-Schmidt
//   PsociGAbasis::expandAndReplaceVectorsNew (:483-583)   collapse V and HV, no recompute
//
// The reference adds one vector per iteration, for the first unconverged root.  Here the
// default is block Davidson: every unconverged root contributes a preconditioned residual
// each iteration, so one pass over H serves the whole block (block = 0 keeps the
// reference's one-vector step).  The basis is kept orthonormal (CGS2 against V, then
// Cholesky-QR twice inside the new block), so S = I and the generalised problem of the
// reference reduces to a symmetric one, solved on the host each iteration
// (psoci_subspace_eigen, symeig.cpp), as the reference's dsygv is.
//
// Initial guess: the lowest eigenvectors of H on the 3072 lowest diagonal elements, found
// by this same solver run on that dense block (a one-CTA Jacobi for blocks of at most 96).
//
// Vectors are N x ld row-major: the k entries of one SEF row are contiguous, which is
// what the sigma kernel gathers.  All subspace arithmetic is FP64 or float-float.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <type_traits>
#include <vector>

#include "ffmath.cuh"
#include "psoci_internal.cuh"

namespace {

constexpr int TS_THREADS = 256;   // k_tn block size
constexpr int TN_MAXK = 16;       // k_tn: B columns (two groups of 8 outputs per i)
constexpr int TN_TILE = 256;      // k_tn: rows of B staged per tile
constexpr int NN_THREADS = 128;   // k_nn block size
constexpr int NN_MAXK = 32;       // k_nn: Y columns (four groups of 8 outputs per row)
constexpr int MAX_SUB = 96;       // subspace limit; the guess Jacobi keeps two m x m FP64 matrices in shared memory

// The tall-skinny products below run in float-float arithmetic on the FP32 pipe (see
// ffmath.cuh): on GB300 the FP64 pipe issues ~2 FMA/clk/SM against 128 FP32 lanes, and
// these products are FP64-bound.  Block partials are combined in FP64.
//
// LOWP (the FP32-element phase of a mixed solve, whose sigma is good to ~1e-7 anyway):
// elements truncated to FP32 (the high word of the float-float split: integer operations
// only), products summed in FP32 over a tile, tile sums added in float-float.
//
// Register tiling: a thread owns 8 outputs and, per row, reads one element of the tall
// operand straight from global memory (coalesced across the warp, several rows in flight)
// and 8 broadcast elements of the other operand from shared memory, so the inner loop
// issues 8 float-float FMAs per load of its own.
template <bool LOWP>
using ts_elt = typename std::conditional<LOWP, float, float2>::type;

template <bool LOWP>
__device__ __forceinline__ ts_elt<LOWP> ts_load(double x) {
  if constexpr (LOWP) return split_f64(x).x;
  else return split_f64(x);
}

// 8 consecutive elements from 16-byte aligned shared memory
template <bool LOWP>
__device__ __forceinline__ void ts_load8(const ts_elt<LOWP> *p, ts_elt<LOWP> (&v)[8]) {
  const float4 *q = reinterpret_cast<const float4 *>(p);
  if constexpr (LOWP) {
    const float4 u = q[0], w = q[1];
    v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
    v[4] = w.x; v[5] = w.y; v[6] = w.z; v[7] = w.w;
  } else {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const float4 u = q[t];
      v[2 * t] = make_float2(u.x, u.y);
      v[2 * t + 1] = make_float2(u.z, u.w);
    }
  }
}

// acc[j] += a * b[j] for the 8 outputs of a thread (float-float, or FP32 when LOWP)
template <bool LOWP>
__device__ __forceinline__ void ts_fma8(float (&h)[8], float (&l)[8], ts_elt<LOWP> a, const ts_elt<LOWP> (&b)[8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if constexpr (LOWP) h[j] = __fmaf_rn(a, b[j], h[j]);
    else ff_fma(h[j], l[j], a, b[j]);
  }
}

// partial[blk][i*k + j] = sum over the block's rows r of A[r, a0+i] * B[r, b0+j]
// (m <= MAX_SUB, k <= TN_MAXK).  Thread: output group g = (i, jb), the 8 outputs
// j in [8jb, 8jb+8) of row i of C, over the rows sub, sub+S, ... of each tile; B's tile is
// split into shared memory once, A is read from global memory (lanes of a warp take
// consecutive i of one row).  The S shares of a group are added in FP64 at the end, in a
// fixed order.
template <bool LOWP>
__global__ void __launch_bounds__(TS_THREADS) k_tn(int64_t n, const double *__restrict__ A, int lda, int a0, int m,
                                                   const double *__restrict__ B, int ldb, int b0, int k,
                                                   double *__restrict__ partial, int64_t rows_per_blk) {
  using E = ts_elt<LOWP>;
  extern __shared__ double sm[];
  const int kp = (k + 7) & ~7;                 // B rows padded with zeros to whole groups (8 or 16)
  const int ksh = (kp == 8) ? 3 : 4;
  E *Bs = reinterpret_cast<E *>(sm);           // [TN_TILE][kp]
  const int tid = threadIdx.x;
  const int G = m * (kp >> 3);
  const int S = max(1, TS_THREADS / G);
  const int g = tid % G, sub = tid / G;
  const int i = g % m, jb = g / m;
  const bool act = sub < S;
  float h[8], l[8], t[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) { h[j] = 0.f; l[j] = 0.f; }
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_blk;
  const int64_t r1 = min(n, r0 + rows_per_blk);
  const double *ai = A + a0 + i;
  for (int64_t rt = r0; rt < r1; rt += TN_TILE) {
    const int rows = (int)min((int64_t)TN_TILE, r1 - rt);
#pragma unroll 4
    for (int e = tid; e < (TN_TILE << ksh); e += TS_THREADS) {
      const int rr = e >> ksh, j = e & (kp - 1);
      Bs[e] = (rr < rows && j < k) ? ts_load<LOWP>(B[(rt + rr) * ldb + b0 + j]) : E{};
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int j = 0; j < 8; ++j) t[j] = 0.f;
      const double *ar = ai + rt * lda;
      int rr = sub;
      for (; rr + 3 * S < rows; rr += 4 * S) {  // four rows in flight
        double av[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) av[u] = __ldg(ar + (int64_t)(rr + u * S) * lda);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          E b[8];
          ts_load8<LOWP>(Bs + ((rr + u * S) << ksh) + 8 * jb, b);
          if constexpr (LOWP) ts_fma8<true>(t, l, ts_load<true>(av[u]), b);
          else ts_fma8<false>(h, l, ts_load<false>(av[u]), b);
        }
      }
      for (; rr < rows; rr += S) {
        E b[8];
        ts_load8<LOWP>(Bs + (rr << ksh) + 8 * jb, b);
        if constexpr (LOWP) ts_fma8<true>(t, l, ts_load<true>(__ldg(ar + (int64_t)rr * lda)), b);
        else ts_fma8<false>(h, l, ts_load<false>(__ldg(ar + (int64_t)rr * lda)), b);
      }
      if constexpr (LOWP)
#pragma unroll
        for (int j = 0; j < 8; ++j) ff_fma(h[j], l[j], make_float2(t[j], 0.f), make_float2(1.f, 0.f));
#pragma unroll
      for (int j = 0; j < 8; ++j) ff_renorm(h[j], l[j]);
    }
    __syncthreads();
  }
  // combine the S shares of each output in FP64 (the tile is no longer needed)
  double *red = sm;  // [S][G][8]
  if (act)
#pragma unroll
    for (int j = 0; j < 8; ++j) red[(sub * G + g) * 8 + j] = (double)h[j] + (double)l[j];
  __syncthreads();
  const int nout = m * k;
  for (int o = tid; o < G * 8; o += TS_THREADS) {
    const int g2 = o >> 3, jj = (g2 / m) * 8 + (o & 7);
    if (jj >= k) continue;
    double s = 0.0;
    for (int q = 0; q < S; ++q) s += red[(q * G + g2) * 8 + (o & 7)];
    partial[(int64_t)blockIdx.x * nout + (g2 % m) * k + jj] = s;
  }
}

// C[i*ldc + c0 + j] = sum_b partial[b][i*k + j]   (fixed order: deterministic).  One block
// per group of 32 outputs; its warps sum interleaved slices of the partials (coalesced along
// the outputs) and one warp adds the slices in warp order.
__global__ void k_reduce_partials(const double *__restrict__ partial, int nblk, int m, int k, double *C, int ldc,
                                  int c0) {
  __shared__ double red[8][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;  // blockDim.x == 256
  const int nout = m * k;
  const int idx = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (idx < nout)
    for (int b = wid; b < nblk; b += 8) s += partial[(int64_t)b * nout + idx];
  red[wid][lane] = s;
  __syncthreads();
  if (wid == 0 && idx < nout) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w][lane];
    const int i = idx / k, j = idx - i * k;
    C[i * ldc + c0 + j] = t;
  }
}

// Out[r, o0+j] = beta*Out[r, o0+j] + alpha * sum_i A[r, a0+i] * Y[i*ldy + y0 + j]
// (m <= MAX_SUB, k <= NN_MAXK; float-float sums, or FP32 sums when LOWP; alpha, beta and
// the update of Out in FP64).  Thread: one row and the 8 outputs of group jb; a block takes
// NN_THREADS/jbp rows (jbp = groups rounded up to a power of two).  Y is split into shared
// memory once per block; the thread reads its row of A from global memory, two elements
// per load where the rows are 16-byte aligned, several loads in flight.  No barrier after
// the staging of Y.
template <bool LOWP>
__global__ void __launch_bounds__(NN_THREADS) k_nn(int64_t n, const double *__restrict__ A, int lda, int a0, int m,
                                                   const double *__restrict__ Y, int ldy, int y0, int k, double alpha,
                                                   double beta, double *Out, int ldo, int o0, int jbp) {
  using E = ts_elt<LOWP>;
  extern __shared__ double sm[];
  const int kp = (k + 7) & ~7;
  E *Ys = reinterpret_cast<E *>(sm);  // [m][kp], 16-byte aligned rows
  const int tid = threadIdx.x;
  for (int e = tid; e < m * kp; e += NN_THREADS) {
    const int i = e / kp, j = e - i * kp;
    Ys[e] = (j < k) ? ts_load<LOWP>(Y[i * ldy + y0 + j]) : E{};
  }
  __syncthreads();
  const int TR = NN_THREADS / jbp;
  const int rr = tid % TR, jb = tid / TR;
  const int64_t r = (int64_t)blockIdx.x * TR + rr;
  if (8 * jb >= k || r >= n) return;
  const double *ar = A + r * lda + a0;
  const E *yj = Ys + 8 * jb;
  float h[8], l[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) { h[j] = 0.f; l[j] = 0.f; }
  int i = 0;
  if (((lda | a0) & 1) == 0) {
#pragma unroll 4
    for (; i + 1 < m; i += 2) {
      const double2 v = __ldg(reinterpret_cast<const double2 *>(ar + i));
      E y[8];
      ts_load8<LOWP>(yj + i * kp, y);
      ts_fma8<LOWP>(h, l, ts_load<LOWP>(v.x), y);
      ts_load8<LOWP>(yj + (i + 1) * kp, y);
      ts_fma8<LOWP>(h, l, ts_load<LOWP>(v.y), y);
    }
  }
#pragma unroll 4
  for (; i < m; ++i) {
    E y[8];
    ts_load8<LOWP>(yj + i * kp, y);
    ts_fma8<LOWP>(h, l, ts_load<LOWP>(__ldg(ar + i)), y);
  }
  double *o = Out + r * ldo + o0 + 8 * jb;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if (8 * jb + j >= k) break;
    const double s = LOWP ? (double)h[j] : (double)h[j] + (double)l[j];
    o[j] = (beta == 0.0) ? alpha * s : fma(beta, o[j], alpha * s);
  }
}

// R[r, j] = HX[r, j] - theta[j] * X[r, j]; partial squared norms per block.  A thread takes
// whole rows (the nr values of a row are contiguous), so each row is read once.
__global__ void k_residual(int64_t n, int nr, const double *__restrict__ X, const double *__restrict__ HX,
                           const double *__restrict__ theta, double *__restrict__ R, double *__restrict__ partial) {
  __shared__ double red[16][8];  // [root][warp], blockDim.x == 256
  double th[16], s[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    th[j] = (j < nr) ? theta[j] : 0.0;
    s[j] = 0.0;
  }
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (j >= nr) break;
      const double v = HX[r * nr + j] - th[j] * X[r * nr + j];
      R[r * nr + j] = v;
      s[j] = fma(v, v, s[j]);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if (j >= nr) break;
    double v = s[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[j][wid] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < nr) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[threadIdx.x][w];
    partial[(int64_t)blockIdx.x * nr + threadIdx.x] = t;
  }
}

__global__ void k_sum_cols(const double *partial, int nblk, int nr, double *out) {
  int j = threadIdx.x;
  if (j >= nr) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += partial[(int64_t)b * nr + j];
  out[j] = s;
}

// T[r, c] = R[r, sel[c]] / (D[r] - theta[sel[c]]) where |D - theta| > dmin, else R.
// The correction is a search direction (the basis is orthonormalised right after), so the
// quotient is formed on the FP32 pipe: D - theta exactly enough in float-float (the
// guard decision sees ~2^-48 relative error), then an FP32 quotient (~2^-23 relative) —
// a slightly perturbed diagonal preconditioner.  FP64 division on GB300 is a sequence of
// FP64-pipe instructions and bounded the kernel.  Consecutive threads take consecutive
// elements of T (coalesced stores); U: 32-bit index arithmetic where n * nsel fits.
__device__ __forceinline__ double f32_to_f64_bits(float f) {
  // exact widening by bit manipulation (normal numbers and zero; others -> NaN or 0)
  const unsigned u = (unsigned)__float_as_int(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned e = (u >> 23) & 0xff;
  if (e == 0) return __longlong_as_double((long long)sign);
  if (e == 0xff) return __longlong_as_double((long long)(sign | 0x7ff8000000000000ull));
  const unsigned long long bits = sign | ((unsigned long long)(e + 1023 - 127) << 52) |
                                  ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

template <typename U>
__global__ void k_precond(int64_t n, int nr, const double *__restrict__ R, const double *__restrict__ D,
                          const double *__restrict__ theta, const int *__restrict__ sel, int nsel, double dmin,
                          double *__restrict__ T, int ldt) {
  __shared__ float2 th[16];
  __shared__ int js[16];
  if ((int)threadIdx.x < nsel) {
    js[threadIdx.x] = sel[threadIdx.x];
    th[threadIdx.x] = split_f64(theta[sel[threadIdx.x]]);
  }
  __syncthreads();
  const float dminf = (float)dmin;
  const U total = (U)n * (U)nsel;
  for (U e = (U)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (U)gridDim.x * blockDim.x) {
    const U r = e / (U)nsel, c = e - r * (U)nsel;
    const double v = R[(size_t)r * nr + js[c]];
    const float2 dd = split_f64(D[r]);
    const float dh = __fsub_rn(dd.x, th[c].x);                // exact when D and theta are close
    const float d = __fadd_rn(dh, __fsub_rn(dd.y, th[c].y));
    double t = v;
    if (fabsf(d) > dminf) t = f32_to_f64_bits(__fdiv_rn(split_f64(v).x, d));
    T[(size_t)r * ldt + c] = t;
  }
}

// Gram matrix S (b x b) -> upper-triangular inverse factor F (b x b'), columns of kept
// vectors compacted, so that T * F has orthonormal columns.  Drops a column whose
// Cholesky pivot falls below drop_tol^2 of its original norm (linear dependence).
__global__ void k_cholqr_factor(const double *S, int b, const double *ref, int ldref, double drop_tol, double *F,
                                int *nkept) {
  __shared__ double Finv[16 * 16];
  __shared__ int keep[16];
  if (threadIdx.x != 0) return;
  // Cholesky S = R^T R with R upper; dropped columns get zero rows
  double Rm[16][16];
  for (int i = 0; i < b; ++i)
    for (int j = 0; j < b; ++j) Rm[i][j] = 0.0;
  int nk = 0;
  for (int j = 0; j < b; ++j) {
    double s = S[j * b + j];
    double orig = ref ? ref[j * ldref + j] : s;
    for (int i = 0; i < j; ++i) s -= Rm[i][j] * Rm[i][j];
    if (!(orig > 0.0) || s <= drop_tol * drop_tol * orig || !(s > 0.0)) {
      keep[j] = 0;
      continue;
    }
    keep[j] = 1;
    ++nk;
    double rjj = sqrt(s);
    Rm[j][j] = rjj;
    for (int c = j + 1; c < b; ++c) {
      double t = S[j * b + c];
      for (int i = 0; i < j; ++i) t -= Rm[i][j] * Rm[i][c];
      Rm[j][c] = t / rjj;
    }
  }
  // invert the kept upper-triangular part: F = R^{-1} restricted to kept rows/cols
  for (int i = 0; i < b * b; ++i) Finv[i] = 0.0;
  for (int j = 0; j < b; ++j) {
    if (!keep[j]) continue;
    Finv[j * b + j] = 1.0 / Rm[j][j];
    for (int i = j - 1; i >= 0; --i) {
      if (!keep[i]) continue;
      double t = 0.0;
      for (int q = i + 1; q <= j; ++q)
        if (keep[q]) t += Rm[i][q] * Finv[q * b + j];
      Finv[i * b + j] = -t / Rm[i][i];
    }
  }
  // compact kept columns
  int c = 0;
  for (int j = 0; j < b; ++j) {
    if (!keep[j]) continue;
    for (int i = 0; i < b; ++i) F[i * b + c] = Finv[i * b + j];
    ++c;
  }
  for (; c < b; ++c)
    for (int i = 0; i < b; ++i) F[i * b + c] = 0.0;
  *nkept = nk;
}

// G (ld x ld): mirror new columns [m0, m1) into rows and symmetrise the new diagonal block
__global__ void k_symmetrize(double *G, int ld, int m0, int m1) {
  for (int e = threadIdx.x; e < m1 * (m1 - m0); e += blockDim.x) {
    int i = e / (m1 - m0), j = m0 + e % (m1 - m0);
    if (i < m0) G[j * ld + i] = G[i * ld + j];
    else if (i < j) {
      double a = 0.5 * (G[i * ld + j] + G[j * ld + i]);
      G[i * ld + j] = a;
      G[j * ld + i] = a;
    }
  }
}

// One-CTA cyclic Jacobi (round-robin parallel ordering) for a symmetric m x m matrix: the
// initial guess's block of H.  Out: theta ascending, Y (ld x ld, column c = eigenvector c).
// status: sweeps used, or -1 if the off-diagonal norm did not fall below tolerance in
// max_sweeps.  Rotations whose off-diagonal element is below 1e-13 |A|_F / m are skipped
// (threshold Jacobi): when all are, the off-diagonal norm already passes the convergence
// test (1e-13 |A|_F).
__global__ void k_jacobi(const double *G, int ld, int m, double *theta, double *Y, int max_sweeps, int *status) {
  extern __shared__ double sm[];
  double *A = sm;                 // m x m
  double *V = sm + m * m;         // m x m
  __shared__ double cs[MAX_SUB / 2 + 1][2];
  __shared__ int pq[MAX_SUB / 2 + 1][2];
  __shared__ double red[512];
  __shared__ int order[MAX_SUB];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < m * m; e += nt) {
    int i = e / m, j = e % m;
    A[e] = G[i * ld + j];
    V[e] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  const int np = (m + 1) & ~1;  // even player count (a dummy when m is odd)
  int sweeps = 0;
  bool converged = (m <= 1);
  for (int sw = 0; sw < max_sweeps && !converged; ++sw) {
    // off-diagonal and total Frobenius norms
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < m * m; e += nt) {
      double a = A[e];
      tot += a * a;
      if (e / m != e % m) off += a * a;
    }
    red[tid] = off;
    __syncthreads();
    for (int o = nt / 2; o > 0; o >>= 1) { if (tid < o) red[tid] += red[tid + o]; __syncthreads(); }
    off = red[0];
    __syncthreads();
    red[tid] = tot;
    __syncthreads();
    for (int o = nt / 2; o > 0; o >>= 1) { if (tid < o) red[tid] += red[tid + o]; __syncthreads(); }
    tot = red[0];
    __syncthreads();
    if (off <= 1e-26 * tot || off == 0.0) { converged = true; break; }
    ++sweeps;
    const double rot_min = 1e-13 * sqrt(tot) / m;
    for (int rnd = 0; rnd < np - 1; ++rnd) {
      // pairs of this round
      for (int kq = tid; kq < np / 2; kq += nt) {
        int a = (kq == 0) ? 0 : 1 + ((kq - 1 + rnd) % (np - 1));
        int bidx = np - 1 - kq;
        int b = 1 + ((bidx - 1 + rnd) % (np - 1));
        int p = min(a, b), q = max(a, b);
        double c = 1.0, s = 0.0;
        if (q < m) {
          double apq = A[p * m + q];
          if (fabs(apq) > rot_min) {
            double tau = (A[q * m + q] - A[p * m + p]) / (2.0 * apq);
            double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        cs[kq][0] = c; cs[kq][1] = s;
        pq[kq][0] = p; pq[kq][1] = q;
      }
      __syncthreads();
      // A <- A J (columns), V <- V J
      for (int e = tid; e < (np / 2) * m; e += nt) {
        int kq = e / m, i = e % m;
        int p = pq[kq][0], q = pq[kq][1];
        double c = cs[kq][0], s = cs[kq][1];
        if (q >= m || s == 0.0) continue;
        double aip = A[i * m + p], aiq = A[i * m + q];
        A[i * m + p] = c * aip - s * aiq;
        A[i * m + q] = s * aip + c * aiq;
        double vip = V[i * m + p], viq = V[i * m + q];
        V[i * m + p] = c * vip - s * viq;
        V[i * m + q] = s * vip + c * viq;
      }
      __syncthreads();
      // A <- J^T A (rows)
      for (int e = tid; e < (np / 2) * m; e += nt) {
        int kq = e / m, j = e % m;
        int p = pq[kq][0], q = pq[kq][1];
        double c = cs[kq][0], s = cs[kq][1];
        if (q >= m || s == 0.0) continue;
        double apj = A[p * m + j], aqj = A[q * m + j];
        A[p * m + j] = c * apj - s * aqj;
        A[q * m + j] = s * apj + c * aqj;
      }
      __syncthreads();
    }
  }
  // sort eigenvalues ascending (rank sort; ties broken by index)
  for (int i = tid; i < m; i += nt) {
    double di = A[i * m + i];
    int rank = 0;
    for (int j = 0; j < m; ++j) {
      double dj = A[j * m + j];
      if (dj < di || (dj == di && j < i)) ++rank;
    }
    order[rank] = i;
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    int i = e / m, c = e % m;
    Y[i * ld + c] = V[i * m + order[c]];
  }
  for (int c = tid; c < m; c += nt) theta[c] = A[order[c] * m + order[c]];
  if (tid == 0) *status = converged ? sweeps : -1;
}

// initial guess from the lowest diagonal block: map[row] = position of the row in idx
__global__ void k_map_set(const int64_t *idx, int M, int32_t *map) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) map[idx[i]] = i;
}

// Hs[i*M + j] = H[idx[i], idx[j]] from the stored rows (one warp per row)
__global__ void k_extract_block(const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                                const double *__restrict__ val, const int64_t *__restrict__ idx, int M,
                                const int32_t *__restrict__ map, double *Hs) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= M) return;
  const int64_t row = idx[i];
  for (int64_t t = rowptr[row] + lane; t < rowptr[row + 1]; t += 32) {
    const int j = map[col[t]];
    if (j >= 0) Hs[(int64_t)i * M + j] = val[t];
  }
}

// V[idx[i], j] = Y[i, j]: the block's lowest eigenvectors as the first basis vectors
__global__ void k_scatter_guess(const double *Y, int ldy, const int64_t *idx, int M, int nr, double *V, int ld) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < M * nr; e += gridDim.x * blockDim.x) {
    const int i = e / nr, j = e - i * nr;
    V[idx[i] * ld + j] = Y[(int64_t)i * ldy + j];
  }
}

__global__ void k_set_unit(double *V, int ld, int c0, const int64_t *idx, int nr) {
  int j = threadIdx.x;
  if (j < nr) V[idx[j] * ld + c0 + j] = 1.0;
}

// dst[r, d0+j] = src[r, s0+j], j < k; consecutive threads take consecutive elements
// (coalesced); U: 32-bit index arithmetic where n * k fits
template <typename U>
__global__ void k_copy_cols(int64_t n, const double *__restrict__ src, int lds, int s0, double *__restrict__ dst,
                            int ldd, int d0, int k) {
  const U total = (U)n * (U)k;
  for (U e = (U)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (U)gridDim.x * blockDim.x) {
    const U r = e / (U)k, j = e - r * (U)k;
    dst[(size_t)r * ldd + d0 + j] = src[(size_t)r * lds + s0 + j];
  }
}

// Y[i, j] = sum_l A[i*n + l] X[l*ldx + j], j < k (k <= 16): the dense guess block applied in
// FP64.  One warp per row (lanes stride the row, coalesced), k sums reduced across lanes.
__global__ void k_dense_mv(int n, const double *__restrict__ A, const double *__restrict__ X, int ldx,
                           double *__restrict__ Y, int ldy, int k) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= n) return;
  double acc[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j] = 0.0;
  const double *a = A + (int64_t)i * n;
  for (int l = lane; l < n; l += 32) {
    const double h = a[l];
    const double *x = X + (int64_t)l * ldx;
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if (j < k) acc[j] = fma(h, x[j], acc[j]);
  }
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    if (j >= k) break;
    double v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) Y[(int64_t)i * ldy + j] = v;
  }
}

struct Work {
  psoci_ctx *c = nullptr;
  int64_t N = 0;
  int ld = 0, nr = 0;
  double *V = nullptr, *HV = nullptr, *G = nullptr, *Y = nullptr, *theta = nullptr;
  double *X = nullptr, *HX = nullptr, *R = nullptr, *T = nullptr, *tmp = nullptr;
  double *partial = nullptr, *small = nullptr, *F = nullptr, *norms = nullptr;
  float *x32 = nullptr;
  int *sel = nullptr, *ibuf = nullptr;
  int64_t *idx = nullptr;
  // the operator: the context's Hamiltonian, or (dense != nullptr) a dense N x N FP64 block
  // of it, the initial guess's subproblem
  const double *dense = nullptr;
  int nblk = 0;
  int64_t rows_per_blk = 0;
  // FP32 subspace products allowed (the FP32-element phase of a mixed solve): used for the
  // orthonormalisation and the new columns of G, whose errors (~1e-7) stay below what that
  // phase resolves; Ritz vectors, their images and collapses keep float-float sums, since
  // the residuals are formed from them
  bool lowp = false;
  std::vector<cudaEvent_t> ev;
  ~Work() {
    psoci_free(V); psoci_free(HV); psoci_free(G); psoci_free(Y); psoci_free(theta); psoci_free(X); psoci_free(HX);
    psoci_free(R); psoci_free(T); psoci_free(tmp); psoci_free(partial); psoci_free(small); psoci_free(F);
    psoci_free(norms); psoci_free(x32); psoci_free(sel); psoci_free(ibuf); psoci_free(idx);
    for (auto e : ev) cudaEventDestroy(e);
  }
};

// C (ldc, column offset c0) = A[:, a0:a0+m]^T B[:, b0:b0+k]
psoci_status tn(Work &w, const double *A, int lda, int a0, int m, const double *B, int ldb, int b0, int k, double *C,
                int ldc, int c0, bool lowp_ok = false) {
  const bool lowp = w.lowp && lowp_ok;
  psoci_ctx *c = w.c;
  if (m < 1 || k < 1 || m > MAX_SUB || k > TN_MAXK) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "tn: block too large");
  // B's tile, and at least the 16 KB of the FP64 combination of the shares
  const int kp = (k + 7) & ~7;
  const size_t smem = std::max<size_t>((size_t)TN_TILE * kp * (lowp ? sizeof(float) : sizeof(float2)),
                                       sizeof(double) * TS_THREADS * 8);
  psoci_note_launch();
  if (lowp)
    k_tn<true><<<w.nblk, TS_THREADS, smem, c->stream>>>(w.N, A, lda, a0, m, B, ldb, b0, k, w.partial, w.rows_per_blk);
  else
    k_tn<false><<<w.nblk, TS_THREADS, smem, c->stream>>>(w.N, A, lda, a0, m, B, ldb, b0, k, w.partial, w.rows_per_blk);
  psoci_note_launch();
  k_reduce_partials<<<(m * k + 31) / 32, 256, 0, c->stream>>>(w.partial, w.nblk, m, k, C, ldc, c0);
  PSOCI_CUDA(c, cudaGetLastError());
  return PSOCI_OK;
}

psoci_status nn(Work &w, const double *A, int lda, int a0, int m, const double *Y, int ldy, int y0, int k, double alpha,
                double beta, double *Out, int ldo, int o0, bool lowp_ok = false) {
  const bool lowp = w.lowp && lowp_ok;
  psoci_ctx *c = w.c;
  if (m < 1 || k < 1 || m > MAX_SUB || k > NN_MAXK) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "nn: block too large");
  const int groups = (k + 7) / 8;
  const int jbp = groups == 1 ? 1 : groups == 2 ? 2 : 4;  // groups rounded up to a power of two
  const int tr = NN_THREADS / jbp;                         // rows per block
  const size_t smem = (lowp ? sizeof(float) : sizeof(float2)) * (size_t)m * 8 * groups;
  const int64_t blocks = (w.N + tr - 1) / tr;
  psoci_note_launch();
  if (lowp)
    k_nn<true><<<(unsigned)blocks, NN_THREADS, smem, c->stream>>>(w.N, A, lda, a0, m, Y, ldy, y0, k, alpha, beta, Out,
                                                                  ldo, o0, jbp);
  else
    k_nn<false><<<(unsigned)blocks, NN_THREADS, smem, c->stream>>>(w.N, A, lda, a0, m, Y, ldy, y0, k, alpha, beta, Out,
                                                                   ldo, o0, jbp);
  PSOCI_CUDA(c, cudaGetLastError());
  return PSOCI_OK;
}

void copy_cols(Work &w, const double *src, int lds, double *dst, int ldd, int k) {
  psoci_note_launch();
  if (w.N * 32 < (int64_t)UINT32_MAX)
    k_copy_cols<uint32_t><<<152 * 8, 256, 0, w.c->stream>>>(w.N, src, lds, 0, dst, ldd, 0, k);
  else
    k_copy_cols<uint64_t><<<152 * 8, 256, 0, w.c->stream>>>(w.N, src, lds, 0, dst, ldd, 0, k);
}

psoci_status sigma_block(Work &w, const double *X, int ldx, double *Y, int ldy, int k, psoci_prec prec) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  w.ev.push_back(e0);
  w.ev.push_back(e1);
  cudaEventRecord(e0, w.c->stream);
  psoci_status s = PSOCI_OK;
  if (w.dense) {
    psoci_note_launch();
    k_dense_mv<<<(unsigned)((w.N + 7) / 8), 256, 0, w.c->stream>>>((int)w.N, w.dense, X, ldx, Y, ldy, k);
    if (cudaGetLastError() != cudaSuccess) s = psoci_fail(w.c, PSOCI_ERR_CUDA, "davidson: guess block product");
  } else {
    s = psoci_sigma_launch(w.c, k, X, ldx, Y, ldy, prec, w.x32);
  }
  cudaEventRecord(e1, w.c->stream);
  return s;
}

// orthonormalise T[:, 0:b] against V[:, 0:m] and within itself; kept columns land in
// V[:, m:m+b'].  Returns b' through *bk.
psoci_status orthonormalize(Work &w, int m, int b, int *bk) {
  psoci_ctx *c = w.c;
  psoci_status s;
  const int ld = w.ld, tld = w.nr;
  // squared norms before the projection: a column that loses all but 1e-10 of its norm
  // against V (or the block's earlier columns) carries no new direction and is dropped
  double *ref = w.small + (size_t)ld * ld / 2;
  if ((s = tn(w, w.T, tld, 0, b, w.T, tld, 0, b, ref, b, 0, true))) return s;
  for (int pass = 0; pass < 2 && m > 0; ++pass) {
    // C = V^T T (m x b) into w.small (ld = b), T -= V C
    if ((s = tn(w, w.V, ld, 0, m, w.T, tld, 0, b, w.small, b, 0, true))) return s;
    if ((s = nn(w, w.V, ld, 0, m, w.small, b, 0, b, -1.0, 1.0, w.T, tld, 0, true))) return s;
  }
  // Cholesky-QR twice: first into tmp, then into V[:, m:]
  int nk = b;
  for (int pass = 0; pass < 2; ++pass) {
    const double *src = (pass == 0) ? w.T : w.tmp;
    int srcld = (pass == 0) ? tld : w.nr;
    if ((s = tn(w, src, srcld, 0, nk, src, srcld, 0, nk, w.small, nk, 0, true))) return s;
    psoci_note_launch();
    k_cholqr_factor<<<1, 32, 0, c->stream>>>(w.small, nk, pass == 0 ? ref : nullptr, b, 1e-10, w.F, w.ibuf);
    PSOCI_CUDA(c, cudaGetLastError());
    int nk2 = 0;
    PSOCI_CUDA(c, cudaMemcpyAsync(&nk2, w.ibuf, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
    if (nk2 == 0) { *bk = 0; return PSOCI_OK; }
    if (pass == 0) {
      if ((s = nn(w, w.T, tld, 0, nk, w.F, nk, 0, nk2, 1.0, 0.0, w.tmp, w.nr, 0, true))) return s;
    } else {
      if ((s = nn(w, w.tmp, w.nr, 0, nk, w.F, nk, 0, nk2, 1.0, 0.0, w.V, ld, m, true))) return s;
    }
    nk = nk2;
  }
  *bk = nk;
  return PSOCI_OK;
}

}  // namespace

namespace {

// Radix select of the M lowest diagonal elements on the device: doubles as order-preserving
// 64-bit keys, eight 8-bit digit passes (256-bin histograms of the elements whose higher
// digits match the prefix found so far) fix the M-th smallest key; the indices of the elements
// at or below it (M plus ties) are collected and ordered on the host by (value, index).
__device__ __forceinline__ uint64_t order_key(double v) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_radix_hist(int64_t n, const double *__restrict__ d, uint64_t prefix, uint64_t pmask, int shift,
                             unsigned *__restrict__ hist) {
  __shared__ unsigned h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = order_key(d[i]);
    if ((k & pmask) == prefix) atomicAdd(&h[(k >> shift) & 255u], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

__global__ void k_select_le(int64_t n, const double *__restrict__ d, uint64_t kth, int64_t *__restrict__ out,
                            unsigned long long *cnt, int64_t cap) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (order_key(d[i]) <= kth) {
      const unsigned long long p = atomicAdd(cnt, 1ull);
      if ((int64_t)p < cap) out[p] = i;
    }
}

__global__ void k_gather_vals(int64_t m, const int64_t *__restrict__ idx, const double *__restrict__ d,
                              double *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = d[idx[i]];
}

// the M lowest elements of the device array d[N], ordered by (value, index)
psoci_status lowest_elements(psoci_ctx *c, const double *d, int64_t N, int M, std::vector<int64_t> &low) {
  cudaStream_t st = c->stream;
  low.clear();
  auto host_path = [&]() -> psoci_status {
    std::vector<double> h(N);
    PSOCI_CUDA(c, cudaMemcpyAsync(h.data(), d, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    PSOCI_CUDA(c, cudaStreamSynchronize(st));
    std::vector<int64_t> order(N);
    std::iota(order.begin(), order.end(), 0);
    std::partial_sort(order.begin(), order.begin() + M, order.end(),
                      [&](int64_t a, int64_t b) { return h[a] < h[b] || (h[a] == h[b] && a < b); });
    low.assign(order.begin(), order.begin() + M);
    return PSOCI_OK;
  };
  if (N <= 65536 || M < 1) return host_path();
  const int64_t cap = 4 * (int64_t)M + 1024;
  unsigned *hist = nullptr;
  int64_t *idx = nullptr;
  double *vals = nullptr;
  unsigned long long *cnt = nullptr;
  psoci_status s;
  auto done = [&](psoci_status r) {
    psoci_free(hist); psoci_free(idx); psoci_free(vals); psoci_free(cnt);
    return r;
  };
  if ((s = psoci_alloc(c, &hist, 256)) || (s = psoci_alloc(c, &idx, cap)) || (s = psoci_alloc(c, &vals, cap)) ||
      (s = psoci_alloc(c, &cnt, 1)))
    return done(s);
  const int blocks = (int)std::min<int64_t>((N + 255) / 256, 152 * 8);
  uint64_t prefix = 0, pmask = 0;
  int64_t rem = M;  // rank of the wanted key among the elements matching the prefix
  unsigned h[256];
  for (int shift = 56; shift >= 0; shift -= 8) {
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(unsigned) * 256, st);
    if (e == cudaSuccess) {
      psoci_note_launch();
      k_radix_hist<<<blocks, 256, 0, st>>>(N, d, prefix, pmask, shift, hist);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, hist, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "davidson: guess selection"));
    int64_t cum = 0;
    int dig = 255;
    for (int b = 0; b < 256; ++b) {
      if (cum + (int64_t)h[b] >= rem) { dig = b; break; }
      cum += h[b];
    }
    rem -= cum;
    prefix |= (uint64_t)dig << shift;
    pmask |= (uint64_t)255 << shift;
  }
  unsigned long long found = 0;
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    psoci_note_launch();
    k_select_le<<<blocks, 256, 0, st>>>(N, d, prefix, idx, cnt, cap);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&found, cnt, sizeof(found), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "davidson: guess selection"));
  if ((int64_t)found > cap || (int64_t)found < M) {  // many ties: the host orders them all
    done(PSOCI_OK);
    return host_path();
  }
  std::vector<int64_t> cand(found);
  std::vector<double> hv(found);
  psoci_note_launch();
  k_gather_vals<<<(unsigned)((found + 255) / 256), 256, 0, st>>>((int64_t)found, idx, d, vals);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(cand.data(), idx, sizeof(int64_t) * found, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hv.data(), vals, sizeof(double) * found, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return done(psoci_cuda_fail(c, e, "davidson: guess selection"));
  done(PSOCI_OK);
  std::vector<size_t> ord(found);
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(),
            [&](size_t a, size_t b) { return hv[a] < hv[b] || (hv[a] == hv[b] && cand[a] < cand[b]); });
  low.resize(M);
  for (int q = 0; q < M; ++q) low[q] = cand[ord[q]];
  return PSOCI_OK;
}

constexpr int GUESS_M = 3072;  // order of the initial guess's block of H (lowest diagonal elements)

// The solver over an operator of order N with diagonal diag (device): the context's
// Hamiltonian (dense == nullptr), or a dense block of it for the initial guess (inner: unit
// vectors as its own guess, no error text on non-convergence).  dX_out (device, N x nroots
// row-major) receives the last Ritz vectors, converged or not.
psoci_status davidson_run(psoci_ctx *c, int64_t N, const double *diag, const double *dense, const psoci_dav_opts *o,
                          bool inner, double *evals, double *evecs, double *rnorms, psoci_dav_stats *stats,
                          double *dX_out) {
  const int nr = o->nroots;
  if (nr < 1 || nr > 16 || nr > N) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "davidson: nroots must be 1..16 and <= N");
  // default basis: 8 vectors per root (capped at MAX_SUB).  Every iteration adds up to nr
  // vectors, so the reference's 4 nr collapses every two or three iterations; for 12 roots
  // of a 3.6M-SEF block 4 nr took 40 iterations and 96 took 26.
  int maxsub = o->max_subspace > 0 ? o->max_subspace : std::min(MAX_SUB, 8 * nr);
  maxsub = std::max(maxsub, 3 * nr);
  maxsub = std::min<int64_t>(maxsub, std::min<int64_t>(MAX_SUB, N));
  if (maxsub < 2 * nr && N >= 2 * nr) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "davidson: subspace too small");
  if (o->prec != PSOCI_PREC_FP64 && o->prec != PSOCI_PREC_MIXED && o->prec != PSOCI_PREC_FF)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "davidson: unknown precision");
  if (o->prec == PSOCI_PREC_MIXED && !dense && !c->d_val32 && !c->direct)
    return psoci_fail(c, PSOCI_ERR_STATE, "davidson: MIXED needs PSOCI_HMODE_CSR_BOTH");
  const double rtol = o->rtol > 0 ? o->rtol : 1e-6;
  const double dmin = o->precond_min > 0 ? o->precond_min : 1e-3;
  const int max_iter = o->max_iter > 0 ? o->max_iter : 1000;
  auto t_start = std::chrono::steady_clock::now();

  Work w;
  w.c = c;
  w.N = N;
  w.dense = dense;
  w.nr = nr;
  w.ld = (maxsub + 1) & ~1;
  const int ld = w.ld;
  w.nblk = (int)std::min<int64_t>(std::max<int64_t>(1, (N + 255) / 256), 152 * 4);
  w.rows_per_blk = (N + w.nblk - 1) / w.nblk;
  psoci_status s;
  if ((s = psoci_alloc(c, &w.V, (size_t)N * ld)) || (s = psoci_alloc(c, &w.HV, (size_t)N * ld)) ||
      (s = psoci_alloc(c, &w.G, (size_t)ld * ld)) || (s = psoci_alloc(c, &w.Y, (size_t)ld * ld)) ||
      (s = psoci_alloc(c, &w.theta, ld)) || (s = psoci_alloc(c, &w.X, (size_t)N * nr)) ||
      (s = psoci_alloc(c, &w.HX, (size_t)N * nr)) || (s = psoci_alloc(c, &w.R, (size_t)N * nr)) ||
      (s = psoci_alloc(c, &w.T, (size_t)N * nr)) || (s = psoci_alloc(c, &w.tmp, (size_t)N * std::max(nr, 2 * nr))) ||
      (s = psoci_alloc(c, &w.partial, (size_t)w.nblk * MAX_SUB * TN_MAXK)) ||
      (s = psoci_alloc(c, &w.small, (size_t)ld * ld)) || (s = psoci_alloc(c, &w.F, 16 * 16)) ||
      (s = psoci_alloc(c, &w.norms, 16)) || (s = psoci_alloc(c, &w.sel, 16)) || (s = psoci_alloc(c, &w.ibuf, 4)) ||
      (s = psoci_alloc(c, &w.idx, 16)))
    return s;
  if (o->prec == PSOCI_PREC_MIXED || o->prec == PSOCI_PREC_FF || o->refine)
    if ((s = psoci_alloc(c, &w.x32, (size_t)N * 16))) return s;  // FF staging: 8 float pairs per row
  cudaStream_t st = c->stream;
  const size_t jac_smem = sizeof(double) * 2 * MAX_SUB * MAX_SUB;
  PSOCI_CUDA(c, cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jac_smem));
  PSOCI_CUDA(c, cudaMemsetAsync(w.V, 0, sizeof(double) * N * ld, st));
  PSOCI_CUDA(c, cudaMemsetAsync(w.G, 0, sizeof(double) * ld * ld, st));

  // guess: the lowest eigenvectors of H restricted to the M lowest diagonal elements (a
  // stored matrix), else unit vectors on the nr lowest diagonal elements
  const int M = inner ? nr : (int)std::min<int64_t>(GUESS_M, N);
  std::vector<int64_t> order;
  if ((s = lowest_elements(c, diag, N, M, order))) return s;
  psoci_prec prec = o->prec;
  bool refine_phase = (prec != PSOCI_PREC_MIXED);  // FP64 and FF iterate to rtol directly
  w.lowp = (prec == PSOCI_PREC_MIXED);
  const double tol_mixed = std::max(rtol, 1e-5);
  int m = nr;
  if (!inner && c->guess_k > 0 && (int64_t)c->guess.size() == (int64_t)c->guess_k * N) {
    // restart vectors first, unit vectors on the lowest diagonal elements for the rest;
    // orthonormalised like any new block
    std::vector<double> t0((size_t)N * nr, 0.0);
    const int kg = std::min(nr, c->guess_k);
    for (int j = 0; j < kg; ++j)
      for (int64_t r = 0; r < N; ++r) t0[(size_t)r * nr + j] = c->guess[(size_t)j * N + r];
    for (int j = kg; j < nr; ++j) t0[(size_t)order[j - kg] * nr + j] = 1.0;
    PSOCI_CUDA(c, cudaMemcpyAsync(w.T, t0.data(), sizeof(double) * N * nr, cudaMemcpyHostToDevice, st));
    int bk = 0;
    if ((s = orthonormalize(w, 0, nr, &bk))) return s;
    if (bk < 1) return psoci_fail(c, PSOCI_ERR_NUMERIC, "davidson: restart vectors are linearly dependent");
    m = bk;
    PSOCI_CUDA(c, cudaStreamSynchronize(st));
  } else if (!inner && !c->direct && c->d_val && M > nr) {
    // the block of H on the M lowest diagonal elements (a stored matrix), its lowest
    // eigenvectors scattered into V: a one-CTA Jacobi when it fits in shared memory, else
    // this solver run on the dense block (FP64, residuals to 1e-4)
    int64_t *gidx = nullptr;
    int32_t *map = nullptr;
    double *Hs = nullptr, *Ys = nullptr, *ths = nullptr, *dg = nullptr;
    int *jst = nullptr;
    auto release = [&]() {
      psoci_free(gidx); psoci_free(map); psoci_free(Hs); psoci_free(Ys); psoci_free(ths); psoci_free(jst);
      psoci_free(dg);
    };
    const bool small = M <= MAX_SUB;
    if ((s = psoci_alloc(c, &gidx, M)) || (s = psoci_alloc(c, &map, N)) || (s = psoci_alloc(c, &Hs, (size_t)M * M)) ||
        (s = psoci_alloc(c, &Ys, small ? (size_t)M * M : (size_t)M * nr)) || (s = psoci_alloc(c, &ths, M)) ||
        (s = psoci_alloc(c, &jst, 1)) || (s = psoci_alloc(c, &dg, M))) {
      release();
      return s;
    }
    cudaError_t e = cudaMemcpyAsync(gidx, order.data(), sizeof(int64_t) * M, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(map, 0xff, sizeof(int32_t) * N, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(Hs, 0, sizeof(double) * M * M, st);
    if (e == cudaSuccess) {
      psoci_note_launch();
      k_map_set<<<(M + 127) / 128, 128, 0, st>>>(gidx, M, map);
      psoci_note_launch();
      k_extract_block<<<(M + 7) / 8, 256, 0, st>>>(c->d_rowptr, c->d_col, c->d_val, gidx, M, map, Hs);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && small) {
      psoci_note_launch();
      k_jacobi<<<1, 256, jac_smem, st>>>(Hs, M, M, ths, Ys, 60, jst);
      psoci_note_launch();
      k_scatter_guess<<<1, 256, 0, st>>>(Ys, M, gidx, M, nr, w.V, ld);
      e = cudaGetLastError();
    } else if (e == cudaSuccess) {
      // diagonal of the block (stride M + 1), then the inner solve
      e = cudaMemcpy2DAsync(dg, sizeof(double), Hs, sizeof(double) * (M + 1), sizeof(double), M,
                            cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) {
        psoci_dav_opts oi = *o;
        oi.rtol = 1e-4;
        oi.prec = PSOCI_PREC_FP64;
        oi.refine = 0;
        oi.block = 1;
        oi.max_iter = 100;
        const psoci_status si = davidson_run(c, M, dg, Hs, &oi, true, nullptr, nullptr, nullptr, nullptr, Ys);
        if (si != PSOCI_OK && si != PSOCI_ERR_NOT_CONVERGED) {
          release();
          return si;
        }
        psoci_note_launch();
        k_scatter_guess<<<(M * nr + 255) / 256, 256, 0, st>>>(Ys, nr, gidx, M, nr, w.V, ld);
        e = cudaGetLastError();
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    release();
    if (e != cudaSuccess) return psoci_cuda_fail(c, e, "davidson: initial block");
  } else {
    PSOCI_CUDA(c, cudaMemcpyAsync(w.idx, order.data(), sizeof(int64_t) * nr, cudaMemcpyHostToDevice, st));
    psoci_note_launch();
    k_set_unit<<<1, 32, 0, st>>>(w.V, ld, 0, w.idx, nr);
  }
  int iters = 0, sigma_calls = 0, collapses = 0, refine_iters = 0;
  if ((s = sigma_block(w, w.V, ld, w.HV, ld, m, prec))) return s;
  sigma_calls += m;
  if ((s = tn(w, w.V, ld, 0, m, w.HV, ld, 0, m, w.G, ld, 0))) return s;
  psoci_note_launch();
  k_symmetrize<<<1, 256, 0, st>>>(w.G, ld, 0, m);

  std::vector<double> h_norm(nr), h_theta(ld), h_g((size_t)ld * ld), h_y((size_t)ld * ld);
  std::vector<int> sel;
  bool done = false, stalled = false;
  double best_mixed = HUGE_VAL;  // smallest largest-residual of the FP32-element phase so far
  int no_gain = 0;               // iterations since it last fell by 30%
  psoci_status result = PSOCI_OK;
  while (!done) {
    if (iters >= max_iter) { result = PSOCI_ERR_NOT_CONVERGED; break; }
    ++iters;
    if (refine_phase && prec != o->prec) ++refine_iters;
    // Rayleigh-Ritz on the host (the reference's dsygv; the basis is orthonormal, so the
    // metric is the identity): G down, eigenpairs up
    PSOCI_CUDA(c, cudaMemcpy2DAsync(h_g.data(), sizeof(double) * ld, w.G, sizeof(double) * ld, sizeof(double) * m, m,
                                    cudaMemcpyDeviceToHost, st));
    PSOCI_CUDA(c, cudaStreamSynchronize(st));
    if (psoci_subspace_eigen(m, h_g.data(), ld, h_theta.data(), h_y.data(), ld) != PSOCI_OK)
      return psoci_fail(c, PSOCI_ERR_NUMERIC, "davidson: subspace eigen-solve failed");
    PSOCI_CUDA(c, cudaMemcpy2DAsync(w.Y, sizeof(double) * ld, h_y.data(), sizeof(double) * ld, sizeof(double) * m, m,
                                    cudaMemcpyHostToDevice, st));
    PSOCI_CUDA(c, cudaMemcpyAsync(w.theta, h_theta.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
    // Ritz vectors, their images and residuals
    if ((s = nn(w, w.V, ld, 0, m, w.Y, ld, 0, nr, 1.0, 0.0, w.X, nr, 0))) return s;
    if ((s = nn(w, w.HV, ld, 0, m, w.Y, ld, 0, nr, 1.0, 0.0, w.HX, nr, 0))) return s;
    int rb = (int)std::min<int64_t>((N + 255) / 256, 152 * 4);
    psoci_note_launch();
    k_residual<<<rb, 256, 0, st>>>(N, nr, w.X, w.HX, w.theta, w.R, w.partial);
    psoci_note_launch();
    k_sum_cols<<<1, 32, 0, st>>>(w.partial, rb, nr, w.norms);
    PSOCI_CUDA(c, cudaGetLastError());
    PSOCI_CUDA(c, cudaMemcpyAsync(h_norm.data(), w.norms, sizeof(double) * nr, cudaMemcpyDeviceToHost, st));
    PSOCI_CUDA(c, cudaStreamSynchronize(st));
    for (int j = 0; j < nr; ++j) {
      if (!std::isfinite(h_norm[j]) || !std::isfinite(h_theta[j]))
        return psoci_fail(c, PSOCI_ERR_NUMERIC, "davidson: non-finite residual or Ritz value");
      h_norm[j] = std::sqrt(h_norm[j]);
    }
    const double tol = refine_phase ? rtol : tol_mixed;
    if (!refine_phase) {
      // the FP32-element phase has a residual floor (FP32 elements, FP32 subspace products);
      // when the largest residual stops falling near it, refine from there
      const double mx = *std::max_element(h_norm.begin(), h_norm.end());
      if (mx < 0.7 * best_mixed) {
        best_mixed = mx;
        no_gain = 0;
      } else if (++no_gain >= 4 && best_mixed < 1e-3) {
        stalled = true;
      }
    }
    sel.clear();
    for (int j = 0; j < nr; ++j)
      if (h_norm[j] > tol) {
        sel.push_back(j);
        if (!o->block) break;
      }
    if (c->verbose)
      fprintf(stderr, "psoci davidson%s it=%d m=%d %s max|r|=%.3e e0=%.12f\n", inner ? " (guess block)" : "", iters, m,
              refine_phase ? "fp64" : "mixed", *std::max_element(h_norm.begin(), h_norm.end()), h_theta[0]);
    if (sel.empty() || stalled) {
      stalled = false;
      if (!refine_phase && o->refine) {
        // FP64 refinement: restart from the Ritz vectors with exact (FP64) H products
        refine_phase = true;
        prec = (o->refine == 2) ? PSOCI_PREC_FP64 : PSOCI_PREC_FF;
        w.lowp = false;
        if ((s = nn(w, w.V, ld, 0, m, w.Y, ld, 0, nr, 1.0, 0.0, w.T, nr, 0))) return s;
        int bk = 0;
        if ((s = orthonormalize(w, 0, nr, &bk))) return s;
        m = bk;
        if (m == 0) return psoci_fail(c, PSOCI_ERR_NUMERIC, "davidson: refinement basis collapsed");
        if ((s = sigma_block(w, w.V, ld, w.HV, ld, m, prec))) return s;
        sigma_calls += m;
        if ((s = tn(w, w.V, ld, 0, m, w.HV, ld, 0, m, w.G, ld, 0))) return s;
        psoci_note_launch();
        k_symmetrize<<<1, 256, 0, st>>>(w.G, ld, 0, m);
        continue;
      }
      done = true;
      break;
    }
    int nsel = (int)sel.size();
    PSOCI_CUDA(c, cudaMemcpyAsync(w.sel, sel.data(), sizeof(int) * nsel, cudaMemcpyHostToDevice, st));
    psoci_note_launch();
    {
      const int pb = (int)std::min<int64_t>((N * nsel + 255) / 256, 152 * 16);
      if (N * 32 < (int64_t)UINT32_MAX)
        k_precond<uint32_t><<<pb, 256, 0, st>>>(N, nr, w.R, diag, w.theta, w.sel, nsel, dmin, w.T, nr);
      else
        k_precond<uint64_t><<<pb, 256, 0, st>>>(N, nr, w.R, diag, w.theta, w.sel, nsel, dmin, w.T, nr);
    }
    PSOCI_CUDA(c, cudaGetLastError());
    if (m + nsel > maxsub) {
      // collapse onto the lowest keep Ritz vectors (reference: 2*nroots), V and HV alike
      const int keep = std::min(m, std::max(nr, std::min(2 * nr, maxsub - nsel)));
      if ((s = nn(w, w.V, ld, 0, m, w.Y, ld, 0, keep, 1.0, 0.0, w.tmp, 2 * nr, 0))) return s;
      copy_cols(w, w.tmp, 2 * nr, w.V, ld, keep);
      if ((s = nn(w, w.HV, ld, 0, m, w.Y, ld, 0, keep, 1.0, 0.0, w.tmp, 2 * nr, 0))) return s;
      copy_cols(w, w.tmp, 2 * nr, w.HV, ld, keep);
      // G = diag(theta[0:keep]) over the new basis
      std::fill(h_g.begin(), h_g.end(), 0.0);
      for (int i = 0; i < keep; ++i) h_g[(size_t)i * ld + i] = h_theta[i];
      PSOCI_CUDA(c, cudaMemcpy2DAsync(w.G, sizeof(double) * ld, h_g.data(), sizeof(double) * ld,
                                      sizeof(double) * keep, keep, cudaMemcpyHostToDevice, st));
      m = keep;
      ++collapses;
    }
    int bk = 0;
    if ((s = orthonormalize(w, m, nsel, &bk))) return s;
    if (bk == 0) {
      // no new direction survived the orthonormalisation: in the FP32-element phase the
      // basis has reached what that phase resolves, so refine from the current Ritz vectors
      // (next pass); otherwise the solve is stuck
      if (!refine_phase && o->refine) {
        stalled = true;
        continue;
      }
      result = PSOCI_ERR_NOT_CONVERGED;
      break;
    }
    if ((s = sigma_block(w, w.V + m, ld, w.HV + m, ld, bk, prec))) return s;
    sigma_calls += bk;
    if ((s = tn(w, w.V, ld, 0, m + bk, w.HV, ld, m, bk, w.G, ld, m, true))) return s;
    psoci_note_launch();
    k_symmetrize<<<1, 256, 0, st>>>(w.G, ld, m, m + bk);
    PSOCI_CUDA(c, cudaGetLastError());
    m += bk;
  }
  PSOCI_CUDA(c, cudaStreamSynchronize(st));
  // outputs
  if (evals) for (int j = 0; j < nr; ++j) evals[j] = h_theta[j];
  if (rnorms) for (int j = 0; j < nr; ++j) rnorms[j] = h_norm[j];
  if (evecs) {
    std::vector<double> hx((size_t)N * nr);
    PSOCI_CUDA(c, cudaMemcpy(hx.data(), w.X, sizeof(double) * N * nr, cudaMemcpyDeviceToHost));
    for (int64_t r = 0; r < N; ++r)
      for (int j = 0; j < nr; ++j) evecs[(size_t)j * N + r] = hx[(size_t)r * nr + j];
  }
  if (stats) {
    stats->iterations = iters;
    stats->sigma_calls = sigma_calls;
    stats->collapses = collapses;
    stats->refine_iters = refine_iters;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    double sig = 0.0;
    for (size_t e = 0; e + 1 < w.ev.size(); e += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, w.ev[e], w.ev[e + 1]) == cudaSuccess) sig += ms * 1e-3;
    }
    stats->sigma_seconds = sig;
  }
  if (dX_out) PSOCI_CUDA(c, cudaMemcpyAsync(dX_out, w.X, sizeof(double) * N * nr, cudaMemcpyDeviceToDevice, st));
  if (result != PSOCI_OK)
    return inner ? result : psoci_fail(c, result, "davidson: did not converge within the iteration limit");
  return PSOCI_OK;
}

}  // namespace

psoci_status psoci_davidson_impl(psoci_ctx *c, const psoci_dav_opts *o, double *evals, double *evecs, double *rnorms,
                                 psoci_dav_stats *stats) {
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "davidson: Hamiltonian not built");
  if (!o) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "davidson: null options");
  return davidson_run(c, c->nsef_total, c->d_diag, nullptr, o, false, evals, evecs, rnorms, stats, nullptr);
}

// ------------------------------------------------------------------------------------
// Step-level Davidson: the basis and subspace objects of the reference's own loop
// (driver.PSOCI.splittest.C:1186-1311), kept on the device between calls so that a host
// program can keep that loop line for line:
//   PsociGAbasis    (PsociGAbasis.C)    vectors V and products HV, guess, orthonormalisation,
//                                       H*v products, precondition, append, expand-and-replace
//   PsociGAsubspace (PsociGAsubspace.C) new columns of the projected matrix, its eigen-solve,
//                                       residual norms
// The basis is kept orthonormal (CGS2 + Cholesky-QR twice, as psoci_davidson does), so the
// overlap matrix S of generateIncrementalSubspace is the identity and diagSubspaceGOP's dsygv
// reduces to a symmetric eigen-solve.  psoci_davidson stays the fast path: it advances all
// unconverged roots per iteration and runs its FP32-element phase with FP32 subspace products.
// ------------------------------------------------------------------------------------
namespace {

// R[r, col] = HX[r, col] - theta * X[r, col] (row stride ld) and the block partial sums of
// its squares
__global__ void k_residual_col(int64_t n, int ld, int col, const double *__restrict__ X,
                               const double *__restrict__ HX, const double *__restrict__ theta,
                               double *__restrict__ R, double *__restrict__ partial) {
  __shared__ double red[8];
  const double th = *theta;
  double s = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double v = HX[r * ld + col] - th * X[r * ld + col];
    R[r * ld + col] = v;
    s = fma(v, v, s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}

__global__ void k_set_diag(double *G, int ld, int m, const double *theta) {
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int i = e / m, j = e % m;
    G[i * ld + j] = (i == j) ? theta[i] : 0.0;
  }
}

}  // namespace

struct psoci_dav_basis {
  Work w;
  int nr = 0;         // sought roots
  int maxv = 0;       // vectors the basis holds
  int m = 0;          // existing vectors
  int products = 0;   // vectors 0..products-1 have their H*v
  int gcols = 0;      // columns of G formed
  bool have_eig = false;
  int eig_m = 0;      // basis size of the last eigen-solve (Y is eig_m x eig_m)
  bool scratch = false;          // T[:, 0] holds a preconditioned vector ready to append
  unsigned res_valid = 0;        // bit j: R[:, j] is the residual of root j+1 of the current eigen-solve
  std::vector<double> h_theta, h_y, h_g;
  double *shift = nullptr;       // device [16]: the preconditioner's shift at the root's slot
  int64_t N = 0;
  ~psoci_dav_basis() { psoci_free(shift); }
};

void psoci_basis_release(psoci_ctx *c) {
  delete c->basis;
  c->basis = nullptr;
}

namespace {
psoci_status basis_ready(psoci_ctx *c, const char *what) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!c->basis) return psoci_fail(c, PSOCI_ERR_STATE, std::string(what) + ": no basis (psoci_basis_create)");
  if (!c->have_h || c->basis->N != c->nsef_total)
    return psoci_fail(c, PSOCI_ERR_STATE, std::string(what) + ": the Hamiltonian changed since psoci_basis_create");
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  return PSOCI_OK;
}
}  // namespace

extern "C" {

psoci_status psoci_basis_create(psoci_ctx *c, int nroots, int max_vectors) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "basis_create: Hamiltonian not built");
  const int64_t N = c->nsef_total;
  if (nroots < 1 || nroots > 16 || nroots > N)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_create: nroots must be 1..16 and <= N");
  if (max_vectors < nroots + 1 || max_vectors > MAX_SUB || max_vectors > N)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_create: max_vectors must be nroots+1..96 and <= N");
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  psoci_basis_release(c);
  psoci_dav_basis *b = new psoci_dav_basis();
  c->basis = b;
  Work &w = b->w;
  b->nr = nroots;
  b->maxv = max_vectors;
  b->N = N;
  w.c = c;
  w.N = N;
  w.nr = nroots;
  w.ld = (max_vectors + 1) & ~1;
  const int ld = w.ld;
  w.nblk = (int)std::min<int64_t>(std::max<int64_t>(1, (N + 255) / 256), 152 * 4);
  w.rows_per_blk = (N + w.nblk - 1) / w.nblk;
  psoci_status s;
  if ((s = psoci_alloc(c, &w.V, (size_t)N * ld)) || (s = psoci_alloc(c, &w.HV, (size_t)N * ld)) ||
      (s = psoci_alloc(c, &w.G, (size_t)ld * ld)) || (s = psoci_alloc(c, &w.Y, (size_t)ld * ld)) ||
      (s = psoci_alloc(c, &w.theta, ld)) || (s = psoci_alloc(c, &w.X, (size_t)N * nroots)) ||
      (s = psoci_alloc(c, &w.HX, (size_t)N * nroots)) || (s = psoci_alloc(c, &w.R, (size_t)N * nroots)) ||
      (s = psoci_alloc(c, &w.T, (size_t)N * nroots)) || (s = psoci_alloc(c, &w.tmp, (size_t)N * ld)) ||
      (s = psoci_alloc(c, &w.partial, (size_t)w.nblk * MAX_SUB * TN_MAXK)) ||
      (s = psoci_alloc(c, &w.small, (size_t)ld * ld)) || (s = psoci_alloc(c, &w.F, 16 * 16)) ||
      (s = psoci_alloc(c, &w.norms, 16)) || (s = psoci_alloc(c, &w.sel, 16)) || (s = psoci_alloc(c, &w.ibuf, 4)) ||
      (s = psoci_alloc(c, &w.idx, 16)) || (s = psoci_alloc(c, &w.x32, (size_t)N * 16)) ||
      (s = psoci_alloc(c, &b->shift, 16))) {
    psoci_basis_release(c);
    return s;
  }
  b->h_theta.assign(ld, 0.0);
  b->h_y.assign((size_t)ld * ld, 0.0);
  b->h_g.assign((size_t)ld * ld, 0.0);
  PSOCI_CUDA(c, cudaMemsetAsync(w.V, 0, sizeof(double) * N * ld, c->stream));
  PSOCI_CUDA(c, cudaMemsetAsync(w.G, 0, sizeof(double) * ld * ld, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  return PSOCI_OK;
}

void psoci_basis_destroy(psoci_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  psoci_basis_release(c);
}

psoci_status psoci_basis_guess(psoci_ctx *c, int mode) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_guess"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  const int64_t N = b->N;
  const int nr = b->nr, ld = w.ld;
  cudaStream_t st = c->stream;
  if (mode < 0 || mode > 2) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_guess: mode must be 0, 1 or 2");
  std::vector<int64_t> order(nr);
  int kg = 0;
  if (mode == 0) {
    std::iota(order.begin(), order.end(), 0);
  } else {
    std::vector<double> hd(N);
    PSOCI_CUDA(c, cudaMemcpyAsync(hd.data(), c->d_diag, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    PSOCI_CUDA(c, cudaStreamSynchronize(st));
    std::vector<int64_t> all(N);
    std::iota(all.begin(), all.end(), 0);
    std::partial_sort(all.begin(), all.begin() + nr, all.end(),
                      [&](int64_t x, int64_t y) { return hd[x] < hd[y] || (hd[x] == hd[y] && x < y); });
    std::copy(all.begin(), all.begin() + nr, order.begin());
    if (mode == 2 && c->guess_k > 0 && (int64_t)c->guess.size() == (int64_t)c->guess_k * N) kg = std::min(nr, c->guess_k);
  }
  PSOCI_CUDA(c, cudaMemsetAsync(w.V, 0, sizeof(double) * N * ld, st));
  PSOCI_CUDA(c, cudaMemsetAsync(w.G, 0, sizeof(double) * ld * ld, st));
  if (kg > 0) {
    // restart vectors (root-major on the host) into the first columns, row-major on the device
    std::vector<double> t((size_t)N * kg);
    for (int j = 0; j < kg; ++j)
      for (int64_t r = 0; r < N; ++r) t[(size_t)r * kg + j] = c->guess[(size_t)j * N + r];
    PSOCI_CUDA(c, cudaMemcpy2DAsync(w.V, sizeof(double) * ld, t.data(), sizeof(double) * kg, sizeof(double) * kg, N,
                                    cudaMemcpyHostToDevice, st));
  }
  if (kg < nr) {
    PSOCI_CUDA(c, cudaMemcpyAsync(w.idx, order.data(), sizeof(int64_t) * (nr - kg), cudaMemcpyHostToDevice, st));
    psoci_note_launch();
    k_set_unit<<<1, 32, 0, st>>>(w.V, ld, kg, w.idx, nr - kg);
    PSOCI_CUDA(c, cudaGetLastError());
  }
  PSOCI_CUDA(c, cudaStreamSynchronize(st));
  b->m = nr;
  b->products = 0;
  b->gcols = 0;
  b->have_eig = false;
  b->scratch = false;
  b->res_valid = 0;
  return PSOCI_OK;
}

psoci_status psoci_basis_orthonormalize_all(psoci_ctx *c, int *dependent_at) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_orthonormalize_all"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  if (dependent_at) *dependent_at = 0;
  if (b->m > b->nr)
    return psoci_fail(c, PSOCI_ERR_UNSUPPORTED, "basis_orthonormalize_all: at most nroots vectors (the guess set)");
  const int m = b->m;
  if (m == 0) return PSOCI_OK;
  copy_cols(w, w.V, w.ld, w.T, w.nr, m);
  PSOCI_CUDA(c, cudaMemsetAsync(w.V, 0, sizeof(double) * b->N * w.ld, c->stream));
  int bk = 0;
  if ((s = orthonormalize(w, 0, m, &bk))) return s;
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  b->products = 0;
  b->gcols = 0;
  b->have_eig = false;
  b->res_valid = 0;
  if (bk < m) {
    b->m = bk;
    if (dependent_at) *dependent_at = bk + 1;
    return psoci_fail(c, PSOCI_ERR_NUMERIC, "basis_orthonormalize_all: linear dependency among the vectors");
  }
  return PSOCI_OK;
}

psoci_status psoci_basis_compute_hv(psoci_ctx *c, int start, int num, psoci_prec prec) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_compute_hv"))) return s;
  psoci_dav_basis *b = c->basis;
  if (start < 0 || num < 1 || start + num > b->m)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_compute_hv: columns outside the existing vectors");
  if (start > b->products) return psoci_fail(c, PSOCI_ERR_STATE, "basis_compute_hv: earlier products missing");
  if (prec == PSOCI_PREC_MIXED && !c->d_val32 && !c->direct)
    return psoci_fail(c, PSOCI_ERR_STATE, "basis_compute_hv: MIXED needs PSOCI_HMODE_CSR_BOTH");
  Work &w = b->w;
  if ((s = sigma_block(w, w.V + start, w.ld, w.HV + start, w.ld, num, prec))) return s;
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  b->products = std::max(b->products, start + num);
  return PSOCI_OK;
}

psoci_status psoci_subspace_generate_incremental(psoci_ctx *c, int num) {
  psoci_status s;
  if ((s = basis_ready(c, "subspace_generate_incremental"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  const int m = b->m;
  if (num < 1 || num > m) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "subspace_generate_incremental: bad num");
  if (b->products < m) return psoci_fail(c, PSOCI_ERR_STATE, "subspace_generate_incremental: H*v products missing");
  if (m - num > b->gcols) return psoci_fail(c, PSOCI_ERR_STATE, "subspace_generate_incremental: earlier columns missing");
  for (int c0 = m - num; c0 < m; c0 += TN_MAXK) {
    const int k = std::min(TN_MAXK, m - c0);
    if ((s = tn(w, w.V, w.ld, 0, m, w.HV, w.ld, c0, k, w.G, w.ld, c0))) return s;
  }
  psoci_note_launch();
  k_symmetrize<<<1, 256, 0, c->stream>>>(w.G, w.ld, m - num, m);
  PSOCI_CUDA(c, cudaGetLastError());
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  b->gcols = m;
  b->have_eig = false;
  b->res_valid = 0;
  return PSOCI_OK;
}

psoci_status psoci_subspace_diag(psoci_ctx *c, double *evals) {
  psoci_status s;
  if ((s = basis_ready(c, "subspace_diag"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  const int m = b->m, ld = w.ld;
  if (m < 1 || b->gcols < m) return psoci_fail(c, PSOCI_ERR_STATE, "subspace_diag: projected matrix incomplete");
  cudaStream_t st = c->stream;
  PSOCI_CUDA(c, cudaMemcpy2DAsync(b->h_g.data(), sizeof(double) * ld, w.G, sizeof(double) * ld, sizeof(double) * m, m,
                                  cudaMemcpyDeviceToHost, st));
  PSOCI_CUDA(c, cudaStreamSynchronize(st));
  if (psoci_subspace_eigen(m, b->h_g.data(), ld, b->h_theta.data(), b->h_y.data(), ld) != PSOCI_OK)
    return psoci_fail(c, PSOCI_ERR_NUMERIC, "subspace_diag: eigen-solve failed");
  for (int j = 0; j < m; ++j)
    if (!std::isfinite(b->h_theta[j])) return psoci_fail(c, PSOCI_ERR_NUMERIC, "subspace_diag: non-finite Ritz value");
  PSOCI_CUDA(c, cudaMemcpy2DAsync(w.Y, sizeof(double) * ld, b->h_y.data(), sizeof(double) * ld, sizeof(double) * m, m,
                                  cudaMemcpyHostToDevice, st));
  PSOCI_CUDA(c, cudaMemcpyAsync(w.theta, b->h_theta.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
  PSOCI_CUDA(c, cudaStreamSynchronize(st));
  if (evals) std::copy(b->h_theta.begin(), b->h_theta.begin() + m, evals);
  b->have_eig = true;
  b->eig_m = m;
  b->res_valid = 0;
  return PSOCI_OK;
}

namespace {
// residual of root j (0-based) of the current eigen-solve into R[:, j]; |r|^2 to *nrm2
psoci_status basis_residual(psoci_ctx *c, int j, double *nrm2) {
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  psoci_status s;
  const int nr = b->nr;
  if ((s = nn(w, w.V, w.ld, 0, b->eig_m, w.Y, w.ld, j, 1, 1.0, 0.0, w.X, nr, j))) return s;
  if ((s = nn(w, w.HV, w.ld, 0, b->eig_m, w.Y, w.ld, j, 1, 1.0, 0.0, w.HX, nr, j))) return s;
  const int rb = (int)std::min<int64_t>((b->N + 255) / 256, 152 * 4);
  psoci_note_launch();
  k_residual_col<<<rb, 256, 0, c->stream>>>(b->N, nr, j, w.X, w.HX, w.theta + j, w.R, w.partial);
  psoci_note_launch();
  k_sum_cols<<<1, 32, 0, c->stream>>>(w.partial, rb, 1, w.norms);
  PSOCI_CUDA(c, cudaGetLastError());
  PSOCI_CUDA(c, cudaMemcpyAsync(nrm2, w.norms, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  b->res_valid |= 1u << j;
  return PSOCI_OK;
}
}  // namespace

psoci_status psoci_subspace_rnorm_single(psoci_ctx *c, int iroot, double *rnorm) {
  psoci_status s;
  if ((s = basis_ready(c, "subspace_rnorm_single"))) return s;
  psoci_dav_basis *b = c->basis;
  if (!rnorm) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "subspace_rnorm_single: null rnorm");
  if (!b->have_eig) return psoci_fail(c, PSOCI_ERR_STATE, "subspace_rnorm_single: no eigen-solve (psoci_subspace_diag)");
  if (iroot < 1 || iroot > b->nr || iroot > b->eig_m)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "subspace_rnorm_single: root outside 1..nroots");
  double r2 = 0.0;
  if ((s = basis_residual(c, iroot - 1, &r2))) return s;
  if (!std::isfinite(r2)) return psoci_fail(c, PSOCI_ERR_NUMERIC, "subspace_rnorm_single: non-finite residual");
  *rnorm = std::sqrt(r2);
  return PSOCI_OK;
}

psoci_status psoci_subspace_rnorms(psoci_ctx *c, double *rnorms) {
  psoci_status s;
  if ((s = basis_ready(c, "subspace_rnorms"))) return s;
  psoci_dav_basis *b = c->basis;
  if (!rnorms) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "subspace_rnorms: null rnorms");
  if (!b->have_eig) return psoci_fail(c, PSOCI_ERR_STATE, "subspace_rnorms: no eigen-solve (psoci_subspace_diag)");
  const int n = std::min(b->nr, b->eig_m);
  for (int j = 0; j < n; ++j) {
    double r2 = 0.0;
    if ((s = basis_residual(c, j, &r2))) return s;
    if (!std::isfinite(r2)) return psoci_fail(c, PSOCI_ERR_NUMERIC, "subspace_rnorms: non-finite residual");
    rnorms[j] = std::sqrt(r2);
  }
  return PSOCI_OK;
}

psoci_status psoci_basis_precondition_new(psoci_ctx *c, int curroot, double shift, double precond_min) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_precondition_new"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  if (curroot < 1 || curroot > b->nr) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_precondition_new: bad root");
  if (!(b->res_valid & (1u << (curroot - 1))))
    return psoci_fail(c, PSOCI_ERR_STATE, "basis_precondition_new: no residual of this root (psoci_subspace_rnorm_single)");
  const int j = curroot - 1;
  const double dmin = precond_min > 0 ? precond_min : 1e-3;
  cudaStream_t st = c->stream;
  PSOCI_CUDA(c, cudaMemcpyAsync(b->shift + j, &shift, sizeof(double), cudaMemcpyHostToDevice, st));
  PSOCI_CUDA(c, cudaMemcpyAsync(w.sel, &j, sizeof(int), cudaMemcpyHostToDevice, st));
  const int pb = (int)std::min<int64_t>((b->N + 255) / 256, 152 * 16);
  psoci_note_launch();
  if (b->N * 32 < (int64_t)UINT32_MAX)
    k_precond<uint32_t><<<pb, 256, 0, st>>>(b->N, b->nr, w.R, c->d_diag, b->shift, w.sel, 1, dmin, w.T, b->nr);
  else
    k_precond<uint64_t><<<pb, 256, 0, st>>>(b->N, b->nr, w.R, c->d_diag, b->shift, w.sel, 1, dmin, w.T, b->nr);
  PSOCI_CUDA(c, cudaGetLastError());
  PSOCI_CUDA(c, cudaStreamSynchronize(st));
  b->scratch = true;
  return PSOCI_OK;
}

psoci_status psoci_basis_append_scratch(psoci_ctx *c, psoci_prec prec, int *appended) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_append_scratch"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  if (appended) *appended = 0;
  if (!b->scratch) return psoci_fail(c, PSOCI_ERR_STATE, "basis_append_scratch: no preconditioned vector");
  if (b->m + 1 > b->maxv)
    return psoci_fail(c, PSOCI_ERR_STATE, "basis_append_scratch: basis full (psoci_basis_expand_replace first)");
  if (b->products < b->m) return psoci_fail(c, PSOCI_ERR_STATE, "basis_append_scratch: H*v products missing");
  if (prec == PSOCI_PREC_MIXED && !c->d_val32 && !c->direct)
    return psoci_fail(c, PSOCI_ERR_STATE, "basis_append_scratch: MIXED needs PSOCI_HMODE_CSR_BOTH");
  int bk = 0;
  if ((s = orthonormalize(w, b->m, 1, &bk))) return s;
  b->scratch = false;
  b->res_valid = 0;
  if (bk == 0) return PSOCI_OK;  // no new direction: the basis is unchanged
  if ((s = sigma_block(w, w.V + b->m, w.ld, w.HV + b->m, w.ld, bk, prec))) return s;
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  b->m += bk;
  b->products = b->m;
  if (appended) *appended = bk;
  return PSOCI_OK;
}

psoci_status psoci_basis_expand_replace(psoci_ctx *c, int num) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_expand_replace"))) return s;
  psoci_dav_basis *b = c->basis;
  Work &w = b->w;
  const int m = b->eig_m, ld = w.ld;
  if (!b->have_eig) return psoci_fail(c, PSOCI_ERR_STATE, "basis_expand_replace: no eigen-solve (psoci_subspace_diag)");
  if (num < 1 || num > m)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_expand_replace: num outside 1..vectors of the last eigen-solve");
  if (b->products < m) return psoci_fail(c, PSOCI_ERR_STATE, "basis_expand_replace: H*v products missing");
  // V <- V[:, :m] Y[:, :num] and HV <- HV[:, :m] Y[:, :num] (no new products), through tmp;
  // m is the basis of the last eigen-solve, so vectors appended after it are dropped, as the
  // reference's expansion with the subspace eigenvectors drops them
  for (int pass = 0; pass < 2; ++pass) {
    double *A = pass == 0 ? w.V : w.HV;
    for (int c0 = 0; c0 < num; c0 += NN_MAXK) {
      const int k = std::min(NN_MAXK, num - c0);
      if ((s = nn(w, A, ld, 0, m, w.Y, ld, c0, k, 1.0, 0.0, w.tmp, ld, c0))) return s;
    }
    copy_cols(w, w.tmp, ld, A, ld, num);
  }
  psoci_note_launch();
  k_set_diag<<<1, 256, 0, c->stream>>>(w.G, ld, num, w.theta);
  PSOCI_CUDA(c, cudaGetLastError());
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  // the expanded vectors are the Ritz vectors: the eigen-solve of the new G is diagonal
  for (int i = 0; i < num; ++i)
    for (int j = 0; j < num; ++j) b->h_y[(size_t)i * ld + j] = (i == j) ? 1.0 : 0.0;
  PSOCI_CUDA(c, cudaMemcpy2DAsync(w.Y, sizeof(double) * ld, b->h_y.data(), sizeof(double) * ld, sizeof(double) * num,
                                  num, cudaMemcpyHostToDevice, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  b->m = num;
  b->products = num;
  b->gcols = num;
  b->eig_m = num;
  b->res_valid = 0;
  b->scratch = false;
  return PSOCI_OK;
}

psoci_status psoci_basis_info(const psoci_ctx *cc, int *existing, int *sought, int *max_vectors, int *products) {
  psoci_ctx *c = const_cast<psoci_ctx *>(cc);
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!c->basis) return psoci_fail(c, PSOCI_ERR_STATE, "basis_info: no basis (psoci_basis_create)");
  if (existing) *existing = c->basis->m;
  if (sought) *sought = c->basis->nr;
  if (max_vectors) *max_vectors = c->basis->maxv;
  if (products) *products = c->basis->products;
  return PSOCI_OK;
}

psoci_status psoci_basis_vectors(psoci_ctx *c, int k, double *vecs) {
  psoci_status s;
  if ((s = basis_ready(c, "basis_vectors"))) return s;
  psoci_dav_basis *b = c->basis;
  if (!vecs || k < 1 || k > b->m) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "basis_vectors: k outside 1..existing");
  std::vector<double> t((size_t)b->N * k);
  PSOCI_CUDA(c, cudaMemcpy2DAsync(t.data(), sizeof(double) * k, b->w.V, sizeof(double) * b->w.ld, sizeof(double) * k,
                                  b->N, cudaMemcpyDeviceToHost, c->stream));
  PSOCI_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int64_t r = 0; r < b->N; ++r)
    for (int j = 0; j < k; ++j) vecs[(size_t)j * b->N + r] = t[(size_t)r * k + j];
  return PSOCI_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------
// Tall-skinny projection C = A^T B three ways, for measuring the choice the Davidson makes
// (generateIncrementalSubspace, PsociGAsubspace.C:273-366): float-float on the FP32 pipe (the
// solver's k_tn), plain FP64 FMA, and FP64 tensor-core MMA (mma.sync m8n8k4 .f64 — the FP64
// matrix instruction sm_103a offers; tcgen05 has no FP64 kind).
// ------------------------------------------------------------------------------------
namespace {

constexpr int TP_THREADS = 256;

// FP64 FMA: thread (i, sub) accumulates row i of C (k <= 8 outputs) over the rows sub,
// sub + S, ... of its block's range; B's rows are read from global memory (8 consecutive
// doubles, broadcast within the warp), the sub shares added in FP64 in shared memory.
__global__ void __launch_bounds__(TP_THREADS) k_tn_f64(int64_t n, const double *__restrict__ A, int lda, int m,
                                                       const double *__restrict__ B, int ldb, int k,
                                                       double *__restrict__ partial, int64_t rows_per_blk) {
  __shared__ double red[TP_THREADS][8];
  const int tid = threadIdx.x;
  const int S = TP_THREADS / m;
  const int i = tid % m, sub = tid / m;
  double acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = 0.0;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_blk, r1 = min(n, r0 + rows_per_blk);
  if (sub < S)
    for (int64_t r = r0 + sub; r < r1; r += S) {
      const double a = __ldg(A + r * lda + i);
      const double *br = B + r * ldb;
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (j < k) acc[j] = fma(a, __ldg(br + j), acc[j]);
    }
#pragma unroll
  for (int j = 0; j < 8; ++j) red[tid][j] = (sub < S) ? acc[j] : 0.0;
  __syncthreads();
  for (int e = tid; e < m * k; e += TP_THREADS) {
    const int ii = e / k, j = e - ii * k;
    double s = 0.0;
    for (int q = 0; q < S; ++q) s += red[q * m + ii][j];
    partial[(int64_t)blockIdx.x * m * k + e] = s;
  }
}

// FP64 MMA: each warp sums C over its rows in steps of 4 with mma.sync.m8n8k4 (A^T's 8 x 4
// fragment: lane (i = lane / 4, kk = lane % 4) holds A[r + kk, 8t + i]; B's 4 x 8 fragment:
// lane (kk = lane % 4, j = lane / 4) holds B[r + kk, j]; the accumulator: lane holds C[8t +
// lane / 4, 2 (lane % 4) + {0, 1}]), one accumulator pair per 8-row tile of C (m <= 40: 5).
__global__ void __launch_bounds__(TP_THREADS) k_tn_dmma(int64_t n, const double *__restrict__ A, int lda, int m,
                                                        const double *__restrict__ B, int ldb, int k,
                                                        double *__restrict__ partial, int64_t rows_per_warp,
                                                        int64_t nwarps) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= nwarps) return;  // whole warps: the last block's spare warps
  const int mt = (m + 7) / 8;
  double c[5][2];
#pragma unroll
  for (int t = 0; t < 5; ++t) { c[t][0] = 0.0; c[t][1] = 0.0; }
  const int64_t r0 = warp * rows_per_warp, r1 = min(n, r0 + rows_per_warp);
  const int kk = lane & 3, hi = lane >> 2;
  for (int64_t r = r0; r < r1; r += 4) {
    const int64_t row = r + kk;
    const bool rv = row < r1;
    const double b = (rv && hi < k) ? __ldg(B + row * ldb + hi) : 0.0;
#pragma unroll
    for (int t = 0; t < 5; ++t) {
      if (t >= mt) break;
      const int col = 8 * t + hi;
      const double a = (rv && col < m) ? __ldg(A + row * lda + col) : 0.0;
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[t][0]), "+d"(c[t][1])
                   : "d"(a), "d"(b));
    }
  }
  double *pw = partial + warp * (int64_t)m * k;
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    if (t >= mt) break;
    const int i = 8 * t + hi;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int j = 2 * kk + q;
      if (i < m && j < k) pw[i * k + j] = c[t][q];
    }
  }
}

}  // namespace

extern "C" psoci_status psoci_tsprod(psoci_ctx *c, int method, int64_t n, const double *dA, int lda, int m,
                                     const double *dB, int ldb, int k, double *dC) {
  if (!c) return PSOCI_ERR_INVALID_ARG;
  if (!dA || !dB || !dC || n < 1 || m < 1 || m > 40 || k < 1 || k > 8 || lda < m || ldb < k)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "tsprod: sizes outside n >= 1, 1 <= m <= 40, 1 <= k <= 8");
  if (method < 0 || method > 2) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "tsprod: method must be 0, 1 or 2");
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  psoci_status s;
  if (method == 0) {
    // the solver's own path (float-float k_tn + reduction)
    Work w;
    w.c = c;
    w.N = n;
    w.nblk = (int)std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), 152 * 4);
    w.rows_per_blk = (n + w.nblk - 1) / w.nblk;
    if ((s = psoci_alloc(c, &w.partial, (size_t)w.nblk * MAX_SUB * TN_MAXK))) return s;
    s = tn(w, dA, lda, 0, m, dB, ldb, 0, k, dC, k, 0);
    if (s) return s;
    PSOCI_CUDA(c, cudaStreamSynchronize(st));
    return PSOCI_OK;
  }
  int nblk = 0;
  int64_t per = 0;
  if (method == 1) {
    nblk = (int)std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), 152 * 8);
    per = (n + nblk - 1) / nblk;
  } else {
    const int64_t warps = std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), 152 * 8 * (TP_THREADS / 32));
    nblk = (int)warps;  // partial sums per warp
    per = ((n + warps - 1) / warps + 3) / 4 * 4;
  }
  double *partial = nullptr;
  if ((s = psoci_alloc(c, &partial, (size_t)nblk * m * k))) return s;
  psoci_note_launch();
  if (method == 1) {
    k_tn_f64<<<nblk, TP_THREADS, 0, st>>>(n, dA, lda, m, dB, ldb, k, partial, per);
  } else {
    PSOCI_CUDA(c, cudaMemsetAsync(partial, 0, sizeof(double) * nblk * m * k, st));
    k_tn_dmma<<<(unsigned)((nblk + TP_THREADS / 32 - 1) / (TP_THREADS / 32)), TP_THREADS, 0, st>>>(n, dA, lda, m, dB,
                                                                                                  ldb, k, partial, per,
                                                                                                  (int64_t)nblk);
  }
  psoci_note_launch();
  k_reduce_partials<<<(m * k + 31) / 32, 256, 0, st>>>(partial, nblk, m, k, dC, k, 0);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  psoci_free(partial);
  if (e != cudaSuccess) return psoci_cuda_fail(c, e, "tsprod");
  return PSOCI_OK;
}
