// Sigma = H * X over k vectors from the stored CSR (both triangles).
//
// Reference: PsociGAhamiltonian::matrixVectorProductsSplitChunkMultipleJchunks
// (PsociGAhamiltonian.C:6921-7270) — one vector per call, lower-triangle storage, x chunks
// broadcast over MPI and partial y reduced with MPI_Allreduce.  Here all k vectors of a
// Davidson block go through one pass over H: a warp owns a row, streams its (col, val)
// pairs once (coalesced), gathers the k contiguous entries of X[col, :] (row-major X keeps
// one row of the block in one or two 32-byte sectors) and reduces k sums across lanes.
//
//   FP64 : FP64 elements, FP64 products and sums.
//   MIXED: FP32 elements and FP32 inputs, FP32 products, compensated FP32 (Kahan / float-
//          float) accumulation, FP64 result.
//   FF   : FP64 elements and inputs split into FP32 hi + lo pairs (inputs once per call,
//          elements as they stream), error-free float-float products and sums — about 47
//          significant bits on the FP32 pipe instead of FP64 on the FP64 pipe.  On GB300 the FP64 pipe issues ~2 FMA/clk/SM,
//          so a kernel that adds in FP64 per element is bound by that pipe, not by HBM.
#include <algorithm>

#include "ffmath.cuh"
#include "psoci_internal.cuh"

namespace {

constexpr int SIG_THREADS = 256;
// stored elements per lane whose gathers are in flight together; 4 was fastest for 8
// vectors (8.96 ms at the benchmark block, 9.13 with 6, 9.67 with 8)
constexpr int SIG_UNROLL = 4;

template <typename T>
__device__ __forceinline__ T ldg_stream(const T *p) { return __ldcs(p); }

// Reduce-scatter of 8 per-lane partial sums across a warp: three halving exchanges
// (offsets 16, 8, 4) leave each lane one partial, two butterflies (2, 1) finish the sum.
// Afterwards lanes 4q..4q+3 hold the total of value q.  9 shuffles instead of 40.
template <typename T, typename Add>
__device__ __forceinline__ T reduce_scatter8(T (&v)[8], int lane, Add add) {
  T a[4], b[2], c;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool hi = lane & 16;
    T send = hi ? v[i] : v[i + 4];
    T keep = hi ? v[i + 4] : v[i];
    a[i] = add(keep, __shfl_xor_sync(0xffffffffu, send, 16));
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool hi = lane & 8;
    T send = hi ? a[i] : a[i + 2];
    T keep = hi ? a[i + 2] : a[i];
    b[i] = add(keep, __shfl_xor_sync(0xffffffffu, send, 8));
  }
  {
    const bool hi = lane & 4;
    T send = hi ? b[0] : b[1];
    T keep = hi ? b[1] : b[0];
    c = add(keep, __shfl_xor_sync(0xffffffffu, send, 4));
  }
  c = add(c, __shfl_xor_sync(0xffffffffu, c, 2));
  c = add(c, __shfl_xor_sync(0xffffffffu, c, 1));
  return c;
}

// float-float pair (hi + lo) and its error-free addition (TwoSum, then renormalise)
struct ff2 {
  float h, l;
};
__device__ __forceinline__ ff2 ff_add(ff2 a, ff2 b) {
  float s = __fadd_rn(a.h, b.h);
  float bp = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bp)), __fsub_rn(b.h, bp));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  float h = __fadd_rn(s, e);
  return ff2{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ ff2 shfl_ff(ff2 v, int o) {
  return ff2{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}

template <int K>
__device__ __forceinline__ void store_reduced_f64(double (&acc)[K], int lane, double *yr) {
  double v[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = (q < K) ? acc[q] : 0.0;
  double tot = reduce_scatter8(v, lane, [](double x, double y) { return x + y; });
  const int q = lane >> 2;
  if ((lane & 3) == 0 && q < K) yr[q] = tot;
}

template <int K>
__global__ void __launch_bounds__(SIG_THREADS) k_spmm_f64(int64_t nrows, const int64_t *__restrict__ rowptr,
                                                          const int32_t *__restrict__ col,
                                                          const double *__restrict__ val,
                                                          const double *__restrict__ x, int ldx,
                                                          double *__restrict__ y, int ldy, bool vec2) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < nrows; r += nwarps) {
    double acc[K];
#pragma unroll
    for (int q = 0; q < K; ++q) acc[q] = 0.0;
    const int64_t e = rowptr[r + 1];
    for (int64_t t = rowptr[r] + lane; t < e; t += 32) {
      const int c = ldg_stream(col + t);
      const double v = ldg_stream(val + t);
      const double *xr = x + (int64_t)c * ldx;
      if (K % 2 == 0 && vec2) {
#pragma unroll
        for (int q = 0; q < K; q += 2) {
          const double2 xx = __ldg(reinterpret_cast<const double2 *>(xr + q));
          acc[q] = fma(v, xx.x, acc[q]);
          acc[q + 1] = fma(v, xx.y, acc[q + 1]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < K; ++q) acc[q] = fma(v, __ldg(xr + q), acc[q]);
      }
    }
    store_reduced_f64<K>(acc, lane, y + r * ldy);
  }
}

// the 8 floats at p (32-byte aligned) in one 256-bit load, cached in L2 only: the gathered
// rows are rarely reused from L1 (hit rate ~9%), and skipping it took 8% off the 8-vector
// sigma (128-bit rows of narrow blocks keep the read-only path, which was faster for them)
__device__ __forceinline__ void ldg_row8(float (&f)[8], const float *p) {
  asm("ld.global.cg.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]), "=f"(f[4]), "=f"(f[5]), "=f"(f[6]), "=f"(f[7])
      : "l"(p));
}

// the first XS (4 or 8) floats at p (aligned to XS floats) in one load
template <int XS>
__device__ __forceinline__ void ldg_row(float (&f)[8], const float *p) {
  if (XS == 8) {
    ldg_row8(f, p);
  } else {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    f[0] = v.x; f[1] = v.y; f[2] = v.z; f[3] = v.w;
    f[4] = f[5] = f[6] = f[7] = 0.f;
  }
}

// Kahan step: the rounding error of every addition is carried in c and fed back
__device__ __forceinline__ void kahan_add(float &s, float &c, float prod) {
  const float yv = __fsub_rn(prod, c);
  const float tt = __fadd_rn(s, yv);
  c = __fsub_rn(__fsub_rn(tt, s), yv);
  s = tt;
}

// MIXED: FP32 element x FP32 input products.  Each lane keeps a compensated FP32 sum per
// vector (Kahan: the rounding error of every addition is carried in c and fed back), so
// no FP64 arithmetic runs in the streaming loop — on GB300 the FP64 pipe, not HBM, would
// otherwise bound the kernel.  The lane sums (value + compensation) are combined as
// float-float pairs, FP64 only at the end.
//
// Variants (chosen per Hamiltonian by psoci_autotune_sigma): LPR lanes per row (32: a warp
// per row; 16: two rows per warp, for short rows) and UNR stored elements per lane whose
// gathers are in flight together.
template <int K, int LPR, int UNR>
__global__ void __launch_bounds__(SIG_THREADS) k_spmm_mixed(int64_t nrows, const int64_t *__restrict__ rowptr,
                                                            const int32_t *__restrict__ col,
                                                            const float *__restrict__ val,
                                                            const float *__restrict__ x, double *__restrict__ y,
                                                            int ldy) {
  // x: FP32 inputs with a row stride of XS floats (8 = 32 bytes for K > 4, 4 = 16 bytes for
  // K <= 4; aligned to the stride), so every gather is one 256- or 128-bit load — one L1
  // wavefront per gathered row, and half the bytes when the block is narrow
  constexpr int XS = (K <= 4) ? 4 : 8;
  constexpr int RPW = 32 / LPR;  // rows per warp
  const int lane = threadIdx.x & 31;
  const int sub = lane % LPR;  // lane within the row group
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // the warp takes RPW consecutive rows at a time, so all its lanes run the same number of
  // rounds (shuffles below)
  for (int64_t base = warp * RPW; base < nrows; base += nwarps * RPW) {
    const int64_t r = base + lane / LPR;
    const bool live = (RPW == 1) || r < nrows;
    float s[K], cmp[K];
#pragma unroll
    for (int q = 0; q < K; ++q) { s[q] = 0.f; cmp[q] = 0.f; }
    const int64_t e = live ? rowptr[r + 1] : 0;
    int64_t t = live ? rowptr[r] + sub : 0;
    // UNR elements per lane in flight: the gathers are latency-bound
    for (; t + LPR * (UNR - 1) < e; t += LPR * UNR) {
      int cc[UNR];
      float vv[UNR], xx[UNR][8];
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        cc[u] = ldg_stream(col + t + LPR * u);
        vv[u] = ldg_stream(val + t + LPR * u);
      }
#pragma unroll
      for (int u = 0; u < UNR; ++u) ldg_row<XS>(xx[u], x + (int64_t)cc[u] * XS);
#pragma unroll
      for (int u = 0; u < UNR; ++u)
#pragma unroll
        for (int q = 0; q < K; ++q) kahan_add(s[q], cmp[q], __fmul_rn(vv[u], xx[u][q]));
    }
    for (; t < e; t += LPR) {
      const int c = ldg_stream(col + t);
      const float v = ldg_stream(val + t);
      float xv[8];
      ldg_row<XS>(xv, x + (int64_t)c * XS);
#pragma unroll
      for (int q = 0; q < K; ++q) kahan_add(s[q], cmp[q], __fmul_rn(v, xv[q]));
    }
    // Kahan leaves sum = s - cmp; reduce (s, -cmp) as float-float pairs within the row group:
    // halving exchanges leave each lane one partial, butterflies finish the sum
    ff2 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = (q < K) ? ff2{s[q], -cmp[q]} : ff2{0.f, 0.f};
    ff2 a[4], b[2], cc;
    constexpr int O1 = LPR / 2, O2 = LPR / 4, O3 = LPR / 8;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const bool hi = lane & O1;
      a[i] = ff_add(hi ? v[i + 4] : v[i], shfl_ff(hi ? v[i] : v[i + 4], O1));
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const bool hi = lane & O2;
      b[i] = ff_add(hi ? a[i + 2] : a[i], shfl_ff(hi ? a[i] : a[i + 2], O2));
    }
    {
      const bool hi = lane & O3;
      cc = ff_add(hi ? b[1] : b[0], shfl_ff(hi ? b[0] : b[1], O3));
    }
#pragma unroll
    for (int o = O3 / 2; o > 0; o >>= 1) cc = ff_add(cc, shfl_ff(cc, o));
    // lanes sub = q * O3 ... hold value q (the halving steps sorted the values by the high bits)
    const int qq = (((sub & O1) ? 1 : 0) | ((sub & O2) ? 2 : 0) | ((sub & O3) ? 4 : 0));
    const int q = ((qq & 1) << 2) | (qq & 2) | ((qq & 4) >> 2);
    if (live && (sub & (O3 - 1)) == 0 && q < K) y[r * ldy + q] = (double)cc.h + (double)cc.l;
  }
}

// warp reduce-scatter of K float-float lane sums; the lane holding value q writes it
template <int K>
__device__ __forceinline__ void store_reduced_ff(ff2 (&v)[8], int lane, double *yr) {
  ff2 a[4], b[2], cc;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool hi = lane & 16;
    a[i] = ff_add(hi ? v[i + 4] : v[i], shfl_ff(hi ? v[i] : v[i + 4], 16));
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const bool hi = lane & 8;
    b[i] = ff_add(hi ? a[i + 2] : a[i], shfl_ff(hi ? a[i] : a[i + 2], 8));
  }
  {
    const bool hi = lane & 4;
    cc = ff_add(hi ? b[1] : b[0], shfl_ff(hi ? b[0] : b[1], 4));
  }
  cc = ff_add(cc, shfl_ff(cc, 2));
  cc = ff_add(cc, shfl_ff(cc, 1));
  const int qq = lane >> 2;
  if ((lane & 3) == 0 && qq < K) yr[qq] = (double)cc.h + (double)cc.l;
}

// FF: FP64 elements split as they stream, inputs pre-split into float pairs (x2, K per row)
template <int K>
__global__ void __launch_bounds__(SIG_THREADS) k_spmm_ff(int64_t nrows, const int64_t *__restrict__ rowptr,
                                                         const int32_t *__restrict__ col,
                                                         const double *__restrict__ val,
                                                         const float2 *__restrict__ x2, double *__restrict__ y,
                                                         int ldy) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < nrows; r += nwarps) {
    float sh[K], sl[K];
#pragma unroll
    for (int q = 0; q < K; ++q) { sh[q] = 0.f; sl[q] = 0.f; }
    const int64_t e = rowptr[r + 1];
    for (int64_t t = rowptr[r] + lane; t < e; t += 32) {
      const int c = ldg_stream(col + t);
      const float2 v = split_f64(ldg_stream(val + t));
      const float2 *xr = x2 + (int64_t)c * K;
      float2 xv[K];
      if (K == 8) {
        // 8 pairs = 64 contiguous, 64-byte-aligned bytes: two 256-bit loads
        float f[16];
        asm("ld.global.cg.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
            : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]), "=f"(f[4]), "=f"(f[5]), "=f"(f[6]), "=f"(f[7])
            : "l"(xr));
        asm("ld.global.cg.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
            : "=f"(f[8]), "=f"(f[9]), "=f"(f[10]), "=f"(f[11]), "=f"(f[12]), "=f"(f[13]), "=f"(f[14]), "=f"(f[15])
            : "l"(xr + 4));
#pragma unroll
        for (int q = 0; q < K; ++q) xv[q] = make_float2(f[2 * q], f[2 * q + 1]);
      } else {
#pragma unroll
        for (int q = 0; q < K; ++q) xv[q] = __ldg(xr + q);
      }
#pragma unroll
      for (int q = 0; q < K; ++q) ff_fma(sh[q], sl[q], v, xv[q]);
    }
    ff2 vv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (q < K) {
        float h = sh[q], l = sl[q];
        ff_renorm(h, l);
        vv[q] = ff2{h, l};
      } else {
        vv[q] = ff2{0.f, 0.f};
      }
    }
    store_reduced_ff<K>(vv, lane, y + r * ldy);
  }
}

// X (FP64, leading dim ldx) -> X2 (float pairs, leading dim k); one thread per row
__global__ void k_split_x(int64_t n, int k, const double *__restrict__ x, int ldx, float2 *__restrict__ x2) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    for (int q = 0; q < k; ++q) x2[r * k + q] = split_f64(x[r * ldx + q]);
  }
}

// X (FP64, leading dim ldx, k <= 8 columns) -> X32 (FP32, row stride 4 when k <= 4, else 8,
// zero padded); one thread per row
__global__ void k_to_f32(int64_t n, int k, const double *__restrict__ x, int ldx, float *__restrict__ x32) {
  const int xs = (k <= 4) ? 4 : 8;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const double *src = x + r * ldx;
    float4 *dst = reinterpret_cast<float4 *>(x32 + r * xs);
    float f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) f[q] = (q < k) ? (float)src[q] : 0.f;
    dst[0] = make_float4(f[0], f[1], f[2], f[3]);
    if (xs == 8) dst[1] = make_float4(f[4], f[5], f[6], f[7]);
  }
}

template <int K>
void launch_k(psoci_ctx *c, int64_t n, const double *dX, int ldx, double *dY, int ldy, psoci_prec prec,
              const float *x32, int ld32) {
  int64_t warps = n;
  int blocks = (int)std::min<int64_t>((warps * 32 + SIG_THREADS - 1) / SIG_THREADS, 152 * 8 * 4);
  if (blocks < 1) blocks = 1;
  psoci_note_launch();
  if (prec == PSOCI_PREC_FP64)
    k_spmm_f64<K><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val, dX, ldx, dY, ldy,
                                                         ((uintptr_t)dX % 16 == 0) && (ldx % 2 == 0));
  else if (prec == PSOCI_PREC_FF)
    k_spmm_ff<K><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val,
                                                        reinterpret_cast<const float2 *>(x32), dY, ldy);
  else {
    // the variant chosen by psoci_autotune_sigma for this Hamiltonian (PSOCI_SIGMA_DEFAULT
    // until it runs)
    switch (c->sigma_variant) {
      case 1:
        k_spmm_mixed<K, 32, 2><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32, dY, ldy);
        break;
      case 2:
        k_spmm_mixed<K, 16, 4><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32, dY, ldy);
        break;
      case 3:
        k_spmm_mixed<K, 16, 2><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32, dY, ldy);
        break;
      case 4:
        k_spmm_mixed<K, 8, 4><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32, dY, ldy);
        break;
      case 5:
        k_spmm_mixed<K, 16, 6><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32, dY, ldy);
        break;
      default:
        k_spmm_mixed<K, 32, SIG_UNROLL><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32,
                                                                              dY, ldy);
    }
  }
}

}  // namespace

// dX32: staging of at least N*8 floats (MIXED) or N*16 floats (FF); may be null for FP64.
psoci_status psoci_sigma_launch(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy,
                                psoci_prec prec, float *dX32) {
  if (prec != PSOCI_PREC_FP64 && prec != PSOCI_PREC_MIXED && prec != PSOCI_PREC_FF)
    return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "sigma: unknown precision");
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "sigma: Hamiltonian not built");
  if (k < 1 || ldx < k || ldy < k) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "sigma: bad k / leading dimensions");
  if (c->direct) return psoci_direct_sigma(c, k, dX, ldx, dY, ldy, prec, dX32);
  if (prec == PSOCI_PREC_MIXED && !c->d_val32)
    return psoci_fail(c, PSOCI_ERR_STATE, "sigma: MIXED needs the FP32 copy (PSOCI_HMODE_CSR_BOTH)");
  const int64_t n = c->nsef_total;
  // process the block in chunks of at most 8 vectors
  for (int q0 = 0; q0 < k; q0 += 8) {
    int kk = std::min(8, k - q0);
    const double *xs = dX + q0;
    double *ys = dY + q0;
    const float *x32 = nullptr;
    if (prec == PSOCI_PREC_MIXED) {
      if (!dX32) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "sigma: MIXED without FP32 staging");
      int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
      psoci_note_launch();
      k_to_f32<<<std::max(blocks, 1), 256, 0, c->stream>>>(n, kk, xs, ldx, dX32);
      x32 = dX32;
    } else if (prec == PSOCI_PREC_FF) {
      if (!dX32) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "sigma: FF without staging");
      int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
      psoci_note_launch();
      k_split_x<<<std::max(blocks, 1), 256, 0, c->stream>>>(n, kk, xs, ldx, reinterpret_cast<float2 *>(dX32));
      x32 = dX32;
    }
    switch (kk) {
      case 1: launch_k<1>(c, n, xs, ldx, ys, ldy, prec, x32, 1); break;
      case 2: launch_k<2>(c, n, xs, ldx, ys, ldy, prec, x32, 2); break;
      case 3: launch_k<3>(c, n, xs, ldx, ys, ldy, prec, x32, 3); break;
      case 4: launch_k<4>(c, n, xs, ldx, ys, ldy, prec, x32, 4); break;
      case 5: launch_k<5>(c, n, xs, ldx, ys, ldy, prec, x32, 5); break;
      case 6: launch_k<6>(c, n, xs, ldx, ys, ldy, prec, x32, 6); break;
      case 7: launch_k<7>(c, n, xs, ldx, ys, ldy, prec, x32, 7); break;
      default: launch_k<8>(c, n, xs, ldx, ys, ldy, prec, x32, 8); break;
    }
    PSOCI_CUDA(c, cudaGetLastError());
  }
  return PSOCI_OK;
}

// Autotuner of the mixed sigma: each variant (lanes per row x gathers in flight) timed with
// CUDA events on the context's stream over k random vectors, best of three after one warm-up
// run; the fastest is kept for this Hamiltonian (reset by the next build).  times_ms may be
// null or receive PSOCI_SIGMA_VARIANTS entries.
psoci_status psoci_sigma_autotune_run(psoci_ctx *c, int k, int *choice, float *times_ms) {
  if (!c->have_h || c->direct || !c->d_val32)
    return psoci_fail(c, PSOCI_ERR_STATE, "autotune_sigma: needs a stored Hamiltonian with the FP32 copy");
  if (k == 0) {
    // no timing: install the variant given in *choice
    if (!choice || *choice < 0 || *choice >= PSOCI_SIGMA_VARIANTS)
      return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "autotune_sigma: variant outside 0..5");
    c->sigma_variant = *choice;
    c->sigma_tuned = true;
    return PSOCI_OK;
  }
  if (k < 1 || k > 8) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "autotune_sigma: k must be 0..8");
  const int64_t n = c->nsef_total;
  double *dX = nullptr, *dY = nullptr;
  float *x32 = nullptr;
  psoci_status s;
  if ((s = psoci_alloc(c, &dX, (size_t)n * k)) || (s = psoci_alloc(c, &dY, (size_t)n * k)) ||
      (s = psoci_alloc(c, &x32, (size_t)n * 8))) {
    psoci_free(dX); psoci_free(dY); psoci_free(x32);
    return s;
  }
  cudaStream_t st = c->stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // inputs: any finite values (the timing does not depend on them)
  cudaMemsetAsync(dX, 0, sizeof(double) * n * k, st);
  const int saved = c->sigma_variant;
  int best = 0;
  float best_ms = 1e30f;
  for (int v = 0; v < PSOCI_SIGMA_VARIANTS; ++v) {
    c->sigma_variant = v;
    float tmin = 1e30f;
    for (int rep = 0; rep < 4 && s == PSOCI_OK; ++rep) {
      cudaEventRecord(e0, st);
      s = psoci_sigma_launch(c, k, dX, k, dY, k, PSOCI_PREC_MIXED, x32);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tmin = std::min(tmin, ms);
    }
    if (times_ms) times_ms[v] = tmin;
    if (tmin < best_ms) { best_ms = tmin; best = v; }
  }
  cudaError_t e = cudaStreamSynchronize(st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  psoci_free(dX); psoci_free(dY); psoci_free(x32);
  if (s != PSOCI_OK) { c->sigma_variant = saved; return s; }
  if (e != cudaSuccess) { c->sigma_variant = saved; return psoci_cuda_fail(c, e, "autotune_sigma"); }
  c->sigma_variant = best;
  c->sigma_tuned = true;
  if (choice) *choice = best;
  return PSOCI_OK;
}
