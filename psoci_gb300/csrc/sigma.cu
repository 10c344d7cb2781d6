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
//   MIXED: FP32 elements and FP32 inputs, FP32 products, FP64 accumulation.
#include <algorithm>

#include "psoci_internal.cuh"

namespace {

constexpr int SIG_THREADS = 256;

template <typename T>
__device__ __forceinline__ T ldg_stream(const T *p) { return __ldcs(p); }

// transpose-reduce: after this, lane q (< K) holds the warp sum of acc[q]
template <int K>
__device__ __forceinline__ double warp_reduce_vec(double (&acc)[K], int lane) {
#pragma unroll
  for (int q = 0; q < K; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
  }
  double mine = 0.0;
#pragma unroll
  for (int q = 0; q < K; ++q)
    if (lane == q) mine = acc[q];
  return mine;
}

template <int K>
__global__ void __launch_bounds__(SIG_THREADS) k_spmm_f64(int64_t nrows, const int64_t *__restrict__ rowptr,
                                                          const int32_t *__restrict__ col,
                                                          const double *__restrict__ val,
                                                          const double *__restrict__ x, int ldx,
                                                          double *__restrict__ y, int ldy) {
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
#pragma unroll
      for (int q = 0; q < K; ++q) acc[q] = fma(v, __ldg(xr + q), acc[q]);
    }
    double s = warp_reduce_vec<K>(acc, lane);
    if (lane < K) y[r * ldy + lane] = s;
  }
}

template <int K>
__global__ void __launch_bounds__(SIG_THREADS) k_spmm_mixed(int64_t nrows, const int64_t *__restrict__ rowptr,
                                                            const int32_t *__restrict__ col,
                                                            const float *__restrict__ val,
                                                            const float *__restrict__ x, int ldx,
                                                            double *__restrict__ y, int ldy) {
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
      const float v = ldg_stream(val + t);
      const float *xr = x + (int64_t)c * ldx;
#pragma unroll
      for (int q = 0; q < K; ++q) acc[q] += (double)__fmul_rn(v, __ldg(xr + q));
    }
    double s = warp_reduce_vec<K>(acc, lane);
    if (lane < K) y[r * ldy + lane] = s;
  }
}

// X (FP64, leading dim ldx) -> X32 (FP32, leading dim k)
__global__ void k_to_f32(int64_t n, int k, const double *__restrict__ x, int ldx, float *__restrict__ x32) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t tot = n * k;
  for (; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / k;
    int q = (int)(i - r * k);
    x32[i] = (float)x[r * ldx + q];
  }
}

template <int K>
void launch_k(psoci_ctx *c, int64_t n, const double *dX, int ldx, double *dY, int ldy, psoci_prec prec,
              const float *x32, int ld32) {
  int64_t warps = n;
  int blocks = (int)std::min<int64_t>((warps * 32 + SIG_THREADS - 1) / SIG_THREADS, 152 * 8 * 4);
  if (blocks < 1) blocks = 1;
  if (prec == PSOCI_PREC_FP64)
    k_spmm_f64<K><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val, dX, ldx, dY, ldy);
  else
    k_spmm_mixed<K><<<blocks, SIG_THREADS, 0, c->stream>>>(n, c->d_rowptr, c->d_col, c->d_val32, x32, ld32, dY, ldy);
}

}  // namespace

// dX32: FP32 staging of at least N*k floats (MIXED only); may be null for FP64.
psoci_status psoci_sigma_launch(psoci_ctx *c, int k, const double *dX, int ldx, double *dY, int ldy,
                                psoci_prec prec, float *dX32) {
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "sigma: Hamiltonian not built");
  if (k < 1 || ldx < k || ldy < k) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "sigma: bad k / leading dimensions");
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
      int blocks = (int)std::min<int64_t>((n * kk + 255) / 256, 152 * 16);
      k_to_f32<<<std::max(blocks, 1), 256, 0, c->stream>>>(n, kk, xs, ldx, dX32);
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
