// Spin-free 1-particle density of CI vectors: the reference's CI-density (CIDEN) path,
// constructCIdensityAltOrbMapChunkJmap (PsociGAhamiltonian.C:11570-11760) with the
// element blocks of generateSOCIblocksForCIDEN (PsociHamiltonian.C:572-705) contracted
// as transformSEFSEFtoMOGET does (PsociGAhamiltonian.C:10027-10099).
//
// Output per root: the packed lower triangle D[tri(p, q)], tri(p, q) = p(p+1)/2 + q for
// p >= q (twoDindex, PsociGAhamiltonian.C:10297-10302).
//   diagonal    D[tri(p, p)] = sum_I occ_p(I) * c_I^T (C_I C_I^T) c_I
//   off-diag    D[tri(p, q)] = sum over unordered configuration pairs {I, J} that differ
//               by one electron moved between p and q (same jsym) of c_I^T S_IJ c_J,
//               S_IJ = C_I d C_J^T, d the +-1/0 determinant block.
//
// Pair discovery ("hole keys").  I and J differ by one electron moved (I = K + e_p,
// J = K + e_q, p != q) exactly when removing one electron from I and one from J leaves
// the same occupation K; K and the pair's orbitals are then unique.  Every configuration
// contributes one key per occupied orbital, (K, jsym) hashed into an open-addressing
// table; configurations sharing a slot form a group and every pair inside a group is a
// candidate, verified exactly (same K, same jsym) before use, so hash collisions cost
// time, never correctness.  The groups depend only on the configuration list and are
// kept in the context for later calls.
//
// Pair elements.  With x_I = C_I^T c_I the determinant coefficients of I, c_I^T S c_J =
// sum over determinant pairs (i, j) that differ by one spin-orbital moved p <-> q of
// s_ij x_I[i] x_J[j]; s_ij = (-1)^(ph_i + ph_j + n), n the electrons of the moved spin in
// determinant i strictly between p and q (generateSEFCIGCIDEN, PsociHamiltonian.C:
// 1123-1269).  Determinant j of J is found by its moved-spin string alone: within one
// configuration the alpha string fixes the beta string and the reverse.
//
// Sums run in an order set by the hardware (shared and global atomics); results agree
// with the reference's sequential sums to rounding.
#include <cstdio>

#include "ffmath.cuh"
#include "psoci_internal.cuh"

namespace {

constexpr int DEN_T = 256;
constexpr int DEN_CHUNK = 4;  // consecutive pairs per thread per step

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 31;
  x *= 0x7fb5d329728ea185ull;
  x ^= x >> 27;
  x *= 0x81dadef4bc2dd44dull;
  x ^= x >> 33;
  return x;
}

template <int W>
__device__ __forceinline__ uint64_t hole_hash(const uint64_t (&e1)[W], const uint64_t (&e2)[W], int jsym) {
  uint64_t h = mix64(0x243f6a8885a308d3ull + (uint64_t)(uint32_t)jsym);
#pragma unroll
  for (int w = 0; w < W; ++w) {
    h = mix64(h ^ e1[w]);
    h = mix64(h + e2[w] * 0x9e3779b97f4a7c15ull);
  }
  return h ? h : 1ull;  // 0 marks an empty slot
}

// occupation with one electron removed from orbital p (occupied)
template <int W>
__device__ __forceinline__ void remove_one(const uint64_t *e1g, const uint64_t *e2g, int p, uint64_t (&e1)[W],
                                           uint64_t (&e2)[W]) {
#pragma unroll
  for (int w = 0; w < W; ++w) { e1[w] = e1g[w]; e2[w] = e2g[w]; }
  const uint64_t b = 1ull << (p & 63);
  const int w = p >> 6;
#pragma unroll
  for (int v = 0; v < W; ++v) {
    if (v != w) continue;
    if (e2[v] & b) e2[v] &= ~b;  // doubly -> singly
    else e1[v] &= ~b;            // singly -> empty
  }
}

__global__ void k_hole_count(int nconf, int W, const uint64_t *__restrict__ e1, int64_t *cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nconf; i += (int64_t)gridDim.x * blockDim.x) {
    int n = 0;
    for (int w = 0; w < W; ++w) n += __popcll(e1[i * W + w]);
    cnt[i] = n;
  }
}

// one key per (configuration, occupied orbital); slot and rank inside the slot's group
template <int W>
__global__ void k_hole_insert(int nconf, const uint64_t *__restrict__ e1g, const uint64_t *__restrict__ e2g,
                              const int32_t *__restrict__ jsym, const int64_t *__restrict__ hoff,
                              unsigned long long *keys, uint64_t mask, int32_t *gcnt, int32_t *ent_slot,
                              int32_t *ent_rank, int *err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nconf; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t e = hoff[i];
    const int js = jsym[i];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t m = e1g[i * W + w];
      while (m) {
        const int p = w * 64 + __ffsll((long long)m) - 1;
        m &= m - 1;
        uint64_t k1[W], k2[W];
        remove_one<W>(e1g + i * W, e2g + i * W, p, k1, k2);
        const unsigned long long h = hole_hash<W>(k1, k2, js);
        uint64_t s = h & mask;
        bool placed = false;
        for (uint64_t probe = 0; probe <= mask; ++probe) {  // bounded: the table has free slots
          const unsigned long long old = atomicCAS(keys + s, 0ull, h);
          if (old == 0ull || old == h) { placed = true; break; }
          s = (s + 1) & mask;
        }
        if (!placed) {
          atomicExch(err, 1);
          ent_slot[e] = -1;
          ent_rank[e] = 0;
        } else {
          ent_slot[e] = (int32_t)s;
          ent_rank[e] = atomicAdd(gcnt + s, 1);
        }
        ++e;
      }
    }
  }
}

__global__ void k_group_flags(int64_t T, const int32_t *__restrict__ gcnt, int64_t *flag) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < T; s += (int64_t)gridDim.x * blockDim.x)
    flag[s] = gcnt[s] >= 2;
}

__global__ void k_group_compact(int64_t T, const int32_t *__restrict__ gcnt, const int64_t *__restrict__ gidx,
                                int32_t *slot2g, int64_t *gm_e, int64_t *gm_p) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < T; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = gcnt[s];
    if (m >= 2) {
      const int64_t g = gidx[s];
      slot2g[s] = (int32_t)g;
      gm_e[g] = m;
      gm_p[g] = m * (m - 1) / 2;
    } else {
      slot2g[s] = -1;
    }
  }
}

// group members in slot order: (configuration, orbital the key removed) and, where the
// determinant and SEF totals fit 31 bits, a packed copy with the configuration's offsets,
// {cfg, first determinant, first SEF, orbital | nopen << 8 | ndet << 16 | phase << 30},
// and its open shells
__global__ void k_hole_scatter(int nconf, int W, const uint64_t *__restrict__ e1g, const uint64_t *__restrict__ e2g,
                               const int64_t *__restrict__ hoff, const int32_t *__restrict__ ent_slot,
                               const int32_t *__restrict__ ent_rank, const int32_t *__restrict__ slot2g,
                               const int64_t *__restrict__ geoff, int32_t *gcfg, uint8_t *gorb,
                               const int64_t *__restrict__ detoff, const int64_t *__restrict__ sefoff,
                               const int32_t *__restrict__ nopen, const uint8_t *__restrict__ phase, int4 *gmem,
                               uint64_t *gopen) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nconf; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t e = hoff[i];
    for (int w = 0; w < W; ++w) {
      uint64_t m = e1g[i * W + w];
      while (m) {
        const int p = w * 64 + __ffsll((long long)m) - 1;
        m &= m - 1;
        const int32_t s = ent_slot[e];
        const int32_t g = s >= 0 ? slot2g[s] : -1;
        if (g >= 0) {
          const int64_t pos = geoff[g] + ent_rank[e];
          gcfg[pos] = (int32_t)i;
          gorb[pos] = (uint8_t)p;
          if (gmem) {
            gmem[pos] = make_int4((int)i, (int)detoff[i], (int)sefoff[i],
                                  p | (nopen[i] << 8) | (int)((detoff[i + 1] - detoff[i]) << 16) |
                                      ((int)(phase[detoff[i]] & 1) << 30));
            for (int v = 0; v < W; ++v) gopen[pos * W + v] = e1g[i * W + v] & ~e2g[i * W + v];
          }
        }
        ++e;
      }
    }
  }
}

// 1 for a group whose members do not all share one exact key (a 64-bit hash collision):
// its pairs are checked one by one
template <int W>
__global__ void k_group_verify(int64_t ng, const int64_t *__restrict__ geoff, const int32_t *__restrict__ gcfg,
                               const uint8_t *__restrict__ gorb, const uint64_t *__restrict__ e1g,
                               const uint64_t *__restrict__ e2g, const int32_t *__restrict__ jsym, uint8_t *gflag) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e0 = geoff[g], e1 = geoff[g + 1];
    const int c0 = gcfg[e0];
    uint64_t k1[W], k2[W];
    remove_one<W>(e1g + (int64_t)c0 * W, e2g + (int64_t)c0 * W, gorb[e0], k1, k2);
    bool mixed = false;
    for (int64_t e = e0 + 1; e < e1; ++e) {
      const int ci = gcfg[e];
      uint64_t a1[W], a2[W];
      remove_one<W>(e1g + (int64_t)ci * W, e2g + (int64_t)ci * W, gorb[e], a1, a2);
#pragma unroll
      for (int w = 0; w < W; ++w) mixed = mixed || a1[w] != k1[w] || a2[w] != k2[w];
      mixed = mixed || jsym[ci] != jsym[c0] || ci == c0;
    }
    gflag[g] = mixed;
  }
}

struct DenParams {
  int nconf, nbf, nelec, ksym, kb, ntri;
  int64_t N;      // SEFs per vector
  int64_t ldv;    // vector stride (root-major)
  const double *v;  // first root of this batch
  const uint64_t *e1, *e2;
  const int32_t *jsym, *nopen;
  const int64_t *sefoff, *detoff;
  const uint64_t *alpha, *beta;
  const uint8_t *phase;
  int64_t ng, npairs;
  const int64_t *geoff, *gpoff;
  const int32_t *gcfg;
  const uint8_t *gorb;
  const int4 *gmem;        // packed members (warp path)
  const uint64_t *gopen;   // members: open shells of the configuration [W]
  const uint8_t *gflag;    // per group: members' keys differ, check each pair
  const float2 *vs;        // float-float roots of this pass, KBW per SEF (warp path)
  const uint32_t *tmpl;    // determinant templates (amask | bmask << 12)
  const int32_t *tmpl_off; // start of each (class, nopen) run
  double *dens;  // [kb][ntri] of this batch
};

// determinant coefficient x_I[d] of root r (ciout: SEF s = r2 (det 2s + m det 2s+1))
__device__ __forceinline__ double det_coef(const DenParams &P, int64_t sef0, int nopen, int msign, int d, int r) {
  const double *v = P.v + (int64_t)r * P.ldv + sef0;
  if (P.nelec & 1) return v[d];
  if (nopen == 0) return v[0];
  const double c = sqrt(0.5) * v[d >> 1];
  return (d & 1) ? msign * c : c;
}

template <int W>
__device__ __forceinline__ bool tb(const uint64_t *x, int p) {
  return (x[p >> 6] >> (p & 63)) & 1ull;
}

// electrons of string x strictly between orbitals lo < hi
template <int W>
__device__ __forceinline__ int popc_between(const uint64_t *x, int lo, int hi) {
  int n = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const int b0 = w * 64;
    const int a = max(lo + 1 - b0, 0), b = min(hi - b0, 64);  // bits [a, b)
    if (a >= b) continue;
    uint64_t m = (b == 64 ? ~0ull : ((1ull << b) - 1)) & ~((1ull << a) - 1);
    n += __popcll(x[w] & m);
  }
  return n;
}

constexpr int KB_MAX = 8;

// c_I^T S_IJ c_J for the roots of this batch, added into the block's accumulator
template <int W>
__device__ void pair_contrib(const DenParams &P, int I, int p, int J, int q, double *acc) {
  // exact check: same hole occupation and same jsym
  if (P.jsym[I] != P.jsym[J]) return;
  {
    uint64_t a1[W], a2[W], b1[W], b2[W];
    remove_one<W>(P.e1 + (int64_t)I * W, P.e2 + (int64_t)I * W, p, a1, a2);
    remove_one<W>(P.e1 + (int64_t)J * W, P.e2 + (int64_t)J * W, q, b1, b2);
    bool same = true;
#pragma unroll
    for (int w = 0; w < W; ++w) same = same && a1[w] == b1[w] && a2[w] == b2[w];
    if (!same || p == q) return;
  }
  const int64_t dI = P.detoff[I], nI = P.detoff[I + 1] - dI;
  const int64_t dJ = P.detoff[J], nJ = P.detoff[J + 1] - dJ;
  const int64_t sI = P.sefoff[I], sJ = P.sefoff[J];
  const int oI = P.nopen[I], oJ = P.nopen[J];
  const int mI = (P.jsym[I] % 2 != P.ksym % 2) ? -1 : 1;  // same jsym: same sign for J
  const int lo = min(p, q), hi = max(p, q);
  double val[KB_MAX];
#pragma unroll
  for (int r = 0; r < KB_MAX; ++r) val[r] = 0.0;
  for (int ii = 0; ii < nI; ++ii) {
    const uint64_t *al = P.alpha + (dI + ii) * W, *be = P.beta + (dI + ii) * W;
    const int phi = P.phase[dI + ii];
#pragma unroll 1
    for (int spin = 0; spin < 2; ++spin) {
      const uint64_t *s = spin ? be : al;
      if (!tb<W>(s, p) || tb<W>(s, q)) continue;
      uint64_t t[W];
#pragma unroll
      for (int w = 0; w < W; ++w) {
        t[w] = s[w];
        if (w == (p >> 6)) t[w] ^= 1ull << (p & 63);
        if (w == (q >> 6)) t[w] ^= 1ull << (q & 63);
      }
      const uint64_t *js = (spin ? P.beta : P.alpha) + dJ * W;
      int jj = -1;
      for (int d = 0; d < nJ; ++d) {
        bool eq = true;
#pragma unroll
        for (int w = 0; w < W; ++w) eq = eq && js[(int64_t)d * W + w] == t[w];
        if (eq) { jj = d; break; }
      }
      if (jj < 0) continue;
      const int n = phi + P.phase[dJ + jj] + popc_between<W>(s, lo, hi);
      const double sg = (n & 1) ? -1.0 : 1.0;
#pragma unroll
      for (int r = 0; r < KB_MAX; ++r) {
        if (r >= P.kb) break;
        val[r] += sg * det_coef(P, sI, oI, mI, ii, r) * det_coef(P, sJ, oJ, mI, jj, r);
      }
    }
  }
  const int idx = hi * (hi + 1) / 2 + lo;
#pragma unroll
  for (int r = 0; r < KB_MAX; ++r) {
    if (r >= P.kb) break;
    if (val[r] != 0.0) atomicAdd(acc + (int64_t)r * P.ntri + idx, val[r]);
  }
}

template <int W>
__global__ void __launch_bounds__(DEN_T) k_density_pairs(DenParams P) {
  extern __shared__ double acc[];  // [kb][ntri]
  for (int t = threadIdx.x; t < P.kb * P.ntri; t += blockDim.x) acc[t] = 0.0;
  __syncthreads();
  const int64_t nchunk = (P.npairs + DEN_CHUNK - 1) / DEN_CHUNK;
  for (int64_t ch = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ch < nchunk; ch += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t0 = ch * DEN_CHUNK;
    // group holding pair t0: last g with gpoff[g] <= t0
    int64_t lo = 0, hi = P.ng - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (P.gpoff[mid] <= t0) lo = mid;
      else hi = mid - 1;
    }
    int64_t g = lo;
    int64_t e0 = P.geoff[g];
    int m = (int)(P.geoff[g + 1] - e0);
    int64_t u = t0 - P.gpoff[g];
    int a = 0;
    while (u >= m - 1 - a) { u -= m - 1 - a; ++a; }
    int b = a + 1 + (int)u;
    const int64_t tend = min(t0 + DEN_CHUNK, P.npairs);
    for (int64_t t = t0; t < tend; ++t) {
      pair_contrib<W>(P, P.gcfg[e0 + a], P.gorb[e0 + a], P.gcfg[e0 + b], P.gorb[e0 + b], acc);
      if (++b == m) {
        if (++a == m - 1) {
          if (++g >= P.ng) break;
          e0 = P.geoff[g];
          m = (int)(P.geoff[g + 1] - e0);
          a = 0;
        }
        b = a + 1;
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < P.kb * P.ntri; t += blockDim.x)
    if (acc[t] != 0.0) atomicAdd(P.dens + t, acc[t]);
}

constexpr int KBW = 4;        // roots per pass of the warp-per-pair kernel
constexpr int INV_NOPEN = 7;  // warp path: at most 6 open shells (32 determinants)

// float-float sum a + b (TwoSum on the high parts, low parts added)
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  return make_float2(s, __fadd_rn(__fadd_rn(a.y, b.y), e));
}
__device__ __forceinline__ float2 shfl_xor_ff(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// Float-float sum of v[0..3] over the warp, scattered: afterwards lane l with (l & 7) == 0
// holds the total of root (l >> 3) & 3.  Two halving exchanges (2 + 1 values) then three
// butterfly steps.
__device__ __forceinline__ float2 reduce_scatter4(const float2 (&v)[4], int lane) {
  float2 w[2];
  const bool b4 = lane & 16, b3 = lane & 8;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float2 send = b4 ? v[i] : v[i + 2];
    const float2 keep = b4 ? v[i + 2] : v[i];
    w[i] = ff_add(keep, shfl_xor_ff(send, 16));
  }
  float2 z = ff_add(b3 ? w[1] : w[0], shfl_xor_ff(b3 ? w[0] : w[1], 8));
  z = ff_add(z, shfl_xor_ff(z, 4));
  z = ff_add(z, shfl_xor_ff(z, 2));
  z = ff_add(z, shfl_xor_ff(z, 1));
  return z;
}

// Inverse template table in shared memory: (class, nopen <= 6, alpha pattern over the open
// shells in ascending order) -> index of that determinant in the configuration, or -1.
// Within one template run the alpha pattern fixes the determinant (beta holds the other
// open shells).
__device__ __forceinline__ void build_inverse(const uint32_t *__restrict__ tmpl, const int32_t *__restrict__ tmpl_off,
                                              int8_t *inv) {
  for (int t = threadIdx.x; t < PSOCI_NCLS * INV_NOPEN * 64; t += blockDim.x) inv[t] = -1;
  __syncthreads();
  for (int t = threadIdx.x; t < PSOCI_NCLS * INV_NOPEN * 32; t += blockDim.x) {
    const int cls = t / (INV_NOPEN * 32), no = (t / 32) % INV_NOPEN, d = t % 32;
    const int r0 = tmpl_off[cls * PSOCI_NOPEN_SLOTS + no], r1 = tmpl_off[cls * PSOCI_NOPEN_SLOTS + no + 1];
    if (d < r1 - r0) inv[(cls * INV_NOPEN + no) * 64 + (tmpl[r0 + d] & 63u)] = (int8_t)d;
  }
  __syncthreads();
}

// SEF of determinant d (ciout: odd electron counts one SEF per determinant; even, open
// shells: SEF s = r2 (det 2s + m det 2s+1); closed shell: one of each)
__device__ __forceinline__ int sef_of_det(int d, bool odd, int nopen) { return odd ? d : (nopen ? d >> 1 : 0); }

// exact check of a pair from a group whose members' keys differ
template <int W>
__device__ __forceinline__ bool pair_exact(const DenParams &P, int I, int p, int J, int q) {
  if (P.jsym[I] != P.jsym[J] || I == J) return false;
  uint64_t a1[W], a2[W], b1[W], b2[W];
  remove_one<W>(P.e1 + (int64_t)I * W, P.e2 + (int64_t)I * W, p, a1, a2);
  remove_one<W>(P.e1 + (int64_t)J * W, P.e2 + (int64_t)J * W, q, b1, b2);
  bool same = true;
#pragma unroll
  for (int w = 0; w < W; ++w) same = same && a1[w] == b1[w] && a2[w] == b2[w];
  return same;
}

// One block per SM holding the [kb][ntri] accumulator once for 24 warps.
constexpr int DEN_WT = 768;

// Warp per configuration pair (both sides <= 32 determinants).  Lane d holds determinant d
// of I; its partner in J under the move p <-> q is looked up in the inverse template table
// from the moved string's alpha pattern over J's open shells.  Products and lane sums are
// float-float on the FP32 pipe (GB300's FP64 pipe is ~64x narrower); each pair's total is
// converted to FP64 once, scaled by the SEF normalisation and added to the accumulator.
template <int W>
__global__ void __launch_bounds__(DEN_WT, 1) k_density_pairs_warp(DenParams P) {
  extern __shared__ double acc[];  // [kb][ntri], then the inverse table
  int8_t *inv = reinterpret_cast<int8_t *>(acc + (size_t)P.kb * P.ntri);
  for (int t = threadIdx.x; t < P.kb * P.ntri; t += blockDim.x) acc[t] = 0.0;
  build_inverse(P.tmpl, P.tmpl_off, inv);
  const int lane = threadIdx.x & 31;
  const bool odd = P.nelec & 1;
  const double r2 = sqrt(0.5);
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t wid = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  // each warp walks one contiguous range of the pair list: one search for its start
  const int64_t t0 = P.npairs * wid / nwarps, tend = P.npairs * (wid + 1) / nwarps;
  if (t0 < tend) {
    int64_t lo = 0, hi = P.ng - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (P.gpoff[mid] <= t0) lo = mid;
      else hi = mid - 1;
    }
    int64_t g = lo;
    int64_t e0 = P.geoff[g];
    int m = (int)(P.geoff[g + 1] - e0);
    bool mixed = P.gflag[g];
    int64_t u = t0 - P.gpoff[g];
    int a = 0;
    while (u >= m - 1 - a) { u -= m - 1 - a; ++a; }
    int b = a + 1 + (int)u;
    int64_t cachedA = -1;
    // row configuration I, cached over the pairs of one group member
    int4 mA = make_int4(0, 0, 0, 0);
    int clsI = 0, negI = 0, oI = 0;
    uint64_t al[W], be[W];
    float2 cI[KBW];
    for (int64_t t = t0; t < tend; ++t) {
      const int64_t ea = e0 + a, eb = e0 + b;
      if (ea != cachedA) {
        mA = P.gmem[ea];
        const int js = P.jsym[mA.x];
        clsI = psoci_det_class(P.nelec & 1, js, P.ksym);
        negI = (js % 2 != P.ksym % 2);  // m = -1: the second determinant of an SEF enters negated
        oI = (mA.w >> 8) & 0xff;
        const int nI = (mA.w >> 16) & 0x3fff;
        const bool has = lane < nI;
        const int64_t d = (int64_t)mA.y + lane;
#pragma unroll
        for (int w = 0; w < W; ++w) {
          al[w] = has ? P.alpha[d * W + w] : 0ull;
          be[w] = has ? P.beta[d * W + w] : 0ull;
        }
        const float4 *src = reinterpret_cast<const float4 *>(P.vs + ((int64_t)mA.z + sef_of_det(lane, odd, oI)) * KBW);
        const float4 c01 = has ? src[0] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 c23 = has ? src[1] : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool flip = has && !odd && oI && (lane & 1) && negI;
        const float sg = flip ? -1.f : 1.f;
        cI[0] = make_float2(sg * c01.x, sg * c01.y);
        cI[1] = make_float2(sg * c01.z, sg * c01.w);
        cI[2] = make_float2(sg * c23.x, sg * c23.y);
        cI[3] = make_float2(sg * c23.z, sg * c23.w);
        cachedA = ea;
      }
      const int4 mB = P.gmem[eb];
      const int p = mA.w & 0xff, q = mB.w & 0xff;
      if (!mixed || pair_exact<W>(P, mA.x, p, mB.x, q)) {
        const int oJ = (mB.w >> 8) & 0xff;
        const int phs = ((mA.w >> 30) ^ (mB.w >> 30)) & 1;  // configuration phases
        uint64_t openJ[W];
#pragma unroll
        for (int w = 0; w < W; ++w) openJ[w] = P.gopen[eb * W + w];
        const int8_t *invJ = inv + (clsI * INV_NOPEN + oJ) * 64;
        const int plo = min(p, q), phi = max(p, q);
        const int wp = p >> 6, wq = q >> 6;
        const uint64_t bp = 1ull << (p & 63), bq = 1ull << (q & 63);
        float2 s[KBW];
#pragma unroll
        for (int r = 0; r < KBW; ++r) s[r] = make_float2(0.f, 0.f);
#pragma unroll
        for (int spin = 0; spin < 2; ++spin) {
          bool ok = true;
          uint64_t ta[W];  // alpha string of the target determinant
          int nb = 0;
#pragma unroll
          for (int w = 0; w < W; ++w) {
            const uint64_t x = spin ? be[w] : al[w];
            if (w == wp) ok = ok && (x & bp);
            if (w == wq) ok = ok && !(x & bq);
            const int b0 = w * 64;
            const int lo1 = max(plo + 1 - b0, 0), hi1 = min(phi - b0, 64);
            if (lo1 < hi1) nb += __popcll(x & ((hi1 == 64 ? ~0ull : ((1ull << hi1) - 1)) & ~((1ull << lo1) - 1)));
            uint64_t tw = al[w];
            if (!spin) {
              if (w == wp) tw ^= bp;
              if (w == wq) tw ^= bq;
            }
            ta[w] = tw;
          }
          // alpha pattern of the target over J's open shells (ascending)
          int pat = 0, k = 0;
#pragma unroll
          for (int w = 0; w < W; ++w) {
            uint64_t om = openJ[w];
            while (om) {
              const uint64_t lowbit = om & (~om + 1);
              if (ta[w] & lowbit) pat |= 1 << k;
              ++k;
              om ^= lowbit;
            }
          }
          const int jj = ok ? invJ[pat & 63] : -1;
          if (jj >= 0) {
            const float4 *src = reinterpret_cast<const float4 *>(P.vs + ((int64_t)mB.z + sef_of_det(jj, odd, oJ)) * KBW);
            const float4 c01 = src[0], c23 = src[1];
            const bool flipJ = !odd && oJ && (jj & 1) && negI;
            const float sg = ((phs + nb + (int)flipJ) & 1) ? -1.f : 1.f;
            const float2 cj[4] = {make_float2(sg * c01.x, sg * c01.y), make_float2(sg * c01.z, sg * c01.w),
                                  make_float2(sg * c23.x, sg * c23.y), make_float2(sg * c23.z, sg * c23.w)};
#pragma unroll
            for (int r = 0; r < KBW; ++r) ff_fma(s[r].x, s[r].y, cI[r], cj[r]);
          }
        }
        const float2 z = reduce_scatter4(s, lane);
        const int r = (lane >> 3) & 3;
        if ((lane & 7) == 0 && r < P.kb) {
          const double f = (odd ? 1.0 : (oI ? r2 : 1.0) * (oJ ? r2 : 1.0));
          const double v = ((double)z.x + (double)z.y) * f;
          if (v != 0.0) atomicAdd(acc + (int64_t)r * P.ntri + phi * (phi + 1) / 2 + plo, v);
        }
      }
      if (++b == m) {
        if (++a == m - 1) {
          if (++g >= P.ng) break;
          e0 = P.geoff[g];
          m = (int)(P.geoff[g + 1] - e0);
          mixed = P.gflag[g];
          a = 0;
        }
        b = a + 1;
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < P.kb * P.ntri; t += blockDim.x)
    if (acc[t] != 0.0) atomicAdd(P.dens + t, acc[t]);
}

// roots r0 .. r0+kb-1 of V as float-float pairs, KBW per SEF (missing roots zero)
__global__ void k_split_roots(int64_t n, int kb, const double *__restrict__ v, int64_t ldv, float2 *__restrict__ vs) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int r = 0; r < KBW; ++r) vs[s * KBW + r] = r < kb ? split_f64(v[(int64_t)r * ldv + s]) : make_float2(0.f, 0.f);
  }
}

// diagonal: D[tri(p,p)] += occ_p(I) c_I^T (C C^T) c_I, one warp-reduction per orbital
template <int W>
__global__ void __launch_bounds__(DEN_T) k_density_diag(DenParams P) {
  extern __shared__ double acc[];  // [kb][nbf]
  for (int t = threadIdx.x; t < P.kb * P.nbf; t += blockDim.x) acc[t] = 0.0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t nwarp_total = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  const double r2 = sqrt(0.5);
  const double ssd = r2 * r2 + r2 * r2;  // (C C^T)_aa of an open-shell SEF with an even electron count
  for (int64_t base = gw * 32; base < P.nconf; base += nwarp_total * 32) {
    const int64_t I = base + lane;
    const bool ok = I < P.nconf;
    double n2[KB_MAX];
    uint64_t o1[W] = {}, o2[W] = {};
#pragma unroll
    for (int r = 0; r < KB_MAX; ++r) n2[r] = 0.0;
    if (ok) {
      const int64_t s0 = P.sefoff[I], ns = P.sefoff[I + 1] - s0;
      const double ss = (!(P.nelec & 1) && P.nopen[I] != 0) ? ssd : 1.0;
      for (int64_t a = 0; a < ns; ++a) {
#pragma unroll
        for (int r = 0; r < KB_MAX; ++r) {
          if (r >= P.kb) break;
          const double c = P.v[(int64_t)r * P.ldv + s0 + a];
          n2[r] += ss * c * c;
        }
      }
#pragma unroll
      for (int w = 0; w < W; ++w) { o1[w] = P.e1[I * W + w]; o2[w] = P.e2[I * W + w]; }
    }
    // orbitals occupied by any lane of the warp
    uint64_t any[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t x = o1[w];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(0xffffffffu, x, o);
      any[w] = x;
    }
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t m = any[w];
      while (m) {
        const int b = __ffsll((long long)m) - 1;
        m &= m - 1;
        const int p = w * 64 + b;
        const double occ = (double)(((o1[w] >> b) & 1ull) + ((o2[w] >> b) & 1ull));
#pragma unroll
        for (int r = 0; r < KB_MAX; ++r) {
          if (r >= P.kb) break;
          double x = occ * n2[r];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
          if (lane == 0) atomicAdd(acc + r * P.nbf + p, x);  // warps of the block share acc
        }
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < P.kb * P.nbf; t += blockDim.x) {
    const int r = t / P.nbf, p = t % P.nbf;
    if (acc[t] != 0.0) atomicAdd(P.dens + (int64_t)r * P.ntri + p * (p + 1) / 2 + p, acc[t]);
  }
}

}  // namespace

void psoci_density_release(psoci_ctx *c) {
  psoci_free(c->den_geoff);
  psoci_free(c->den_gpoff);
  psoci_free(c->den_gcfg);
  psoci_free(c->den_gorb);
  psoci_free(c->den_gmem);
  psoci_free(c->den_gopen);
  psoci_free(c->den_vs);
  c->den_vs_cap = 0;
  psoci_free(c->den_gflag);
  c->den_ng = 0;
  c->den_npairs = 0;
  c->den_ready = false;
}

// hole-key groups of the current configuration list
static psoci_status density_groups(psoci_ctx *c) {
  if (c->den_ready) return PSOCI_OK;
  cudaStream_t st = c->stream;
  const int nconf = c->nconf, W = c->words;
  const int grid = 4 * 152;
  psoci_status s;
  int64_t *hcnt = nullptr, *hoff = nullptr, *flag = nullptr, *gidx = nullptr, *gm_e = nullptr, *gm_p = nullptr;
  unsigned long long *keys = nullptr;
  int32_t *gcnt = nullptr, *ent_slot = nullptr, *ent_rank = nullptr, *slot2g = nullptr;
  int *err = nullptr;
  int64_t E = 0, ng = 0, E2 = 0, P = 0;
  uint64_t T = 1024;
  auto cleanup = [&]() {
    psoci_free(hcnt); psoci_free(hoff); psoci_free(flag); psoci_free(gidx); psoci_free(gm_e); psoci_free(gm_p);
    psoci_free(keys); psoci_free(gcnt); psoci_free(ent_slot); psoci_free(ent_rank); psoci_free(slot2g);
    psoci_free(err);
  };
#define DEN_TRY(x)              \
  do {                          \
    if ((s = (x)) != PSOCI_OK) { \
      cleanup();                \
      return s;                 \
    }                           \
  } while (0)
#define DEN_CU(x)                          \
  do {                                     \
    cudaError_t _e = (x);                  \
    if (_e != cudaSuccess) {               \
      cleanup();                           \
      return psoci_cuda_fail(c, _e, #x);   \
    }                                      \
  } while (0)
  DEN_TRY(psoci_alloc(c, &hcnt, nconf));
  DEN_TRY(psoci_alloc(c, &hoff, (size_t)nconf + 1));
  psoci_note_launch();
  k_hole_count<<<grid, DEN_T, 0, st>>>(nconf, W, c->d_e1, hcnt);
  DEN_TRY(psoci_scan_i64(c, hcnt, hoff, nconf, &E));
  while (T < (uint64_t)(2 * E)) T <<= 1;
  if (T > (1ull << 31)) {
    cleanup();
    return psoci_fail(c, PSOCI_ERR_UNSUPPORTED, "density1: more than 2^30 hole keys");
  }
  DEN_TRY(psoci_alloc(c, &keys, T));
  DEN_TRY(psoci_alloc(c, &gcnt, T));
  DEN_TRY(psoci_alloc(c, &ent_slot, E));
  DEN_TRY(psoci_alloc(c, &ent_rank, E));
  DEN_TRY(psoci_alloc(c, &err, 1));
  DEN_CU(cudaMemsetAsync(keys, 0, sizeof(unsigned long long) * T, st));
  DEN_CU(cudaMemsetAsync(gcnt, 0, sizeof(int32_t) * T, st));
  DEN_CU(cudaMemsetAsync(err, 0, sizeof(int), st));
  psoci_note_launch();
  if (W == 1)
    k_hole_insert<1><<<grid, DEN_T, 0, st>>>(nconf, c->d_e1, c->d_e2, c->d_jsym, hoff, keys, T - 1, gcnt, ent_slot,
                                             ent_rank, err);
  else
    k_hole_insert<2><<<grid, DEN_T, 0, st>>>(nconf, c->d_e1, c->d_e2, c->d_jsym, hoff, keys, T - 1, gcnt, ent_slot,
                                             ent_rank, err);
  psoci_free(keys);
  DEN_TRY(psoci_alloc(c, &flag, T));
  DEN_TRY(psoci_alloc(c, &gidx, T + 1));
  psoci_note_launch();
  k_group_flags<<<grid, DEN_T, 0, st>>>((int64_t)T, gcnt, flag);
  DEN_TRY(psoci_scan_i64(c, flag, gidx, (int64_t)T, &ng));
  psoci_free(flag);
  int h_err = 0;
  DEN_CU(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  DEN_CU(cudaStreamSynchronize(st));
  if (h_err) {
    cleanup();
    return psoci_fail(c, PSOCI_ERR_NUMERIC, "density1: hole-key table overflow");
  }
  DEN_TRY(psoci_alloc(c, &slot2g, T));
  DEN_TRY(psoci_alloc(c, &gm_e, ng));
  DEN_TRY(psoci_alloc(c, &gm_p, ng));
  psoci_note_launch();
  k_group_compact<<<grid, DEN_T, 0, st>>>((int64_t)T, gcnt, gidx, slot2g, gm_e, gm_p);
  DEN_TRY(psoci_alloc(c, &c->den_geoff, (size_t)ng + 1));
  DEN_TRY(psoci_alloc(c, &c->den_gpoff, (size_t)ng + 1));
  DEN_TRY(psoci_scan_i64(c, gm_e, c->den_geoff, ng, &E2));
  DEN_TRY(psoci_scan_i64(c, gm_p, c->den_gpoff, ng, &P));
  DEN_TRY(psoci_alloc(c, &c->den_gcfg, E2));
  DEN_TRY(psoci_alloc(c, &c->den_gorb, E2));
  DEN_TRY(psoci_alloc(c, &c->den_gflag, ng));
  const bool packed = c->ndet_total < (1ll << 31) && c->nsef_total < (1ll << 31);
  if (packed) {
    DEN_TRY(psoci_alloc(c, &c->den_gmem, E2));
    DEN_TRY(psoci_alloc(c, &c->den_gopen, (size_t)E2 * W));
  }
  psoci_note_launch();
  k_hole_scatter<<<grid, DEN_T, 0, st>>>(nconf, W, c->d_e1, c->d_e2, hoff, ent_slot, ent_rank, slot2g, c->den_geoff,
                                         c->den_gcfg, c->den_gorb, c->d_detoff, c->d_sefoff, c->d_nopen,
                                         c->d_phase, packed ? c->den_gmem : nullptr,
                                         packed ? c->den_gopen : nullptr);
  if (ng > 0) {
    psoci_note_launch();
    if (W == 1)
      k_group_verify<1><<<grid, DEN_T, 0, st>>>(ng, c->den_geoff, c->den_gcfg, c->den_gorb, c->d_e1, c->d_e2,
                                                c->d_jsym, c->den_gflag);
    else
      k_group_verify<2><<<grid, DEN_T, 0, st>>>(ng, c->den_geoff, c->den_gcfg, c->den_gorb, c->d_e1, c->d_e2,
                                                c->d_jsym, c->den_gflag);
  }
  DEN_CU(cudaStreamSynchronize(st));
  DEN_CU(cudaGetLastError());
  cleanup();
#undef DEN_CU
#undef DEN_TRY
  c->den_ng = ng;
  c->den_npairs = P;
  c->den_ready = true;
  return PSOCI_OK;
}

// device vectors (root-major, stride ldv), device output [k][nbf(nbf+1)/2] (overwritten)
extern "C" psoci_status psoci_density1_device(psoci_ctx *c, int k, const double *dV, int64_t ldv, double *dD) {
  if (!c || k < 1 || !dV || !dD) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "density1: build the determinants first");
  if (ldv < c->nsef_total) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "density1: ldv < N");
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  psoci_status s;
  if ((s = density_groups(c))) return s;
  cudaStream_t st = c->stream;
  const int ntri = c->nbf * (c->nbf + 1) / 2;
  PSOCI_CUDA(c, cudaMemsetAsync(dD, 0, sizeof(double) * (size_t)k * ntri, st));
  // roots per pass (spread evenly over the passes), bounded by the block accumulator
  // one warp per configuration pair when every configuration has at most 32 determinants
  const bool warp_path = c->max_ndet <= 32 && c->den_gmem != nullptr;
  // accumulator budget: one block per SM on the warp path, two on the thread path
  int kbmax = (int)(((warp_path ? 200 : 100) * 1024) / (sizeof(double) * ntri));
  if (kbmax < 1) kbmax = 1;
  if (kbmax > (warp_path ? KBW : KB_MAX)) kbmax = warp_path ? KBW : KB_MAX;
  const int npass = (k + kbmax - 1) / kbmax;
  const int kb = (k + npass - 1) / npass;
  int dev = c->device, nsm = 0;
  PSOCI_CUDA(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (warp_path && c->den_vs_cap < (size_t)c->nsef_total * KBW) {
    if ((s = psoci_alloc(c, &c->den_vs, (size_t)c->nsef_total * KBW))) return s;
    c->den_vs_cap = (size_t)c->nsef_total * KBW;
  }
  for (int r0 = 0; r0 < k; r0 += kb) {
    DenParams P{};
    P.nconf = c->nconf;
    P.nbf = c->nbf;
    P.nelec = c->nelec;
    P.ksym = c->ksym;
    P.kb = (k - r0 < kb) ? (k - r0) : kb;
    P.ntri = ntri;
    P.N = c->nsef_total;
    P.ldv = ldv;
    P.v = dV + (int64_t)r0 * ldv;
    P.e1 = c->d_e1;
    P.e2 = c->d_e2;
    P.jsym = c->d_jsym;
    P.nopen = c->d_nopen;
    P.sefoff = c->d_sefoff;
    P.detoff = c->d_detoff;
    P.alpha = c->d_alpha;
    P.beta = c->d_beta;
    P.phase = c->d_phase;
    P.ng = c->den_ng;
    P.npairs = c->den_npairs;
    P.geoff = c->den_geoff;
    P.gpoff = c->den_gpoff;
    P.gcfg = c->den_gcfg;
    P.gorb = c->den_gorb;
    P.gmem = c->den_gmem;
    P.gopen = c->den_gopen;
    P.gflag = c->den_gflag;
    P.vs = c->den_vs;
    P.tmpl = c->d_tmpl;
    P.tmpl_off = c->d_tmpl_off;
    P.dens = dD + (int64_t)r0 * ntri;
    const size_t sm_diag = sizeof(double) * P.kb * c->nbf;
    const size_t sm_pair = sizeof(double) * (size_t)P.kb * ntri + (warp_path ? PSOCI_NCLS * INV_NOPEN * 64 : 0);
    if (warp_path && P.npairs > 0) {
      psoci_note_launch();
      k_split_roots<<<4 * nsm, 256, 0, st>>>(c->nsef_total, P.kb, P.v, ldv, c->den_vs);
      PSOCI_CUDA(c, cudaGetLastError());
    }
    auto kd = (c->words == 1) ? k_density_diag<1> : k_density_diag<2>;
    auto kp = warp_path ? ((c->words == 1) ? k_density_pairs_warp<1> : k_density_pairs_warp<2>)
                        : ((c->words == 1) ? k_density_pairs<1> : k_density_pairs<2>);
    const int nthr = warp_path ? DEN_WT : DEN_T;
    PSOCI_CUDA(c, cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_pair));
    psoci_note_launch();
    kd<<<2 * nsm, DEN_T, sm_diag, st>>>(P);
    PSOCI_CUDA(c, cudaGetLastError());
    if (P.npairs > 0) {
      int per = 0;
      PSOCI_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kp, nthr, sm_pair));
      if (per < 1) per = 1;
      psoci_note_launch();
      kp<<<per * nsm, nthr, sm_pair, st>>>(P);
      PSOCI_CUDA(c, cudaGetLastError());
    }
  }
  return PSOCI_OK;
}

extern "C" psoci_status psoci_density1(psoci_ctx *c, int k, const double *vecs, double *dens) {
  if (!c || k < 1 || !vecs || !dens) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_dets) return psoci_fail(c, PSOCI_ERR_STATE, "density1: build the determinants first");
  psoci_status s;
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  const size_t need = (size_t)c->nsef_total * k;
  const int ntri = c->nbf * (c->nbf + 1) / 2;
  if (c->xy_cap < need) {
    if ((s = psoci_alloc(c, &c->d_x, need)) || (s = psoci_alloc(c, &c->d_y, need))) return s;
    c->xy_cap = need;
  }
  double *dD = nullptr;
  if ((s = psoci_alloc(c, &dD, (size_t)k * ntri))) return s;
  cudaError_t e = cudaMemcpyAsync(c->d_x, vecs, sizeof(double) * need, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    s = psoci_density1_device(c, k, c->d_x, c->nsef_total, dD);
    if (s == PSOCI_OK) {
      e = cudaMemcpyAsync(dens, dD, sizeof(double) * (size_t)k * ntri, cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
  }
  psoci_free(dD);
  if (s != PSOCI_OK) return s;
  if (e != cudaSuccess) return psoci_cuda_fail(c, e, "density1");
  return PSOCI_OK;
}
