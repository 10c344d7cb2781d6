// Determinant layer on the device: configuration bit-planes, determinant bit-strings,
// fermionic phases and spin projections.
//
// Reference: PsociDeterminants.C — computeConfigs (:856-975: nsef = (2^(k/2))^2,
// ndet = 2^k with k = max(nopen-1,0)), generateDeterminants (:1467-1505: class choice),
// the per-open-shell templates (:1680-4353) and computePhaseAndSort (:4355-4476).
//
// The reference builds each determinant as an insertion-ordered orbital list (doubles
// ascending, then the open shells that template assigns to that spin, ascending),
// counts the inversions of that order for the phase and sorts.  Here a determinant is a
// pair of bit-strings (alpha, beta; bit p = orbital p), which are sorted by construction;
// the phase is the same inversion count, done with popcounts.
//
// Template order.  Let the open shells be positions 0..n-1 of the ascending singly list and
// a "combo" a bitmask over them.  Enumerating combos of a given size in increasing numeric
// order reproduces the reference's nested loops (outer loop = largest position), and the
// complement of the c-th combo is the (C-1-c)-th combo of the complementary size, which
// is how the reference's forward/backward loops pair up.  Even electron counts
// (:2848-4353): per |delta| section, determinant 2c has alpha = combo c (size n/2+delta),
// beta = complement, ms = msbas+delta, and 2c+1 is its spin-flipped partner with ms =
// msbas-delta; the delta = 0 section uses only the first half of the combos; EVEN class
// sections are delta = 0,2,4,..., ODD class delta = 1,3,5,...  Odd electron counts
// (:1680-2779): section s = 0,1,... gives one determinant per combo of size (n-1)/2+1+s
// of the forward spin (alpha for even s, beta for odd s), the other spin holding the
// complement, with ms = msbas + (1 + k*isgn)/2, k = (2s+1)(-1)^s; isgn = -1 swaps alpha
// and beta of every determinant (pushBackToJoutfg, :2833-2846).
#include <cstdio>
#include <cstring>

#include "psoci_internal.cuh"

namespace {

constexpr int NCLS = PSOCI_NCLS;
constexpr int NOPEN_SLOTS = PSOCI_NOPEN_SLOTS;

struct TmplEntry {
  uint32_t amask, bmask;
  int32_t msoff;
};

void combos(int n, int k, std::vector<uint32_t> &out) {
  out.clear();
  for (uint32_t m = 0; m < (1u << n); ++m)
    if (__builtin_popcount(m) == k) out.push_back(m);
}

// Template run of one (class, nopen); empty when the pair cannot occur.
void template_run(int cls, int n, std::vector<TmplEntry> &run) {
  run.clear();
  uint32_t full = (1u << n) - 1u;
  std::vector<uint32_t> cb;
  if (cls == CLS_FRAC_P || cls == CLS_FRAC_M) {
    if (n % 2 == 0) return;
    int isgn = (cls == CLS_FRAC_P) ? 1 : -1;
    int m = (n - 1) / 2;
    for (int s = 0; m + 1 + s <= n; ++s) {
      combos(n, m + 1 + s, cb);
      int k = (2 * s + 1) * ((s % 2 == 0) ? 1 : -1);
      for (uint32_t fw : cb) {
        uint32_t bw = full & ~fw;
        TmplEntry e;
        e.amask = (s % 2 == 0) ? fw : bw;
        e.bmask = (s % 2 == 0) ? bw : fw;
        if (isgn == -1) std::swap(e.amask, e.bmask);
        e.msoff = (1 + k * isgn) / 2;
        run.push_back(e);
      }
    }
    return;
  }
  if (n % 2 == 1) return;
  if (n == 0) {
    run.push_back({0u, 0u, 0});
    return;
  }
  int m = n / 2;
  for (int delta = (cls == CLS_EVEN) ? 0 : 1; delta <= m; delta += 2) {
    combos(n, m + delta, cb);
    size_t used = (delta == 0) ? cb.size() / 2 : cb.size();
    for (size_t t = 0; t < used; ++t) {
      uint32_t a = cb[t], b = full & ~cb[t];
      run.push_back({a, b, delta});
      run.push_back({b, a, -delta});
    }
  }
}

// one warp per configuration; lanes stride over its determinants
template <int W>
__global__ void k_build_dets(int nconf, int nelec, int ksym, int msbas, const uint64_t *__restrict__ e1,
                             const uint64_t *__restrict__ e2, const int32_t *__restrict__ jsym,
                             const int32_t *__restrict__ nopen, const int64_t *__restrict__ detoff,
                             const uint32_t *__restrict__ tmpl, const int32_t *__restrict__ tmpl_ms,
                             const int32_t *__restrict__ tmpl_off, uint64_t *__restrict__ alpha,
                             uint64_t *__restrict__ beta, uint8_t *__restrict__ phase,
                             uint8_t *__restrict__ nalpha, int32_t *__restrict__ ms) {
  int lane = threadIdx.x & 31;
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < nconf; i += nwarps) {
    uint64_t D[W], S[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      D[w] = e2[i * W + w];
      S[w] = e1[i * W + w] & ~D[w];
    }
    int no = nopen[i];
    int sing[PSOCI_MAX_OPEN];
    int cnt = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t s = S[w];
      while (s && cnt < PSOCI_MAX_OPEN) {
        int b = __ffsll((long long)s) - 1;
        sing[cnt++] = 64 * w + b;
        s &= s - 1;
      }
    }
    // inversions between the doubles (inserted first) and each open shell inserted after
    // them: the number of doubles above it.  Every open shell lands in exactly one spin list.
    int inv = 0;
    for (int t = 0; t < cnt; ++t) {
      int p = sing[t];
#pragma unroll
      for (int w = 0; w < W; ++w) {
        int lo = p + 1 - 64 * w;
        uint64_t m = (lo <= 0) ? ~0ull : (lo >= 64 ? 0ull : (~0ull << lo));
        inv += __popcll(D[w] & m);
      }
    }
    int cls = psoci_det_class(nelec & 1, jsym[i], ksym);
    int run0 = tmpl_off[cls * NOPEN_SLOTS + no];
    int nd = 1 << (no > 1 ? no - 1 : 0);
    int64_t d0 = detoff[i];
    for (int d = lane; d < nd; d += 32) {
      uint32_t ent = tmpl[run0 + d];
      uint32_t am = ent & 0xfffu, bm = (ent >> 12) & 0xfffu;
      uint64_t A[W], B[W];
#pragma unroll
      for (int w = 0; w < W; ++w) { A[w] = D[w]; B[w] = D[w]; }
      for (int t = 0; t < cnt; ++t) {
        int p = sing[t];
        if (am & (1u << t)) A[p >> 6] |= 1ull << (p & 63);
        if (bm & (1u << t)) B[p >> 6] |= 1ull << (p & 63);
      }
      int na = 0;
#pragma unroll
      for (int w = 0; w < W; ++w) {
        alpha[(d0 + d) * W + w] = A[w];
        beta[(d0 + d) * W + w] = B[w];
        na += __popcll(A[w]);
      }
      // open shells are inserted in ascending order, so they add no inversions among
      // themselves; the phase is the doubles/open-shell inversion count mod 2.
      phase[d0 + d] = (uint8_t)(inv & 1);
      nalpha[d0 + d] = (uint8_t)na;
      ms[d0 + d] = msbas + tmpl_ms[run0 + d];
    }
  }
}

}  // namespace

void psoci_dets_release(psoci_ctx *c) {
  psoci_free(c->d_sefoff);
  psoci_free(c->d_detoff);
  psoci_free(c->d_alpha);
  psoci_free(c->d_beta);
  psoci_free(c->d_phase);
  psoci_free(c->d_nalpha);
  psoci_free(c->d_ms);
  psoci_free(c->d_tmpl);
  psoci_free(c->d_tmpl_ms);
  psoci_free(c->d_tmpl_off);
  c->have_dets = false;
}

psoci_status psoci_dets_build(psoci_ctx *c) {
  if (!c->have_cfgs) return psoci_fail(c, PSOCI_ERR_STATE, "psoci_build_determinants: no configurations set");
  psoci_h_release(c);
  psoci_dets_release(c);
  const int n = c->nconf;
  // counts and offsets (host; O(nconf))
  c->h_sefoff.assign(n + 1, 0);
  c->h_detoff.assign(n + 1, 0);
  c->max_nsef = c->max_ndet = 0;
  std::vector<int32_t> nopen(n);
  for (int i = 0; i < n; ++i) {
    int no = 0;
    const uint8_t *o = &c->h_occ[(size_t)i * c->nbf];
    for (int p = 0; p < c->nbf; ++p) no += (o[p] == 1);
    nopen[i] = no;
    int k = no > 1 ? no - 1 : 0;
    int nd = 1 << k, ns = (1 << (k / 2)) * (1 << (k / 2));
    c->h_detoff[i + 1] = c->h_detoff[i] + nd;
    c->h_sefoff[i + 1] = c->h_sefoff[i] + ns;
    if (nd > c->max_ndet) c->max_ndet = nd;
    if (ns > c->max_nsef) c->max_nsef = ns;
  }
  c->nsef_total = c->h_sefoff[n];
  c->ndet_total = c->h_detoff[n];
  if (c->nsef_total > INT32_MAX) return psoci_fail(c, PSOCI_ERR_UNSUPPORTED, "more than 2^31-1 SEFs");

  // template table
  std::vector<uint32_t> tm;
  std::vector<int32_t> tms, toff(NCLS * NOPEN_SLOTS + 1, 0);
  std::vector<TmplEntry> run;
  for (int cls = 0; cls < NCLS; ++cls)
    for (int no = 0; no < NOPEN_SLOTS; ++no) {
      toff[cls * NOPEN_SLOTS + no] = (int32_t)tm.size();
      template_run(cls, no, run);
      for (auto &e : run) {
        tm.push_back(e.amask | (e.bmask << 12));
        tms.push_back(e.msoff);
      }
    }
  toff[NCLS * NOPEN_SLOTS] = (int32_t)tm.size();
  psoci_status st;
  if ((st = psoci_alloc(c, &c->d_sefoff, n + 1)) || (st = psoci_alloc(c, &c->d_detoff, n + 1)) ||
      (st = psoci_alloc(c, &c->d_alpha, (size_t)c->ndet_total * c->words)) ||
      (st = psoci_alloc(c, &c->d_beta, (size_t)c->ndet_total * c->words)) ||
      (st = psoci_alloc(c, &c->d_phase, (size_t)c->ndet_total)) ||
      (st = psoci_alloc(c, &c->d_nalpha, (size_t)c->ndet_total)) ||
      (st = psoci_alloc(c, &c->d_ms, (size_t)c->ndet_total)) || (st = psoci_alloc(c, &c->d_tmpl, tm.size())) ||
      (st = psoci_alloc(c, &c->d_tmpl_ms, tms.size())) || (st = psoci_alloc(c, &c->d_tmpl_off, toff.size())))
    return st;
  cudaStream_t s = c->stream;
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_sefoff, c->h_sefoff.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_detoff, c->h_detoff.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_nopen, nopen.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_tmpl, tm.data(), sizeof(uint32_t) * tm.size(), cudaMemcpyHostToDevice, s));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_tmpl_ms, tms.data(), sizeof(int32_t) * tms.size(), cudaMemcpyHostToDevice, s));
  PSOCI_CUDA(c, cudaMemcpyAsync(c->d_tmpl_off, toff.data(), sizeof(int32_t) * toff.size(), cudaMemcpyHostToDevice, s));

  int threads = 256;
  int64_t warps = n;
  int blocks = (int)std::min<int64_t>((warps * 32 + threads - 1) / threads, 152 * 64);
  if (blocks < 1) blocks = 1;
  psoci_note_launch();
  if (c->words == 1)
    k_build_dets<1><<<blocks, threads, 0, s>>>(n, c->nelec, c->ksym, c->mx_open / 2, c->d_e1, c->d_e2, c->d_jsym,
                                                c->d_nopen, c->d_detoff, c->d_tmpl, c->d_tmpl_ms, c->d_tmpl_off,
                                                c->d_alpha, c->d_beta, c->d_phase, c->d_nalpha, c->d_ms);
  else
    k_build_dets<2><<<blocks, threads, 0, s>>>(n, c->nelec, c->ksym, c->mx_open / 2, c->d_e1, c->d_e2, c->d_jsym,
                                                c->d_nopen, c->d_detoff, c->d_tmpl, c->d_tmpl_ms, c->d_tmpl_off,
                                                c->d_alpha, c->d_beta, c->d_phase, c->d_nalpha, c->d_ms);
  PSOCI_CUDA(c, cudaGetLastError());
  PSOCI_CUDA(c, cudaStreamSynchronize(s));
  c->have_dets = true;
  return PSOCI_OK;
}
