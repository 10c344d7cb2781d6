// Mixed-precision sigma that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc while they run —
//   * host programs that hand the whole GPU memory budget to their own allocator up front
//     and forbid other allocations (as the reference's Global Arrays runtime does with its
//     fixed per-rank memory), and
//   * loops that must not take the implicit device synchronisation a cudaMalloc/cudaFree can
//     cause.
// psoci_sigma_device stages its FP32 input copy in a buffer that it grows with cudaMalloc on
// demand; this variant stages it in the fixed array below instead.  The caller still owns
// the input and output (device pointers) and the Hamiltonian must already be built with its
// FP32 copy (PSOCI_HMODE_CSR_BOTH).
//
// Limits and sharing:
//   * the array holds kNoAllocScratchFloats floats (16 MiB); the staging needs N * 8 floats,
//     so N (SEFs) must not exceed 524,288 — larger problems get PSOCI_ERR_UNSUPPORTED;
//   * every device that loads this library keeps the 16 MiB array until the process exits;
//   * all calls on a device share the array and it keeps the last call's contents; each call
//     overwrites every entry it reads before reading it, so nothing has to start at zero;
//   * all contexts on a device share the one array; calls that overlap on the GPU (other
//     streams, other contexts on the same device) race on it and must be serialised by the
//     caller;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress)
//     and caches it; make that first call before any stream capture begins.
#include <mutex>
#include <string>

#include "psoci_internal.cuh"

namespace {

constexpr size_t kNoAllocScratchFloats = (size_t)4 << 20;  // 4 Mi floats = 16 MiB per device
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_x32[kNoAllocScratchFloats];

// device address of g_noalloc_x32 on each device (host code cannot use the symbol directly)
float *g_noalloc_ptr[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mu;

psoci_status noalloc_scratch(psoci_ctx *c, float **out) {
  if (c->device < 0 || c->device >= kNoAllocMaxDevices)
    return psoci_fail(c, PSOCI_ERR_UNSUPPORTED, "sigma_mixed_noalloc: device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[c->device]) {
    PSOCI_CUDA(c, cudaSetDevice(c->device));
    void *p = nullptr;
    PSOCI_CUDA(c, cudaGetSymbolAddress(&p, g_noalloc_x32));
    g_noalloc_ptr[c->device] = static_cast<float *>(p);
  }
  *out = g_noalloc_ptr[c->device];
  return PSOCI_OK;
}

}  // namespace

extern "C" psoci_status psoci_sigma_mixed_noalloc(psoci_ctx *c, int k, const double *dX, int ldx, double *dY,
                                                  int ldy) {
  if (!c || !dX || !dY) return PSOCI_ERR_INVALID_ARG;
  if (!c->have_h) return psoci_fail(c, PSOCI_ERR_STATE, "sigma_mixed_noalloc: Hamiltonian not built");
  if (c->direct) return psoci_fail(c, PSOCI_ERR_STATE, "sigma_mixed_noalloc: direct mode stores no matrix");
  if (!c->d_val32)
    return psoci_fail(c, PSOCI_ERR_STATE, "sigma_mixed_noalloc: needs the FP32 copy (PSOCI_HMODE_CSR_BOTH)");
  if (k < 1 || ldx < k || ldy < k) return psoci_fail(c, PSOCI_ERR_INVALID_ARG, "sigma_mixed_noalloc: bad k / ld");
  // the staging holds one chunk of at most 8 vectors: N * 8 floats
  if ((size_t)c->nsef_total * 8 > kNoAllocScratchFloats)
    return psoci_fail(c, PSOCI_ERR_UNSUPPORTED,
                      "sigma_mixed_noalloc: N = " + std::to_string(c->nsef_total) +
                          " SEFs exceeds the static scratch (N * 8 <= 4 Mi floats, i.e. N <= 524288)");
  psoci_status s;
  PSOCI_CUDA(c, cudaSetDevice(c->device));
  float *scratch = nullptr;
  if ((s = noalloc_scratch(c, &scratch))) return s;
  return psoci_sigma_launch(c, k, dX, ldx, dY, ldy, PSOCI_PREC_MIXED, scratch);
}
