// Error helpers and the device-wide exclusive scan used by the builders.
#include <atomic>
#include <cstdio>
#include <mutex>
#include <unordered_map>
#include <vector>
#include <algorithm>

#include "psoci_internal.cuh"

// Process-wide count of kernels this library has launched (all contexts, all devices).
static std::atomic<unsigned long long> g_launches{0};
void psoci_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
extern "C" unsigned long long psoci_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

psoci_status psoci_fail(psoci_ctx *c, psoci_status s, const std::string &msg) {
  if (c) c->err = msg;
  return s;
}

// The device-memory cache of psoci_alloc.  One lock guards the owner and size of every
// live block, every context's pool of released blocks and the bytes the pools of each
// device hold: a block may be released on one thread while another context's call runs on
// another, and a failed cudaMalloc empties the pools of every context on its device.
namespace {
std::mutex g_mu;
std::unordered_map<void *, std::pair<psoci_ctx *, size_t>> g_blocks;
std::unordered_map<int, size_t> g_pooled;                 // bytes in the pools, per device
std::unordered_map<int, std::vector<psoci_ctx *>> g_ctxs; // live contexts, per device

// every context's released blocks on one device go back to the driver (g_mu held);
// cudaFree waits for the device, so no stream still uses them afterwards
void flush_device_locked(int dev) {
  auto it = g_ctxs.find(dev);
  if (it != g_ctxs.end())
    for (psoci_ctx *c : it->second) {
      for (auto &kv : c->pool) cudaFree(kv.second);
      c->pool.clear();
      c->pool_bytes = 0;
    }
  g_pooled[dev] = 0;
}
}  // namespace

void psoci_pool_register(psoci_ctx *c) {
  std::lock_guard<std::mutex> g(g_mu);
  g_ctxs[c->device].push_back(c);
}

void *psoci_device_alloc(psoci_ctx *c, size_t bytes, cudaError_t *err) {
  if (bytes == 0) bytes = 1;
  void *p = nullptr;
  if (!c) {
    *err = cudaMalloc(&p, bytes);
    return (*err == cudaSuccess) ? p : nullptr;
  }
  bool reused = false;
  {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = c->pool.lower_bound(bytes);
    if (it != c->pool.end() && it->first - bytes <= bytes / 4) {
      const size_t sz = it->first;
      p = it->second;
      c->pool.erase(it);
      c->pool_bytes -= sz;
      g_pooled[c->device] -= sz;
      g_blocks[p] = {c, sz};
      reused = true;
    }
  }
  if (reused) {
    // work of this context that used the block before its release ends first (cudaFree
    // would have waited for it)
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      {
        std::lock_guard<std::mutex> g(g_mu);
        g_blocks.erase(p);
      }
      cudaFree(p);
      *err = e;
      return nullptr;
    }
    *err = cudaSuccess;
    return p;
  }
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    bool had = false;
    {
      std::lock_guard<std::mutex> g(g_mu);
      had = g_pooled[c->device] > 0;
      if (had) flush_device_locked(c->device);
    }
    if (had) e = cudaMalloc(&p, bytes);
  }
  if (e != cudaSuccess) {
    *err = e;
    return nullptr;
  }
  std::lock_guard<std::mutex> g(g_mu);
  g_blocks[p] = {c, bytes};
  *err = cudaSuccess;
  return p;
}

void psoci_device_free(void *p) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_blocks.find(p);
    if (it != g_blocks.end()) {
      psoci_ctx *c = it->second.first;
      const size_t sz = it->second.second;
      g_blocks.erase(it);
      // the cap holds for all contexts of the device together
      if (c && g_pooled[c->device] + sz <= c->pool_cap) {
        c->pool.insert({sz, p});
        c->pool_bytes += sz;
        g_pooled[c->device] += sz;
        return;
      }
    }
  }
  cudaFree(p);
}

void psoci_pool_flush(psoci_ctx *c) {
  std::lock_guard<std::mutex> g(g_mu);
  for (auto &kv : c->pool) cudaFree(kv.second);
  c->pool.clear();
  g_pooled[c->device] -= c->pool_bytes;
  c->pool_bytes = 0;
}

// blocks of a context that is going away and were never released; the context leaves the
// device's list
void psoci_pool_forget(psoci_ctx *c) {
  std::lock_guard<std::mutex> g(g_mu);
  for (auto it = g_blocks.begin(); it != g_blocks.end();) {
    if (it->second.first == c) {
      cudaFree(it->first);
      it = g_blocks.erase(it);
    } else {
      ++it;
    }
  }
  auto &v = g_ctxs[c->device];
  v.erase(std::remove(v.begin(), v.end(), c), v.end());
}

psoci_status psoci_cuda_fail(psoci_ctx *c, cudaError_t e, const char *where) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  if (c) c->err = buf;
  return (e == cudaErrorMemoryAllocation) ? PSOCI_ERR_NOMEM : PSOCI_ERR_CUDA;
}

namespace {
constexpr int SCAN_T = 512;
constexpr int SCAN_PER = 8;
constexpr int SCAN_CHUNK = SCAN_T * SCAN_PER;

// block-wide exclusive scan of one chunk; writes per-block total
__global__ void k_scan_chunk(const int64_t *in, int64_t *out, int64_t n, int64_t *blocksum, const int64_t *blockoff) {
  __shared__ int64_t warp_tot[SCAN_T / 32];
  int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_PER;
  int64_t v[SCAN_PER];
  int64_t sum = 0;
#pragma unroll
  for (int q = 0; q < SCAN_PER; ++q) {
    int64_t idx = base + q;
    v[q] = (idx < n) ? in[idx] : 0;
    sum += v[q];
  }
  // warp inclusive scan of per-thread sums
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int64_t w = (lane < SCAN_T / 32) ? warp_tot[lane] : 0;
    int64_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < SCAN_T / 32) warp_tot[lane] = wi - w;  // exclusive warp offsets
    if (lane == SCAN_T / 32 - 1 && blocksum) blocksum[blockIdx.x] = wi;
  }
  __syncthreads();
  if (out) {
    int64_t run = warp_tot[wid] + (incl - sum) + (blockoff ? blockoff[blockIdx.x] : 0);
#pragma unroll
    for (int q = 0; q < SCAN_PER; ++q) {
      int64_t idx = base + q;
      if (idx < n) out[idx] = run;
      run += v[q];
    }
  }
}

__global__ void k_write_total(const int64_t *in, const int64_t *out, int64_t n, int64_t *total_slot) {
  // out[n] = out[n-1] + in[n-1]
  if (n == 0) *total_slot = 0;
  else *total_slot = out[n - 1] + in[n - 1];
}
}  // namespace

// exclusive scan of n counts into out[0..n]; out[n] = total; total also returned on host.
// in and out must not alias.
psoci_status psoci_scan_i64(psoci_ctx *c, const int64_t *d_in, int64_t *d_out, int64_t n, int64_t *total) {
  cudaStream_t s = c->stream;
  if (n <= 0) {
    int64_t z = 0;
    PSOCI_CUDA(c, cudaMemcpyAsync(d_out, &z, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    PSOCI_CUDA(c, cudaStreamSynchronize(s));
    if (total) *total = 0;
    return PSOCI_OK;
  }
  int64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  int64_t *d_bs = nullptr, *d_bo = nullptr;
  psoci_status st = psoci_alloc(c, &d_bs, nb + 1);
  if (st) return st;
  st = psoci_alloc(c, &d_bo, nb + 1);
  if (st) { psoci_free(d_bs); return st; }
  psoci_note_launch();
  k_scan_chunk<<<(unsigned)nb, SCAN_T, 0, s>>>(d_in, nullptr, n, d_bs, nullptr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    if (nb > 1) {
      int64_t tb = 0;
      st = psoci_scan_i64(c, d_bs, d_bo, nb, &tb);
    } else {
      int64_t z = 0;
      e = cudaMemcpyAsync(d_bo, &z, sizeof(int64_t), cudaMemcpyHostToDevice, s);
    }
  }
  if (e == cudaSuccess && st == PSOCI_OK) {
    psoci_note_launch();
    k_scan_chunk<<<(unsigned)nb, SCAN_T, 0, s>>>(d_in, d_out, n, nullptr, d_bo);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && st == PSOCI_OK) {
    psoci_note_launch();
    k_write_total<<<1, 1, 0, s>>>(d_in, d_out, n, d_out + n);
    e = cudaGetLastError();
  }
  int64_t tot = 0;
  if (e == cudaSuccess && st == PSOCI_OK) e = cudaMemcpyAsync(&tot, d_out + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && st == PSOCI_OK) e = cudaStreamSynchronize(s);
  psoci_free(d_bs);
  psoci_free(d_bo);
  if (st != PSOCI_OK) return st;
  if (e != cudaSuccess) return psoci_cuda_fail(c, e, "psoci_scan_i64");
  if (total) *total = tot;
  return PSOCI_OK;
}
