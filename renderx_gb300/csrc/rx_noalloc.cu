// Closest hit without any allocation at call time.
//
// Some callers cannot allocate device memory when they trace: a host application whose
// device memory is owned by its own pool allocator (cudaMalloc would bypass or exhaust
// it), or a latency-sensitive loop that must not pay cudaMalloc's implicit device
// synchronisation. rx_trace_closest_device grows a per-context scratch buffer with
// cudaMalloc on first use of a larger batch; this entry point instead runs the same
// kernels with their scratch in one file-scope device array of fixed size:
//   counters  : 8 x uint64 (eager-queue length, diagnostics, batch cursor)
//   hit_leaf  : one uint32 per ray (each winner's reference leaf)
//   queue     : one uint32 per ray (rays re-walked exactly)
// for at most kNoAllocMaxRays rays per call, 8 MiB + 64 B. Every GPU that loads the
// library holds the array until the process exits. Each call clears the counters (a
// memset, no allocation); they are not added to the context's trace statistics.
#include <mutex>

#include "rx_internal.h"

namespace {

constexpr uint32_t kNoAllocMaxRays = 1u << 20;
constexpr size_t kCounterBytes = 8 * sizeof(unsigned long long);
constexpr size_t kScratchBytes = kCounterBytes + 2 * sizeof(uint32_t) * (size_t)kNoAllocMaxRays;

static __device__ __align__(256) unsigned char g_trace_scratch[kScratchBytes];

// Device address of g_trace_scratch per device: host code only holds a stand-in for
// the array, so the address is looked up once per device with that device current.
// The address belongs to the device's primary context (the one the CUDA runtime
// uses); it stays valid until that context is destroyed (cudaDeviceReset).
std::mutex g_mu;
constexpr int kMaxDevices = 64;
void* g_addr[kMaxDevices] = {};

cudaError_t scratch_address(int device, void** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!g_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_trace_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *out = g_addr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" rx_status rx_trace_closest_noalloc(rx_context* c, const rx_ray* d_rays, uint32_t n, int32_t* d_tid,
                                              float* d_dist, void* stream) {
  if (!c) return RX_ERR_INVALID;
  if (!c->accel_ready) return c->fail(RX_ERR_STATE, "accelerator not built");
  if (n == 0) return RX_OK;
  if (n > kNoAllocMaxRays)
    return c->fail(RX_ERR_INVALID, "rx_trace_closest_noalloc: " + std::to_string(n) +
                                       " rays exceed the limit of 1048576 rays per call");
  if (!d_rays || !d_tid || !d_dist) return c->fail(RX_ERR_INVALID, "null buffer");
  if (reinterpret_cast<uintptr_t>(d_rays) % 16) return c->fail(RX_ERR_INVALID, "rays must be 16-byte aligned");
  rx::DeviceGuard guard(c->device);
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e == cudaSuccess && cur != c->device) e = cudaErrorInvalidDevice;  // the switch did not take
  if (e != cudaSuccess) return c->cuda(e, "trace_closest_noalloc: select the context's device");
  void* base = nullptr;
  if ((e = scratch_address(c->device, &base)) != cudaSuccess) return c->cuda(e, "trace_closest_noalloc: scratch address");
  auto* counters = static_cast<unsigned long long*>(base);
  auto* queue = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + kCounterBytes);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  // counters start at zero on every call (the previous call's values stay in the array)
  e = cudaMemsetAsync(counters, 0, kCounterBytes, st);
  if (e == cudaSuccess)
    e = rx::launch_trace_closest(c->accel, d_rays, n, d_tid, d_dist, queue, counters, c->trace_cfg, st, nullptr,
                                 false);
  return c->cuda(e, "trace_closest_noalloc");
}
