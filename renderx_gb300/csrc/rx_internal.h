// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <string>
#include <vector>

#include "../../include/renderx.h"
#include "rx_accel.h"
#include "rx_device.h"
#include "rx_scene.h"

namespace rx {

struct GuideState;
void guide_free(GuideState* g);

// Closest-hit launch shape: variant 0 = one thread per ray, 1-2 = persistent warps
// refilling finished lanes (binary BVH), 3 = the same over the 4-wide BVH, 4 = 3 with the
// first 16 stack entries in shared memory; blocks_per_sm x sms blocks of 128 threads.
struct TraceConfig {
  int variant = 4;
  int blocks_per_sm = 12;
  int sms = 152;
  int pt_blocks_per_sm = 8;  // wavefront extend / shade kernels
  int check_thread = 1;      // reference-visibility check: 1 = thread per ray, 0 = warp per ray
  uint32_t bin_min = 1u << 18;  // bin rays before the walk from this batch size on (0 = never)
  int bin_cell_bits = 4;        // binning key: 2^bits origin cells per axis (Morton order)
  int bin_dir_bits = 4;         // and 2^bits direction levels per octahedral coordinate (or axis)
  int bin_dir_map = 1;          // 1: octahedral map (2^20 bins); 0: direction components
  int walk_stack = 0;           // walk stack entries: 0 = 32 when the BVH is shallower, else 64
};

// Launch shape of the wavefront's extend / shade kernels: blocks of 128 threads per SM
// and the walk: 4 = the 4-wide BVH, 5 = the same with the first 16 stack entries in
// shared memory, 32 or 64 = the binary BVH with that many stack entries (must exceed
// the BVH depth); and the paths per pass.
struct PtShape {
  int blocks_per_sm = 8;
  int stack = 64;
  uint32_t paths_per_pass = 0;  // paths per pass (the queue size)
};

// Scratch of a closest-hit launch over n rays (rx_trace.cu): winner leaves, re-walk
// queue, the ray binning's keys and permutation, the walk's answers by binned slot
// (16 bytes a ray, 16-byte aligned), and bin counters.
constexpr uint32_t kRayBins = 1u << 18;     // the default key's bins (16^3 cells x 4^3 directions)
constexpr uint32_t kRayBinsMax = 1u << 21;  // the finest key rx_trace_set_binning allows
inline size_t trace_scratch_bytes(size_t n) {
  return n * 32 + (size_t)(kRayBinsMax + kRayBinsMax / 1024) * 4 + 4096;
}
// Launchers (rx_trace.cu). `queue`: trace_scratch_bytes(n) bytes, or 8 n bytes when
// `bin` is false. bin: reorder rays by origin cell and direction before the walk (for
// large batches). `ev` (optional): four events recorded before the walk kernel, after
// it, after the visibility check and after the re-walk.
cudaError_t launch_trace_closest(const DevAccel& A, const rx_ray* rays, uint32_t n, int32_t* tid, float* dist,
                                 uint32_t* queue, unsigned long long* counters, const TraceConfig& cfg,
                                 cudaStream_t s, const cudaEvent_t* ev = nullptr, bool bin = true);
// The unit normal of each of the BVH's triangle slots (3 float4 each), for tri_exact_n.
cudaError_t launch_slot_normals(const float4* tris, uint32_t nslots, float4* nrm, cudaStream_t s);
cudaError_t launch_trace_reforder(const DevAccel& A, const rx_ray* rays, uint32_t n, int32_t* tid, float* dist,
                                  unsigned long long* counters, cudaStream_t s);

// Makes `dev` current for a scope and restores the caller's device afterwards.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// A device allocation, released when its owner goes away (move-only).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  cudaError_t alloc(size_t b) {
    release();
    if (b == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    else p = nullptr;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

// A CUDA event, destroyed with its owner (null until created).
struct Event {
  cudaEvent_t e = nullptr;
  Event() = default;
  Event(const Event&) = delete;
  Event& operator=(const Event&) = delete;
  ~Event() {
    if (e) cudaEventDestroy(e);
  }
  cudaError_t create(unsigned flags = cudaEventDefault) { return cudaEventCreateWithFlags(&e, flags); }
  operator cudaEvent_t() const { return e; }
};

// A captured CUDA graph and its executable, destroyed with their owner.
struct Graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t x = nullptr;
  Graph() = default;
  Graph(const Graph&) = delete;
  Graph& operator=(const Graph&) = delete;
  ~Graph() {
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
  }
};

}  // namespace rx

struct rx_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream[2] = {nullptr, nullptr};
  std::string err;

  // host scene
  std::vector<float> verts, vnormals;
  std::vector<uint32_t> tris, tri_obj, tri_local;
  bool has_normals = false;
  std::vector<rx_object> objects;
  bool geometry_dirty = true;

  // acceleration
  rx::RefOrder ref;
  rx::Bvh bvh;
  rx::DevAccel accel{};
  rx::TraceConfig trace_cfg;
  bool accel_ready = false;
  rx::Bvh4 bvh4, bvh8;
  rx::DevBuf d_bvh4, d_bvh8;
  rx::DevBuf d_bvh, d_tris, d_tri_nrm, d_ref, d_ref_leaf_node, d_ref_leaf_range, d_ref_tris, d_anc_range, d_anc_nodes, d_anc_box;
  rx::DevScene scene{};
  bool scene_ready = false;
  rx::DevBuf d_slot_n, d_tri_v, d_tri_n, d_tri_obj, d_objects, d_light_cdf, d_light_tri;
  rx::DevBuf d_counters;     // 4 x u64 diagnostics + per-slot queue lengths
  rx::DevBuf d_queue;        // closest-hit scratch (winner leaves + eager queue)
  // staging ring for host-buffer calls
  static constexpr int kRing = 3;  // staging slots of the host-buffer trace
  rx::DevBuf ring_rays[kRing], ring_tid[kRing], ring_dist[kRing], ring_queue[kRing], ring_counters[kRing];
  cudaEvent_t ring_ev[kRing][3] = {};       // per slot: rays copied in, traced, results copied out
  cudaStream_t ring_stream[kRing] = {};     // per slot: the kernels of its chunks
  size_t ring_chunk = 0;
  size_t stage_rays = (size_t)1 << 22;  // rays per staged chunk (rx_trace_set_staging)
  // per-kernel timing of device-buffer closest-hit calls (rx_trace_set_timing)
  std::vector<cudaEvent_t> timing_ev;  // 4 per recorded call
  size_t timing_used = 0;
  bool timing_on = false;
  // learned guiding (rx_guide.cu)
  rx::GuideState* guide = nullptr;
  // convergence snapshots (rx_set_snapshots)
  double snap_every = 0;
  rx_snapshot_fn snap_fn = nullptr;
  void* snap_user = nullptr;

  rx_status build_scene();
  rx_status fail(rx_status s, const std::string& m) {
    err = m;
    return s;
  }
  rx_status cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return RX_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? RX_ERR_OOM : RX_ERR_CUDA;
  }
};

namespace rx {
// Convergence snapshots of one render (rx_set_snapshots): `due` after each pass or
// iteration; `take` waits for the stream, copies the device film sum and hands the mean
// (sum / count(pixel)) to the context's callback.
struct Snapshots {
  const rx_context* c;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double next;
  std::vector<double> sum, mean;
  explicit Snapshots(const rx_context* ctx) : c(ctx), next(ctx->snap_every) {}
  bool on() const { return c->snap_fn && c->snap_every > 0; }
  double elapsed() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
  bool due() const { return on() && elapsed() >= next; }
  template <class Count>
  cudaError_t take(const double* film_sum, uint32_t w, uint32_t h, double samples, Count&& count, cudaStream_t s) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    const size_t np = (size_t)w * h;
    sum.resize(3 * np);
    mean.resize(3 * np);
    if ((e = cudaMemcpy(sum.data(), film_sum, 3 * np * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
      return e;
    for (size_t k = 0; k < 3 * np; k++) {
      const double n = count(k / 3);
      mean[k] = n > 0 ? sum[k] / n : 0.0;
    }
    const double t = elapsed();
    c->snap_fn(c->snap_user, t, samples, mean.data(), w, h);
    while (next <= t) next += c->snap_every;
    return cudaSuccess;
  }
};

// One scene of a path-traced render: a context with a built scene, its camera and options,
// and the offset (pixels) of its image in the shared film.
struct PtJob {
  const rx_context* ctx;
  rx_camera cam;
  rx_pt_options opt;
  uint64_t film_base;
};
struct PtRun {
  uint32_t paths_per_pass = 0;  // 0 = 2^22
  bool use_graph = true;        // replay a captured pass
  bool autotune = false;        // time launch shapes on the first passes
  bool bin = false;             // bin bounce rays by origin cell and direction before each extend
                                // (measured slower for path tracing: off)
  double time_budget_s = 0;     // > 0: stop launching passes once this much wall time has
                                // passed (checked as each pass is queued, one pass in flight)
};
// Renders all jobs in one wavefront into device films (sum, optional sum of squares).
cudaError_t render_pt_jobs(rx_context* c, const PtJob* jobs, int nj, const PtRun& run, double* film_sum,
                           double* film_sq, rx_render_stats* stats, PtShape* chosen, cudaStream_t s);
// Path tracing (rx_pt.cu): renders into device films (sum, optional sum of squares).
cudaError_t render_pt(rx_context* c, const rx_camera& cam, const rx_pt_options& opt, double* film_sum,
                      double* film_sq, rx_render_stats* stats, cudaStream_t s);
// Vertex connection and merging (rx_vcm.cu): adds iteration images to `film` (sum).
// With kVcmBidirectional in opt.flags, the BidirectionalPathTracer instead (no merging,
// one light path per pixel; radius and alpha unused).
constexpr uint32_t kVcmBidirectional = 1u << 31;
cudaError_t render_vcm(rx_context* c, const rx_camera& cam, const rx_vcm_options& opt, double* film,
                       rx_render_stats* stats, cudaStream_t s);
// PhotonMap (rx_vcm.cu): adds iteration images to `film` (sum).
cudaError_t render_pm(rx_context* c, const rx_camera& cam, const rx_pm_options& opt, double* film,
                      rx_render_stats* stats, cudaStream_t s);
}  // namespace rx
