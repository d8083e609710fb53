/*
 * renderx.h - C ABI of the GB300 light-transport library (librenderx_gb300.so).
 *
 * Plain C types only: pointers, sizes, POD structs. Every call returns an rx_status;
 * rx_last_error() gives the message of the last failure on a context. A context owns
 * one CUDA stream on one device; calls on one context are not thread-safe, calls on
 * different contexts are.
 *
 * Each entry point names the reference interface it replaces (reference file:line).
 */
#ifndef RENDERX_H
#define RENDERX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rx_context rx_context;

typedef enum rx_status {
  RX_OK = 0,
  RX_ERR_INVALID = 1,     /* bad argument */
  RX_ERR_CUDA = 2,        /* CUDA runtime error */
  RX_ERR_OOM = 3,         /* device or host allocation failed */
  RX_ERR_STATE = 4,       /* call out of order (e.g. trace before build) */
  RX_ERR_TIMEOUT = 5,     /* a bounded device loop ran out of iterations */
  RX_ERR_UNSUPPORTED = 6
} rx_status;

/* Material codes (reference ConfigManager.cpp:25-164 <type> values). */
enum {
  RX_MAT_DIFFUSE = 0,     /* SceneDiffuseObject / DiffuseMaterial */
  RX_MAT_GLOSSY = 1,      /* SceneGlossyObject / GlossyMaterial (Phong lobe) */
  RX_MAT_REFRACTIVE = 2,  /* SceneRefractiveObject / RefractiveMaterial */
  RX_MAT_EMISSIVE = 3,    /* SceneEmissiveObject */
  RX_MAT_PHONG = 4,       /* ScenePhongObject: glossy + diffuse, lobe picked at random */
  RX_MAT_REFLECTIVE = 5,  /* SceneReflectiveObject: RefractiveMaterial with coeff -1 */
  RX_MAT_VPM = 6          /* SceneVPMObject: dielectric boundary + homogeneous medium */
};

/* One scene object: its triangle range in the global triangle list and its material.
 * Mirrors the SceneObject subclasses' fields set by ConfigManager::generateSceneObject
 * (reference ConfigManager.cpp:25-164). */
typedef struct rx_object {
  uint32_t tri_begin, tri_count;  /* global triangle range (object-major order) */
  uint32_t material;              /* RX_MAT_* */
  uint32_t has_vertex_normals;    /* 1: shading normals interpolate vertex normals */
  float color[3];                 /* diffuse albedo / glossy colour / emission / surface colour */
  float coeff;                    /* glossy exponent */
  float diffuse_color[3];         /* Phong diffuse component */
  float ior;                      /* refractive index (<0: mirror) */
  float sigma_s[3], sigma_a[3];   /* homogeneous medium */
  float g;                        /* HG asymmetry */
  float decay[3];                 /* RefractiveMaterial decayColor (per unit length) */
  float step_size;                /* medium ray-marching step of PhotonMap (SceneVPMObject::stepSize,
                                     <stepsize>; 0 = the reference's 0.0005) */
} rx_object;

typedef struct rx_build_options {
  int32_t split_policy;   /* 0: reference as built by GCC/libstdc++ (x axis always);
                             1: best-ratio axis (libc++/MSVC builds of the reference) */
  int32_t leaf_size;      /* BVH leaf size (1..8), 0 = default 3 (the fastest walk on the
                              4.1M-triangle bench scene: 8.97 ms per 2^24 rays against
                              9.18 / 9.36 / 9.41 / 9.52 at 2 / 4 / 6 / 8; the answers do
                              not depend on it) */
  int32_t host_threads;   /* 0 = all cores */
  int32_t reserved;
} rx_build_options;

/* A ray: origin and direction, 32 bytes (w components ignored). */
typedef struct rx_ray {
  float ox, oy, oz, ow;
  float dx, dy, dz, dw;
} rx_ray;

/* Pinhole camera with the reference's integer sightDist in pixels (reference
 * include/Camera.h:10-31, ConfigManager.cpp:263-269). */
typedef struct rx_camera {
  uint32_t width, height;
  uint32_t sight_dist;
  uint32_t reserved;
  float position[3];
  float focus[3];
  float up[3];
} rx_camera;

/* Path-tracing options. */
typedef struct rx_pt_options {
  uint32_t spp;            /* samples per pixel */
  uint32_t max_depth;      /* MCRenderer::maxDepth (bounce rays per path) */
  uint32_t rr_mode;        /* 0: the reference's Russian roulette at every bounce
                              (p = max albedo); 1: roulette only from depth 3 on */
  uint32_t nee;            /* 0: PathTracer (BSDF sampling only); 1: PathTracerTest
                              (light sampling + balance-heuristic MIS) */
  uint64_t seed;
  uint32_t paths_per_pass; /* wavefront size, 0 = 2^22 */
  uint32_t flags;          /* RX_PT_GUIDED or 0 */
  float time_budget_s;     /* > 0: stop after the pass during which this much wall time
                              has passed (whole passes, spp the cap); paths run in
                              sample-major order, each pixel's mean divides by its own
                              sample count (stats.paths = paths done). rx_render_pt only:
                              0 in batch items. The equal-time comparisons of
                              MCRenderer's per-iteration timer (reference
                              include/MCRenderer.h:60, src/PathTracer.cpp:9,22). */
  uint32_t reserved;       /* 0 */
} rx_pt_options;

/* rx_pt_options.flags: sample directions at diffuse / glossy / Phong vertices by
 * one-sample MIS between the BSDF and the context's guiding network (rx_guide_init),
 * training the network on the render's own samples during the first train_passes
 * passes; the first warmup_passes passes sample by the BSDF alone. PathTracer (nee = 0)
 * only. */
#define RX_PT_GUIDED 1u

/* Learned path guiding (no reference counterpart): a BF16 MLP on the tensor cores,
 * 80 encoded inputs -> 4 x 64 ReLU -> 8 von Mises-Fisher lobes, trained online with Adam. */
typedef struct rx_guide_options {
  float learning_rate;     /* Adam step size (5e-3) */
  float bsdf_fraction;     /* one-sample MIS: probability of sampling the BSDF (0.5) */
  uint32_t batch;          /* training records per Adam step (2^18) */
  uint32_t train_passes;   /* rendering passes whose samples train the network */
  uint32_t steps_per_pass; /* Adam steps after each training pass */
  uint32_t warmup_passes;  /* first passes sample by the BSDF alone (no inference) */
  uint64_t seed;           /* weight initialisation */
} rx_guide_options;

/* One scene of a batched path-traced render. */
typedef struct rx_batch_item {
  rx_context* scene;       /* context holding the scene (objects set, accelerator built) */
  rx_camera camera;
  rx_pt_options options;   /* spp, max_depth, rr_mode, nee, seed, flags (RX_PT_GUIDED: guided
                              by the scene context's network, rx_guide_init); paths_per_pass
                              unused, time_budget_s 0 */
  double* film_rgb;        /* host output: width*height*3 per-pixel means, rows from the top */
} rx_batch_item;

typedef struct rx_batch_options {
  uint32_t paths_per_pass; /* wavefront size shared by all scenes, 0 = 2^22 */
  uint32_t use_graph;      /* 1: capture one pass as a CUDA graph and replay it */
  uint32_t autotune;       /* 1: time candidates on the first passes, two passes each (their
                              samples count): the launch shapes at paths_per_pass (the
                              4-wide short-stack walks, 6 and 5, when every scene's 4-wide
                              tree fits, else the binary walks; 4, 8 or 16 shading blocks
                              per SM), then the pass sizes 2^20..2^23 with the best shape. Guided batches take an
                              equal share of every item in each pass; autotuned ones do so in
                              the tuning passes only, then take the items one after another
                              (a pass then touches one or two scenes' trees). */
  uint32_t chosen_paths_per_pass;  /* out: paths per pass of the remaining passes */
  int32_t chosen_blocks_per_sm;  /* out: extend / shade blocks per SM used */
  int32_t chosen_stack;          /* out: walk used: 4 = 4-wide BVH, 5 = 4-wide BVH with a
                                    shared-memory short stack, 6 = 5 on persistent warps
                                    that refill finished lanes (the default), 32 / 64 =
                                    binary BVH with that stack depth */
} rx_batch_options;

/* Vertex connection and merging options (VCMTracer, reference include/VCMTracer.h). */
typedef struct rx_vcm_options {
  uint32_t iterations;     /* progressive iterations (the reference loops until its time budget) */
  uint32_t max_depth;      /* MCRenderer::maxDepth, at most 21 */
  uint32_t light_paths;    /* light subpaths per iteration, 0 = width*height (the reference) */
  uint32_t flags;          /* RX_VCM_FULL_PATH_MIS or 0 */
  float radius;            /* initial merge radius (VCMTracer::mergeRadius, <radius> in XML) */
  float alpha;             /* radius shrink: r *= ((s+alpha)/(s+1))^(1/3) (reference default 0.6667) */
  uint64_t seed;
  float time_budget_s;     /* > 0: stop after the iteration during which this much wall time
                              has passed (VCMTracer.cpp:142, the <time> runtime), iterations
                              the cap; the mean is over the iterations done (stats.paths =
                              pixels x iterations done) */
  uint32_t reserved;       /* 0 */
} rx_vcm_options;
/* Evaluate each merge's colour and MIS weight with the reference's loops over the whole
 * joined path (VCMTracer::connectColorProb / connectMergeWeight, O(path length) per
 * pair) instead of the per-subpath records (O(1) per pair). Same estimator; slower. */
#define RX_VCM_FULL_PATH_MIS 1u

/* BidirectionalPathTracer options (reference include/BidirectionalPathTracer.h): per
 * iteration one eye and one light subpath per pixel, all their connections. */
typedef struct rx_bpt_options {
  uint32_t iterations;     /* samples per pixel (BidirectionalPathTracer::spp) */
  uint32_t max_depth;      /* MCRenderer::maxDepth, at most 21 */
  uint32_t flags;          /* RX_VCM_FULL_PATH_MIS or 0 */
  float time_budget_s;     /* > 0: stop after the iteration during which this much wall time
                              has passed (BidirectionalPathTracer.cpp:114), as rx_vcm_options */
  uint64_t seed;
} rx_bpt_options;

/* PhotonMap options (reference include/Photonmap.h): progressive photon mapping with
 * ray marching through media. */
typedef struct rx_pm_options {
  uint32_t iterations;     /* progressive iterations (PhotonMap::spp) */
  uint32_t max_depth;      /* light-path depth (MCRenderer::maxDepth), at most 21 */
  uint32_t light_paths;    /* photon paths per iteration, 0 = width*height (mPhotonsNum) */
  uint32_t flags;          /* 0 */
  float radius;            /* base radius (PhotonMap::setRadius, <radius>) */
  float alpha;             /* radius exponent, 0 = the reference's 2/3 */
  uint64_t seed;
  float time_budget_s;     /* > 0: stop after the iteration during which this much wall time
                              has passed, as rx_vcm_options */
  uint32_t reserved;       /* 0 */
} rx_pm_options;

typedef struct rx_render_stats {
  uint64_t extension_rays; /* closest-hit rays traced (camera + bounce) */
  uint64_t shadow_rays;    /* next-event-estimation visibility rays */
  uint64_t paths;          /* pixel samples */
  float ms;                /* device time of the render (CUDA events) */
  float merge_ms;          /* VCM: device time of the merge gather (grid walk + pair evaluation) */
  uint64_t merges;         /* VCM: (eye vertex, photon) pairs merged; PhotonMap: photons stored */
  uint64_t merge_queries;  /* VCM: eye vertices that queried the photon grid */
  uint64_t photons;        /* VCM, PhotonMap: photons stored in the grids, all iterations */
} rx_render_stats;

/* ---- context ------------------------------------------------------------------- */
/* Replaces the process-global GPU state of IntersectionGPU::init
 * (reference src/IntersectionGPU.cpp:16-44). */
rx_status rx_create(rx_context** out, int device);
void rx_destroy(rx_context* ctx);
const char* rx_last_error(const rx_context* ctx);
/* Build identification string (kernels, architecture). */
const char* rx_version(void);

/* ---- scene --------------------------------------------------------------------- */
/* Scene::buildKDTree's input (reference src/Scene.cpp:248-285): world-space vertices
 * of all objects concatenated, triangle vertex-index triples (global), and per
 * triangle its ObjSourceInformation {objID, triangleID} (reference include/Scene.h:13-17).
 * vnormals_xyz may be NULL (face normals everywhere). */
rx_status rx_scene_set_geometry(rx_context* ctx, const float* verts_xyz, uint32_t nv, const uint32_t* tri_vidx,
                                uint32_t nt, const uint32_t* tri_obj, const uint32_t* tri_local,
                                const float* vnormals_xyz);
/* Materials per object (reference ConfigManager.cpp:25-164 generateSceneObject). */
rx_status rx_scene_set_objects(rx_context* ctx, const rx_object* objs, uint32_t nobj);
/* KDTree::build (reference src/KDTree.cpp:230-246, include/KDTree.h:54): builds the
 * reference-order tree (tie ranks, visibility boxes) and the device BVH, uploads both. */
rx_status rx_build_accel(rx_context* ctx, const rx_build_options* opts);
/* Tree statistics: [0] BVH nodes, [1] BVH depth, [2] reference nodes,
 * [3] reference depth, [4] triangles, [5] reference leaves, [6] 4-wide BVH depth,
 * [7] 8-wide BVH depth. */
rx_status rx_accel_stats(rx_context* ctx, int64_t out[8]);
/* KDTree::serializeForGPU (reference include/KDTree.h:56, src/KDTree.cpp:346-382) of
 * the reference-order tree this library builds, host only (no device, no context).
 * nodes12: 12 floats per node (parent, rightChild, leafStart, leafEnd, min.xyz, 0,
 * max.xyz, 0); leaf_tid: triangle id per leaf slot. Pass NULL outputs to query
 * *num_nodes and *num_leaf_tris; with outputs, their capacities are read from the same
 * two counters and must suffice. */
rx_status rx_reftree_serialize(const float* verts_xyz, uint32_t nv, const uint32_t* tri_vidx, uint32_t nt,
                               int32_t split_policy, float* nodes12, uint32_t* num_nodes, float* leaf_tid,
                               uint32_t* num_leaf_tris);

/* ---- scene files ------------------------------------------------------------------ */
/* What a config file asks for (ConfigManager::load, reference src/ConfigManager.cpp:166-405). */
typedef struct rx_config_info {
  char renderer[32];       /* <Renderer><type> as written ("PT", "PTtest", "VCM", ...) */
  int32_t estimator;       /* 0 PathTracer, 1 PathTracerTest, 2 VCMTracer, 3 BidirectionalPathTracer,
                              4 PhotonMap, -1 other */
  uint32_t max_depth;      /* <maxDepth>, default 20 (MCRenderer) */
  uint32_t spp;            /* <spp>, 0 if absent */
  float radius;            /* <radius> (VCM merge radius), 0 if absent */
  double runtime_s;        /* <time> hours and minutes, in seconds */
  uint32_t num_objects, num_triangles;
  rx_camera camera;        /* the <Camera> the config names */
  char save_path[256];     /* <savePath>, empty if absent */
} rx_config_info;

typedef struct rx_host_scene rx_host_scene;
/* Reads a config file, its scene file(s) and meshes (OBJ / .shp) into host arrays, the
 * geometry Scene::buildKDTree would see (objects concatenated, world space) and the
 * object table of ConfigManager::generateSceneObject. No device, no context. err
 * (optional) receives a message on failure. */
rx_status rx_config_read(const char* config_path, rx_host_scene** out, rx_config_info* info, char* err,
                         size_t err_len);
void rx_host_scene_free(rx_host_scene* scene);
/* Views of a host scene's arrays (valid until rx_host_scene_free); *vnormals is NULL when
 * no mesh has vertex normals. Any output pointer may be NULL. */
rx_status rx_host_scene_arrays(const rx_host_scene* scene, const float** verts_xyz, uint32_t* nv,
                               const uint32_t** tri_vidx, uint32_t* nt, const uint32_t** tri_obj,
                               const uint32_t** tri_local, const float** vnormals_xyz, const rx_object** objs,
                               uint32_t* nobj);
/* rx_config_read, then rx_scene_set_geometry and rx_scene_set_objects on ctx (call
 * rx_build_accel next). */
rx_status rx_scene_load_config(rx_context* ctx, const char* config_path, rx_config_info* info);
/* MCRenderer::saveImagePFM (reference src/MCRenderer.cpp:556-574): width*height*3 RGB
 * values, rows from the top, written as a little-endian PFM with rows from the bottom. */
rx_status rx_write_pfm(const char* path, uint32_t width, uint32_t height, const double* rgb);

/* Time-stamped convergence snapshots (MCRenderer::showCurrentResult with time and
 * iteration, reference src/MCRenderer.cpp:465-490, called every timeStep seconds from
 * the renderers' loops, e.g. src/PathTracer.cpp:75-82). With every_s > 0 and fn set,
 * the next rx_render_pt (single scene), rx_render_vcm, rx_render_bpt and rx_render_pm
 * calls invoke fn after the pass or iteration during which the elapsed wall time
 * reached each next multiple of every_s: elapsed_s, samples = samples per pixel (path
 * tracing: paths done / pixels) or iterations done, and the running mean so far as
 * width*height*3 RGB values, rows from the top, valid during the call. The render
 * waits for the device before each snapshot. every_s = 0 or fn = NULL turns them off. */
typedef void (*rx_snapshot_fn)(void* user, double elapsed_s, double samples, const double* film_rgb, uint32_t width,
                               uint32_t height);
rx_status rx_set_snapshots(rx_context* ctx, double every_s, rx_snapshot_fn fn, void* user);

/* ---- closest hit --------------------------------------------------------------- */
/* KDTree::intersect(ray, triangleID, NULL) (reference include/KDTree.h:50,
 * src/KDTree.cpp:335-339) over a batch, host buffers: out_tid[i] = global triangle id
 * or -1, out_dist[i] = hit distance or -1. The rays go to the device in chunks that ramp
 * up to rx_trace_set_staging's size (2^22 by default) through three device slots: the
 * copies in and out overlap other chunks' kernels, and each slot's kernels run on a
 * stream of their own. Returns when the answers are in host memory (page-locked host
 * buffers give the full copy rate). */
rx_status rx_trace_closest(rx_context* ctx, const rx_ray* rays, uint32_t n, int32_t* out_tid, float* out_dist);
/* Same on device buffers (no copies), enqueued on `stream` (a cudaStream_t, NULL for
 * the context's stream). */
rx_status rx_trace_closest_device(rx_context* ctx, const rx_ray* d_rays, uint32_t n, int32_t* d_tid,
                                  float* d_dist, void* stream);
/* Same answers as rx_trace_closest_device, for callers that cannot allocate device
 * memory while they trace (a host whose device memory belongs to its own pool
 * allocator, or a latency-sensitive loop that must not pay cudaMalloc's implicit
 * synchronisation). No counterpart in the reference. It calls no cudaMalloc/cudaFree:
 * its scratch (winner leaves, re-walk queue, counters) is one fixed device array of
 * 8 MiB that every GPU loading the library holds until exit. At most 1048576 rays
 * per call; larger batches are rejected with RX_ERR_INVALID. The first call on a
 * device looks up the array's device address with that device current; make that
 * first call before any stream capture. All calls share the one array: calls whose
 * work overlaps on the GPU (other streams, other contexts on the device) race on it
 * and must be serialised by the caller. The array's address is that of the device's
 * primary context, valid until cudaDeviceReset. Calls are not counted in
 * rx_trace_counters. Requires a built accelerator. */
rx_status rx_trace_closest_noalloc(rx_context* ctx, const rx_ray* d_rays, uint32_t n, int32_t* d_tid,
                                   float* d_dist, void* stream);
/* Same semantics, without the BVH: walks every triangle the reference tree lets the
 * ray see, in the reference's own order (slow; a consistency check on small scenes). */
rx_status rx_trace_closest_reforder_device(rx_context* ctx, const rx_ray* d_rays, uint32_t n, int32_t* d_tid,
                                           float* d_dist, void* stream);
/* ---- rendering ------------------------------------------------------------------ */
/* MCRenderer::renderPixels(const Camera&) of PathTracer (reference
 * src/PathTracer.cpp:6-89) or PathTracerTest (src/PathTracerTest.cpp:7-86) for a fixed
 * sample count: film_rgb receives width*height*3 doubles, the per-pixel mean radiance,
 * rows from the top (the order of renderPixels' vector<vec3f>). film_sq (optional)
 * receives the per-pixel mean of squared sample values, for standard errors. Needs
 * rx_scene_set_objects before rx_build_accel. */
rx_status rx_render_pt(rx_context* ctx, const rx_camera* cam, const rx_pt_options* opts, double* film_rgb,
                       double* film_sq, rx_render_stats* stats);

/* Many scenes in one wavefront (no reference counterpart: the reference renders one
 * scene per Renderer): every item's paths share the pass queues; paths of uneven
 * length compact away per bounce. Each item's image equals what rx_render_pt gives for
 * the same options (up to the summation order of the FP64 film). ctx supplies the
 * stream and device; every item's scene must live on the same device.
 * Guided items (RX_PT_GUIDED) each use the network of their scene's context (items
 * sharing a context share it) with that context's guide options; all networks warm up,
 * train and guide on the same schedule of passes, because every pass then takes an equal
 * share of each item's samples (each item's image is still unbiased; with guided items
 * the pass order, and so the random numbers, differ from rx_render_pt's). Inference runs
 * grouped: the live paths sorted by network, each network's rows through its own weights;
 * each network trains on its own scene's records. */
rx_status rx_render_pt_batch(rx_context* ctx, const rx_batch_item* items, uint32_t n, rx_batch_options* opts,
                             rx_render_stats* stats);

/* VCMTracer::renderPixels (reference src/VCMTracer.cpp:6-143) for a fixed number of
 * iterations: film_rgb receives the running mean of the vignetting-corrected
 * iteration images (width*height*3 doubles, rows from the top). Light-path and
 * merge normalisation use light_paths (width*height in the reference). */
rx_status rx_render_vcm(rx_context* ctx, const rx_camera* cam, const rx_vcm_options* opts, double* film_rgb,
                        rx_render_stats* stats);
/* Replaces BidirectionalPathTracer::renderPixels (reference
 * src/BidirectionalPathTracer.cpp:6-112): the running mean of `iterations` images, each
 * from one eye and one light subpath per pixel joined by every (s, t) connection,
 * weighted by connectWeight (balance heuristic, no merging), with light-tracing splats
 * and the vignetting correction. Output as rx_render_vcm. */
rx_status rx_render_bpt(rx_context* ctx, const rx_camera* cam, const rx_bpt_options* opts, double* film_rgb,
                        rx_render_stats* stats);
/* Replaces PhotonMap::renderPixels (reference src/Photonmap.cpp:12-138): the running mean
 * of `iterations` progressive photon-mapping images (surface gather at the first random
 * eye vertex, ray-marched gather through homogeneous media with each medium's
 * step_size). Output as rx_render_vcm. */
rx_status rx_render_pm(rx_context* ctx, const rx_camera* cam, const rx_pm_options* opts, double* film_rgb,
                       rx_render_stats* stats);

/* Closest-hit launch shape (what the autotuner picks): variant 0 = one thread per
 * ray, 1 = persistent warps that refill finished lanes, 2 = the same with speculative
 * leaf postponing, 3 = persistent over the 4-wide BVH, 4 = 3 with the first 16 entries
 * of each walk's stack in shared memory (the default), 5 = 4 over the 8-wide BVH
 * (256-byte nodes, half the levels). 4 and 5 take the other wide tree when theirs is
 * too deep for its stack (4-wide: 21 levels, 8-wide: 11); 3 to 5 fall back to 2 when no
 * wide tree fits. Blocks of 128 threads, blocks_per_sm per SM. No reference
 * counterpart (launch tuning). */
rx_status rx_trace_set_config(rx_context* ctx, int32_t variant, int32_t blocks_per_sm);
/* Closest-hit options (no reference counterpart): check_mode = how each walk's winner
 * is checked for reference visibility, 1 = one thread per ray (default), 0 = one warp
 * per ray (one ancestor box per lane); bin_min = batches of at least this many rays are
 * reordered by origin cell and direction before the walk (counting sort), 0 = never
 * (default 262144); walk_stack = entries of the walk's stack: 0 or 32 = 32 when the
 * BVH is shallower than 32 levels, else 64 (default 0); 64 = always 64. Answers depend
 * on none of them. */
rx_status rx_trace_set_options(rx_context* ctx, int32_t check_mode, uint32_t bin_min, int32_t walk_stack);
/* Host-buffer rx_trace_closest: rays per staged chunk; chunks rotate through three
 * device slots, each with its own kernel stream, so one chunk's copies overlap other
 * chunks' kernels and the next chunk's walk fills the tail of the last. 0 = the default
 * (2^22), otherwise at least 65,536. Answers do not depend on it. No reference
 * counterpart. */
rx_status rx_trace_set_staging(rx_context* ctx, uint32_t chunk_rays);
/* Closest-hit ray binning key (no reference counterpart; launch tuning): rays are sorted
 * by the Morton code of their origin's cell on a 2^cell_bits per axis grid over the
 * scene bounds (cell_bits 3..5), then by a direction bin: dir_map 0 = each component
 * quantised to 2^dir_bits levels (dir_bits 1..3, cell_bits + dir_bits <= 7); 1 = the
 * octahedral map of the direction on a 2^dir_bits square grid in Morton order (dir_bits
 * 1..6, 3 cell_bits + 2 dir_bits <= 21). Default 4, 4, 1 (16^3 cells x 16^2 directions).
 * Answers do not depend on it. */
rx_status rx_trace_set_binning(rx_context* ctx, int32_t cell_bits, int32_t dir_bits, int32_t dir_map);
/* Per-kernel device timing of rx_trace_closest_device calls: the next max_calls calls
 * record CUDA events around their three kernels (walk, reference-visibility check,
 * re-walk of rejected winners); 0 turns timing off. No reference counterpart
 * (measurement). */
rx_status rx_trace_set_timing(rx_context* ctx, int32_t max_calls);
/* ms3[3*i + j]: device milliseconds of kernel j in recorded call i (waits for the
 * events); *calls = number of recorded calls. ms3 may be NULL to query the count. */
rx_status rx_trace_read_timing(rx_context* ctx, float* ms3, int32_t* calls);
/* Rays whose lazy winner failed the reference-visibility check and were re-traced
 * exactly, counted since the last reset (diagnostic). */
rx_status rx_trace_counters(rx_context* ctx, uint64_t out[4], int reset);

/* ---- learned guiding ------------------------------------------------------------- */
/* Creates (or re-creates) the context's guiding network with seeded weights. box6 = the
 * position-encoding box {min xyz, max xyz}; NULL takes the bounds of the scene geometry.
 * Records everywhere below are 16 floats: position, shading normal, outgoing direction,
 * incident direction, weight (integrand / sampling density), 3 unused. */
rx_status rx_guide_init(rx_context* ctx, const rx_guide_options* opts, const float* box6);
/* FP32 master parameters, 21504 floats: layer l's [out][in] row-major block at
 * {0, 5120, 9216, 13312, 17408}, widths in = {80, 64, 64, 64, 64}, 64 rows each (the last
 * layer's rows 40..63 are zero). set_params also resets the Adam moments. */
rx_status rx_guide_get_params(rx_context* ctx, float* params);
rx_status rx_guide_set_params(rx_context* ctx, const float* params);
/* Forward pass (inference kernel) on n host records: raw40 (n x 40, optional) = the
 * network outputs; pdf (n, optional) = the mixture density of each record's incident
 * direction. */
rx_status rx_guide_eval(rx_context* ctx, const float* recs, uint32_t n, float* raw40, float* pdf);
/* The same on device buffers (16-byte aligned records), enqueued on `stream` (NULL: the
 * context's stream); d_raw40 / d_pdf may each be NULL. */
rx_status rx_guide_eval_device(rx_context* ctx, const float* d_recs, uint32_t n, float* d_raw40, float* d_pdf,
                               void* stream);
/* Gradient (training kernel, no update) of the batch loss
 * -sum_s w_s log q(wi_s) / sum_s w_s (weights clipped at 32 x their mean) over n host
 * records: grad receives 21504 floats, *loss the loss. */
rx_status rx_guide_gradient(rx_context* ctx, const float* recs, uint32_t n, float* grad, float* loss);
/* One Adam step on n device records (16-byte aligned), enqueued on `stream`; with loss
 * non-NULL waits and returns the batch loss. */
rx_status rx_guide_train_step(rx_context* ctx, const float* d_recs, uint32_t n, float* loss, void* stream);

/* ---- diagnostics ---------------------------------------------------------------- */
/* Tensor-core operand-layout self-test (no reference counterpart): D = A * B^T with A
 * M x K and B N x K row-major BF16 host arrays, through one CTA's tcgen05 MMAs with FP32
 * accumulation in tensor memory. a_mn / b_mn stage A / B in the MN-major instead of the
 * K-major shared-memory view. d_out (host) receives all 128 tensor-memory lanes x N
 * columns, zero where the accumulator does not reach. M is 64 or 128, N 16..128 and K
 * 16..128, both in steps of 16. */
rx_status rx_diag_umma_gemm(rx_context* ctx, uint32_t M, uint32_t N, uint32_t K, int32_t a_mn, int32_t b_mn,
                            const uint16_t* a_bf16, const uint16_t* b_bf16, float* d_out);
/* Tensor-core issue rate (no reference counterpart): `count` back-to-back BF16 MMAs of
 * M = 128, K = 16 and N = 64, 128 or 256 (the guiding network's layers are N = 64) issued
 * by one thread of one CTA; returns SM clock cycles per MMA to the last issue and to the
 * completion of all (the second launch of two). count 1..4096. */
rx_status rx_diag_umma_rate(rx_context* ctx, uint32_t N, uint32_t count, double* issue_clk, double* done_clk);

#ifdef __cplusplus
}
#endif
#endif /* RENDERX_H */
