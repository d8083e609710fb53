// Wavefront path tracing: the reference's PathTracer (BSDF sampling only,
// src/PathTracer.cpp:19-69) and PathTracerTest (next-event estimation with
// balance-heuristic MIS, src/PathTracerTest.cpp:7-136) estimators over the bounce loop
// of MCRenderer::samplePathIter (src/MCRenderer.cpp:151-267).
//
// Stages per bounce, each a grid-stride kernel whose work count lives in device memory
// (no host round trip inside a pass): extend (closest legal hit), shade (emission,
// material scatter, next-event estimation with an inline shadow ray, Russian
// roulette) with queue compaction by warp ballot + one atomic per warp. Film
// accumulation is FP64.
#include <algorithm>
#include <cstring>
#include <vector>

#include "rx_internal.h"
#include "rx_pt.cuh"

namespace rx {

struct CamDev {
  F3 pos, front, right, up;
  float sight;
  int width, height;
};

struct PtParams {
  CamDev cam;
  uint64_t seed;
  uint32_t max_depth;
  uint32_t rr_mode;  // 0: reference RR at every bounce, 1: RR from depth 3 on
  uint32_t nee;      // 0: PathTracer, 1: PathTracerTest
  uint32_t pixels;
  uint64_t path_base;
  uint32_t npaths;
};

// Path state, structure of arrays (one slot per live path).
struct PathSoA {
  float4* o;     // origin, w = pdf of the sampled direction (MIS)
  float4* d;     // direction, w = unused
  float4* T;     // throughput, w = unused
  float4* L;     // accumulated radiance, w = unused
  int4* info;    // pixel, contact object, inside object, depth | last-specular << 8
  uint64_t* id;  // path id (random-number key)
};

// -------------------------------------------------------------------------------------
// Camera (reference src/Camera.cpp:4-47, 78-96)
// -------------------------------------------------------------------------------------
__device__ __forceinline__ F3 camera_dir(const CamDev& c, float xp, float yp) {
  float x = xp - c.width * 0.5f, y = c.height * 0.5f - yp;
  return normalize(c.front * c.sight + c.right * x + c.up * y);
}

__global__ void k_generate(PtParams P, PathSoA S, unsigned* count) {
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.npaths; i += stride) {
    uint64_t pid = P.path_base + i;
    uint32_t pixel = (uint32_t)(pid % P.pixels);
    int x = pixel % P.cam.width, y = pixel / P.cam.width;
    Rng rng(P.seed, pid, 0);
    float jx = rng.next(), jy = rng.next();
    F3 d = camera_dir(P.cam, x + jx, y + jy);
    float w = 1.0f;
    if (!P.nee) {
      // camera ray's cosine term (Camera::getWorldNormal = front, Ray::getCosineTerm)
      // over the pixel-centre cosine of eliminateVignetting
      F3 dc = camera_dir(P.cam, x + 0.5f, y + 0.5f);
      w = fmaxf(fabsf(dot(P.cam.front, d)), 1e-6f) / fabsf(dot(dc, P.cam.front));
    }
    S.o[i] = make_float4(P.cam.pos.x, P.cam.pos.y, P.cam.pos.z, 1.0f);
    S.d[i] = make_float4(d.x, d.y, d.z, 0.0f);
    S.T[i] = make_float4(w, w, w, 0.0f);
    S.L[i] = make_float4(0, 0, 0, 0);
    S.info[i] = make_int4((int)pixel, -1, -1, 1 << 8);
    S.id[i] = pid;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = P.npaths;
}

__global__ void __launch_bounds__(128) k_extend(DevScene SC, PathSoA S, const unsigned* count, int2* hit,
                                                unsigned long long* rays) {
  uint32_t n = *count;
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float4 o = S.o[i], d = S.d[i];
    int4 inf = S.info[i];
    bool camera = (inf.w & 255) == 0;
    PHit h = trace_cond<false>(SC, f3(o), f3(d), INFINITY, camera ? -1 : inf.y, camera ? -1 : inf.z);
    hit[i] = make_int2(h.tid, __float_as_int(h.t));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rays, (unsigned long long)n);
}

// -------------------------------------------------------------------------------------
// Materials
// -------------------------------------------------------------------------------------
struct Scatter {
  F3 dir, color;
  float prob;
  bool definite;  // Ray::DEFINITE (specular / pass-through)
  bool killed;    // direction of length 0: the path ends here
  int inside, contact;
};

__device__ __forceinline__ F3 refl(F3 n, F3 d) { return n * (-dot(n, d) * 2.0f) + d; }

// DiffuseMaterial::scatter, src/DiffuseMaterial.cpp:4-77
__device__ Scatter scatter_diffuse(F3 color, F3 n, F3 din, int obj, int inside, bool russian, Rng& rng) {
  Scatter s;
  s.inside = inside;
  s.contact = obj;
  s.killed = false;
  if (dot(din, n) > 0.0f) {  // leaving: pass through
    s.dir = din;
    s.color = {1, 1, 1};
    s.prob = 1.0f;
    s.definite = true;
    return s;
  }
  Frame f = frame_from(n);
  float r1 = rng.next(), r2 = rng.next();
  s.dir = to_world(f, hemi_cos(1.0f, r1, r2));
  float p = maxc(color);
  s.definite = false;
  if (!russian || rng.next() < p) {
    bool ok = dot(n, din) <= 0.0f && dot(n, s.dir) >= 0.0f;  // DiffuseBSDF::evaluate
    s.color = ok ? color * (1.0f / RX_PI) : F3{0, 0, 0};
    float pdf = cos_lobe_pdf(n, s.dir, 1.0f);
    s.prob = russian ? p * pdf : pdf;
  } else {
    s.dir = {0, 0, 0};
    s.color = {0, 0, 0};
    s.prob = 1.0f - p;
    s.killed = true;
  }
  return s;
}

// GlossyMaterial::scatter, src/GlossyMaterial.cpp:4-57 (Phong lobe, no (n+2)/2pi
// normalisation, GlossyBSDF.h:24-33)
__device__ Scatter scatter_glossy(F3 color, float coeff, F3 n, F3 din, int obj, int inside, bool russian, Rng& rng) {
  Scatter s;
  s.inside = inside;
  s.contact = obj;
  s.definite = false;
  s.killed = false;
  F3 r = refl(n, din);
  Frame f = frame_from(r);
  float r1 = rng.next(), r2 = rng.next();
  s.dir = to_world(f, hemi_cos(coeff, r1, r2));
  F3 c = {0, 0, 0};
  if (dot(n, din) <= 0.0f && dot(n, s.dir) >= 0.0f) {
    float rw = dot(r, s.dir);
    if (rw > 0.0f) c = color * powf(rw, coeff);
  }
  s.color = c;
  s.prob = cos_lobe_pdf(r, s.dir, coeff);
  float p = maxc(color);
  if (c.x == 0.0f && c.y == 0.0f && c.z == 0.0f) {
    s.dir = {0, 0, 0};
    s.prob = 1.0f;
    s.killed = true;
    return s;
  }
  if (!russian) return s;
  if (rng.next() < p) {
    s.prob *= p;
  } else {
    s.dir = {0, 0, 0};
    s.color = {0, 0, 0};
    s.prob = 1.0f - p;
    s.killed = true;
  }
  return s;
}

// RefractiveMaterial::scatter, src/RefractiveMaterial.cpp:132-269: unpolarised Fresnel
// choice between mirror reflection and Snell refraction (rotMat(n x d, phi) * n is the
// rotation of n toward d by phi), total internal reflection ends the path, the
// (n_i/n_t)^2 radiance scaling on eye paths. cos_out: |n . dir| as
// Ray::getCosineTerm, clamped at 1e-6.
__device__ Scatter scatter_refractive(F3 surf, float ior, F3 n, F3 din, int obj, int inside, float cur_n, float next_n,
                                      int outside, bool light_path, Rng& rng) {
  Scatter s;
  s.contact = obj;
  s.definite = true;
  s.killed = false;
  s.inside = inside;
  F3 r = refl(n, din);
  if (ior < 0.0f) {  // mirror (SceneReflectiveObject)
    s.dir = r;
    s.prob = 1.0f;
    s.color = surf * (1.0f / fmaxf(fabsf(dot(n, r)), 1e-6f));
    return s;
  }
  float cd = fminf(fmaxf(dot(din, n), -1.0f), 1.0f);
  float theta = acosf(cd);
  float sin_phi = cur_n / next_n * sinf(theta);
  if (sin_phi >= 1.0f) {  // total internal reflection kills the path
    s.dir = {0, 0, 0};
    s.color = {0, 0, 0};
    s.prob = 1.0f;
    s.killed = true;
    s.contact = -1;
    return s;
  }
  float phi = asinf(sin_phi);
  if (theta > RX_PI * 0.5f) phi = RX_PI - phi;
  F3 tp = normalize(din - n * cd);
  float sp, cp;
  sincosf(phi, &sp, &cp);
  F3 wt = normalize(n * cp + tp * sp);
  float ct = fabsf(cosf(theta)), cph = fabsf(cp);
  float a = fabsf(cur_n * ct - next_n * cph) / (cur_n * ct + next_n * cph);
  float b = fabsf(next_n * ct - cur_n * cph) / (next_n * ct + cur_n * cph);
  float er = (a * a + b * b) * 0.5f;
  float p = fminf(fmaxf(er, 0.0f), 1.0f);
  if (rng.next() < p) {
    s.dir = normalize(r);
    s.color = surf * (er / fmaxf(fabsf(dot(n, r)), 1e-6f));
    s.prob = p;
  } else {
    F3 c = surf;
    if (!light_path) c = c * ((cur_n * cur_n) / (next_n * next_n));
    s.color = c * ((1.0f - er) / fmaxf(fabsf(dot(n, wt)), 1e-6f));
    s.prob = 1.0f - p;
    s.inside = outside;
    s.dir = wt;
  }
  return s;
}

// BSDF value and sampling pdf for a connection (SceneObject::getBSDF sums the
// materials, getDirectionSampleProbDensity averages them; SceneObject.cpp:323-359).
// Glossy's getBSDF carries an extra factor max(colour) (GlossyMaterial.cpp:207-217);
// diffuse's pdf includes its roulette factor (DiffuseMaterial.cpp:79-87).
__device__ void bsdf_eval(const DevObject& ob, F3 n, F3 din, F3 wo, F3& f, float& pdf) {
  f = {0, 0, 0};
  pdf = 0.0f;
  bool front = dot(n, din) <= 0.0f && dot(n, wo) >= 0.0f;
  int nm = 0;
  if (ob.material == kDiffuse || ob.material == kPhong) {
    F3 c = ob.material == kPhong ? f3v(ob.diffuse_color) : f3v(ob.color);
    if (front) f = f + c * (1.0f / RX_PI);
    pdf += maxc(c) * cos_lobe_pdf(n, wo, 1.0f);
    nm++;
  }
  if (ob.material == kGlossy || ob.material == kPhong) {
    F3 c = f3v(ob.color);
    F3 r = refl(n, din);
    if (front) {
      float rw = dot(r, wo);
      if (rw > 0.0f) f = f + c * (maxc(c) * powf(rw, ob.coeff));
    }
    pdf += cos_lobe_pdf(r, wo, ob.coeff);
    nm++;
  }
  if (nm > 1) pdf /= (float)nm;
}

// -------------------------------------------------------------------------------------
// Shade: one bounce of MCRenderer::samplePathIter plus the estimator's bookkeeping.
// -------------------------------------------------------------------------------------
__device__ __forceinline__ void film_add(double* sum, double* sq, int pixel, F3 L) {
  double* s = sum + 3 * (size_t)pixel;
  double* q = sq + 3 * (size_t)pixel;
  atomicAdd(s, (double)L.x);
  atomicAdd(s + 1, (double)L.y);
  atomicAdd(s + 2, (double)L.z);
  if (q) {
    atomicAdd(q, (double)L.x * L.x);
    atomicAdd(q + 1, (double)L.y * L.y);
    atomicAdd(q + 2, (double)L.z * L.z);
  }
}

__device__ __forceinline__ F3 decay_of(const DevScene& SC, int inside, float t) {
  if (inside < 0) return {1, 1, 1};
  const DevObject& ob = SC.objects[inside];
  if (ob.material == kRefractive) {  // RefractiveMaterial::getRadianceDecay: decay^dist
    return {powf(ob.decay[0], t), powf(ob.decay[1], t), powf(ob.decay[2], t)};
  }
  if (ob.material == kVPM) {  // SceneVPMObject: exp(-sigma_t d) per channel
    return {expf(-(ob.sigma_s[0] + ob.sigma_a[0]) * t), expf(-(ob.sigma_s[1] + ob.sigma_a[1]) * t),
            expf(-(ob.sigma_s[2] + ob.sigma_a[2]) * t)};
  }
  return {1, 1, 1};
}

__global__ void __launch_bounds__(128) k_shade(DevScene SC, PtParams P, PathSoA S, const unsigned* count,
                                               const int2* hit, PathSoA N, unsigned* next_count, double* film_sum,
                                               double* film_sq, unsigned long long* shadow_rays) {
  uint32_t n = *count;
  uint32_t stride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  unsigned shadows = 0;
  // every lane of a warp walks the same number of iterations (ballots need all 32)
  uint32_t nwarp_iter = (n + stride - 1) / stride;
  for (uint32_t it = 0; it < nwarp_iter; it++) {
    uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    bool live = i < n, cont = false;
    float4 o4, d4, T4, L4;
    int4 inf;
    F3 xo{}, wo{}, T{}, L{};
    float pdf_out = 1.0f;
    int contact_out = -1, inside_out = -1, depth = 0;
    bool spec_out = true;
    uint64_t pid = 0;
    if (live) {
      o4 = S.o[i];
      d4 = S.d[i];
      T4 = S.T[i];
      L4 = S.L[i];
      inf = S.info[i];
      pid = S.id[i];
      depth = inf.w & 255;
      bool last_spec = (inf.w >> 8) & 1;
      int inside = inf.z;
      T = f3(T4);
      L = f3(L4);
      F3 o = f3(o4), d = f3(d4);
      int2 h = hit[i];
      Rng rng(P.seed, pid, 16u + 32u * (uint32_t)depth);
      bool done = true;
      if (h.x >= 0) {
        float t = __int_as_float(h.y);
        F3 x = o + d * t;
        TriGeom g = tri_geom(SC, h.x);
        int hit_obj = g.obj;
        F3 dec = decay_of(SC, inside, t);
        if (!P.nee) T = T * dec;
        int sobj = inside >= 0 ? inside : hit_obj;  // samplePathIter: the inside object scatters
        const DevObject& ob = SC.objects[sobj];
        const DevObject& hob = SC.objects[hit_obj];
        if (ob.material == kEmissive) {
          F3 fn = world_normal(g, ob.has_normals, x);
          F3 Le = f3v(ob.color);
          if (!P.nee) {
            // SceneEmissiveObject::scatter: emitted only toward the front
            if (dot(d, fn) <= 0.0f) L = L + T * Le;
          } else {
            // PathTracerTest.cpp:37-56: two-sided, MIS against light sampling
            float mis = 1.0f;
            if (depth > 0 && !last_spec) {
              float cosine = dot(fn, -d);
              float pdfw = (1.0f / SC.light_area) * t * t / fabsf(cosine);
              mis = o4.w / (o4.w + pdfw);
            }
            L = L + T * Le * mis;
          }
        } else {
          F3 ns = world_normal(g, hob.has_normals, x);  // shading normal at the hit
          bool russian = P.rr_mode == 0 || depth >= 3;
          Scatter sc;
          uint32_t kind = ob.material;
          if (kind == kPhong) kind = rng.next() < 0.5f ? kGlossy : kDiffuse;  // rand()%2, SceneObject.cpp:373-380
          if (kind == kDiffuse) {
            F3 c = ob.material == kPhong ? f3v(ob.diffuse_color) : f3v(ob.color);
            sc = scatter_diffuse(c, ns, d, sobj, inside, russian, rng);
          } else if (kind == kGlossy) {
            sc = scatter_glossy(f3v(ob.color), ob.coeff, ns, d, sobj, inside, russian, rng);
          } else {
            // refractive / reflective / medium boundary
            bool going_out = inside == sobj;
            int outside = going_out ? -1 : sobj;  // findInsideObject: no enclosing volume
            float cur_n = inside >= 0 ? fabsf(SC.objects[inside].ior) : 1.0f;
            if (inside >= 0 && SC.objects[inside].material != kRefractive && SC.objects[inside].material != kVPM)
              cur_n = 1.0f;
            float next_n = outside >= 0 ? fabsf(SC.objects[outside].ior) : 1.0f;
            sc = scatter_refractive(f3v(ob.color), ob.material == kReflective ? -1.0f : ob.ior, ns, d, sobj, inside,
                                    cur_n, next_n, outside, false, rng);
          }
          // shading-normal light-leak kill, MCRenderer.cpp:183-217
          if (!sc.killed && sc.inside < 0 && sc.contact >= 0) {
            F3 fl = world_normal(g, hob.has_normals, x, true);
            F3 wi = -d;
            if (dot(ns, wi) * dot(fl, wi) <= 0.0f || dot(ns, sc.dir) * dot(fl, sc.dir) <= 0.0f) {
              sc.dir = {0, 0, 0};
              sc.color = {0, 0, 0};
              sc.killed = true;
            }
          }
          bool capped = !sc.killed && depth + 1 > (int)P.max_depth;
          if (P.nee && !sc.definite && !capped && SC.num_lights > 0) {
            // PathTracerTest::colorByConnectingLights, PathTracerTest.cpp:88-136
            float ru = rng.next() * SC.light_area;
            int lo = 0, hi = (int)SC.num_lights - 1;
            while (lo < hi) {
              int mid = (lo + hi) >> 1;
              if (__ldg(&SC.light_cdf[mid]) < ru) lo = mid + 1;
              else hi = mid;
            }
            int lt = (int)__ldg(&SC.light_tri[lo]);
            TriGeom lg = tri_geom(SC, lt);
            float u1 = rng.next(), u2 = rng.next();
            float su1 = sqrtf(u1);
            float bu = 1.0f - su1, bv = u2 * su1;
            F3 xl = lg.v0 * bu + lg.v1 * bv + lg.v2 * (1.0f - bu - bv);
            F3 ld = x - xl;
            float dist = length(ld);
            ld = ld * (1.0f / dist);
            F3 wl = -ld;
            F3 f;
            float bpdf;
            bsdf_eval(ob, ns, d, wl, f, bpdf);
            F3 nl = world_normal(lg, SC.objects[lg.obj].has_normals, xl);
            float cos_l = fminf(fabsf(dot(nl, ld)), 1.0f);
            if (lum(f) >= 1e-7f && cos_l >= 1e-6f) {
              shadows++;
              PHit sh = trace_cond<true>(SC, x, wl, dist - 1e-5f, sc.contact, sc.inside);
              if (sh.tid < 0) {
                float cos_s = fminf(fabsf(dot(ns, wl)), 1.0f);
                float pdfa = 1.0f / SC.light_area;
                float pdfw = pdfa * dist * dist / cos_l;
                float mis = pdfw / (pdfw + bpdf);
                F3 Le = f3v(SC.objects[lg.obj].color);
                L = L + T * Le * f * (cos_l * cos_s / (pdfa * dist * dist) * mis);
              }
            }
          }
          if (!sc.killed && !capped) {
            float cos_o = fmaxf(fabsf(dot(ns, sc.dir)), 1e-6f);  // Ray::getCosineTerm
            T = T * sc.color * (cos_o / sc.prob);
            if (P.nee) T = T * dec;  // PathTracerTest applies the previous segment's decay here
            xo = x;
            wo = sc.dir;
            pdf_out = sc.prob;
            spec_out = sc.definite;
            contact_out = sc.contact;
            inside_out = sc.inside;
            done = false;
          }
        }
      }
      if (done) {
        if (L.x != 0.0f || L.y != 0.0f || L.z != 0.0f) film_add(film_sum, film_sq, inf.x, L);
      } else {
        cont = true;
      }
    }
    // compaction: warp ballot, one atomic per warp
    unsigned m = __ballot_sync(0xffffffffu, cont);
    if (m) {
      unsigned base = 0;
      int leader = __ffs(m) - 1;
      if (lane == leader) base = atomicAdd(next_count, (unsigned)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (cont) {
        uint32_t j = base + __popc(m & ((1u << lane) - 1));
        N.o[j] = make_float4(xo.x, xo.y, xo.z, pdf_out);
        N.d[j] = make_float4(wo.x, wo.y, wo.z, 0.0f);
        N.T[j] = make_float4(T.x, T.y, T.z, 0.0f);
        N.L[j] = make_float4(L.x, L.y, L.z, 0.0f);
        N.info[j] = make_int4(inf.x, contact_out, inside_out, (depth + 1) | ((spec_out ? 1 : 0) << 8));
        N.id[j] = pid;
      }
    }
  }
  for (int s2 = 16; s2 > 0; s2 >>= 1) shadows += __shfl_xor_sync(0xffffffffu, shadows, s2);
  if (lane == 0 && shadows) atomicAdd(shadow_rays, (unsigned long long)shadows);
}

__global__ void k_zero(unsigned* p) { *p = 0; }

// -------------------------------------------------------------------------------------
// Host driver
// -------------------------------------------------------------------------------------
static cudaError_t alloc_soa(PathSoA& s, std::vector<DevBuf>& bufs, size_t n) {
  size_t sizes[6] = {16, 16, 16, 16, 16, 8};
  void** ptrs[6] = {(void**)&s.o, (void**)&s.d, (void**)&s.T, (void**)&s.L, (void**)&s.info, (void**)&s.id};
  for (int k = 0; k < 6; k++) {
    bufs.emplace_back();
    cudaError_t e = bufs.back().alloc(sizes[k] * n);
    if (e != cudaSuccess) return e;
    *ptrs[k] = bufs.back().p;
  }
  return cudaSuccess;
}

cudaError_t render_pt(rx_context* c, const rx_camera& cam, const rx_pt_options& opt, double* film_sum,
                      double* film_sq, rx_render_stats* stats, cudaStream_t s) {
  const DevScene& SC = c->scene;
  PtParams P{};
  auto v3 = [](const float* p) { return F3{p[0], p[1], p[2]}; };
  auto hn = [](F3 a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return l > 0 ? F3{a.x / l, a.y / l, a.z / l} : a;
  };
  auto hc = [](F3 l, F3 r) { return F3{l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x}; };
  F3 pos = v3(cam.position), foc = v3(cam.focus), up = v3(cam.up);
  P.cam.pos = pos;
  P.cam.front = hn(F3{foc.x - pos.x, foc.y - pos.y, foc.z - pos.z});
  P.cam.right = hn(hc(P.cam.front, up));
  P.cam.up = hc(P.cam.right, P.cam.front);
  P.cam.sight = (float)cam.sight_dist;
  P.cam.width = (int)cam.width;
  P.cam.height = (int)cam.height;
  P.seed = opt.seed;
  P.max_depth = opt.max_depth;
  P.rr_mode = opt.rr_mode;
  P.nee = opt.nee;
  P.pixels = cam.width * cam.height;
  uint64_t total = (uint64_t)P.pixels * opt.spp;
  uint32_t per_pass = opt.paths_per_pass ? opt.paths_per_pass : (1u << 21);
  per_pass = (uint32_t)std::min<uint64_t>(per_pass, total);
  if (per_pass == 0) return cudaSuccess;

  std::vector<DevBuf> bufs;
  PathSoA A{}, B{};
  cudaError_t e;
  if ((e = alloc_soa(A, bufs, per_pass)) != cudaSuccess) return e;
  if ((e = alloc_soa(B, bufs, per_pass)) != cudaSuccess) return e;
  bufs.emplace_back();
  if ((e = bufs.back().alloc(per_pass * sizeof(int2))) != cudaSuccess) return e;
  int2* hit = bufs.back().as<int2>();
  bufs.emplace_back();
  if ((e = bufs.back().alloc(64 * sizeof(unsigned long long))) != cudaSuccess) return e;
  unsigned long long* ctr = bufs.back().as<unsigned long long>();  // [0] ext rays, [1] shadow rays
  unsigned* cnt = reinterpret_cast<unsigned*>(ctr + 8);            // two queue counts
  cudaMemsetAsync(ctr, 0, 64 * sizeof(unsigned long long), s);

  int grid = c->trace_cfg.sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  for (uint64_t base = 0; base < total; base += per_pass) {
    P.path_base = base;
    P.npaths = (uint32_t)std::min<uint64_t>(per_pass, total - base);
    PathSoA* cur = &A;
    PathSoA* nxt = &B;
    unsigned* ccur = cnt;
    unsigned* cnxt = cnt + 1;
    k_generate<<<grid, 256, 0, s>>>(P, *cur, ccur);
    for (uint32_t depth = 0; depth <= opt.max_depth; depth++) {
      k_extend<<<grid, 128, 0, s>>>(SC, *cur, ccur, hit, ctr);
      k_zero<<<1, 1, 0, s>>>(cnxt);
      k_shade<<<grid, 128, 0, s>>>(SC, P, *cur, ccur, hit, *nxt, cnxt, film_sum, film_sq, ctr + 1);
      std::swap(cur, nxt);
      std::swap(ccur, cnxt);
    }
  }
  cudaEventRecord(e1, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (stats) {
    unsigned long long h[2];
    cudaMemcpy(h, ctr, sizeof h, cudaMemcpyDeviceToHost);
    stats->extension_rays = h[0];
    stats->shadow_rays = h[1];
    stats->paths = total;
    stats->ms = ms;
  }
  return cudaSuccess;
}

}  // namespace rx
