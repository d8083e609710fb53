// ORACLE — test infrastructure only. A CPU restatement of the reference's PathTracer
// estimator (reference src/PathTracer.cpp:19-69) over its bounce loop
// (MCRenderer::samplePathIter, src/MCRenderer.cpp:151-267), with the reference's own
// closest-hit traversal (rxo_tree.h: the unpruned KDTree walk, the
// NoSelfIntersectionCondition of src/NoSelfIntersectionCondition.cpp:12-27 on every
// candidate). Only tests/ and bench.py's CPU-baseline leg load it: it times the
// reference's CPU path on the host cores and checks the GPU renders statistically; the
// product never uses it.
//
// Scope: the surface materials (diffuse, glossy, Phong, dielectric, mirror, emissive) on
// scenes whose closed objects neither overlap nor nest, with the camera outside every
// object (the benchmark scenes). Homogeneous media are not restated here.
//
// Parity pin: tests/test_oracle_pt.py checks this restatement against the goldens made
// by the reference's own PathTracer (tests/golden/render_*_pt.npz) per pixel within
// 3 sigma.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rxo_tree.h"

using namespace rxo;

extern "C" {
// Material codes (the library's RX_MAT_* values).
enum { kDiffuse = 0, kGlossy = 1, kRefractive = 2, kEmissive = 3, kPhong = 4, kReflective = 5, kVpm = 6 };

typedef struct rxo_pt_object {
  uint32_t kind;
  float color[3];          // albedo / glossy colour / emission / surface colour
  float coeff;             // glossy exponent
  float diffuse_color[3];  // Phong diffuse part
  float ior;               // refractive index (< 0: mirror)
  float decay[3];          // RefractiveMaterial decay colour (per unit length)
  uint32_t has_normals;    // shading normals from vertex normals
} rxo_pt_object;

typedef struct rxo_pt_camera {
  uint32_t width, height, sight_dist, reserved;
  float position[3], focus[3], up[3];
} rxo_pt_camera;
}

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kCosTermMin = 1e-6f;  // COS_TERM_MIN, include/macros.h:9

inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 mulv(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float len(V3 a) { return std::sqrt(dot(a, a)); }
inline float maxc(V3 a) { return std::max(a.x, std::max(a.y, a.z)); }
inline V3 v3(const float* p) { return {p[0], p[1], p[2]}; }

// Per-thread random numbers (splitmix64), 24-bit floats like RNG::genFloat.
struct Rng {
  uint64_t s;
  Rng(uint64_t seed, uint64_t stream) : s(seed * 0x9E3779B97F4A7C15ull ^ (stream + 0x632BE59BD9B4E019ull)) {}
  float next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(z >> 40) * (1.0f / 16777216.0f);
  }
};

// LocalFrame::buildFromNormal / toWorld (include/LocalFrame.h:13-27).
struct Frame {
  V3 s, n, t;
};
inline Frame frame_from(V3 n) {
  V3 tmp = std::fabs(n.z) > 0.99f ? V3{1, 0, 0} : V3{0, 0, 1};
  Frame f;
  f.n = n;
  f.s = normalized(cross(n, tmp));
  f.t = normalized(cross(f.s, n));
  return f;
}
inline V3 to_world(const Frame& f, V3 a) { return add(add(mul(f.s, a.x), mul(f.n, a.y)), mul(f.t, a.z)); }

// RandGenerator::genHemiCosDirection (src/RandGenerator.cpp:152-167).
inline V3 hemi_cos(float e, Rng& rng) {
  float r1 = rng.next(), r2 = rng.next();
  float u1 = 2.0f * kPi * r1, u2 = std::pow(r2, 1.0f / (e + 1.0f)), u3 = std::sqrt(std::max(0.0f, 1.0f - u2 * u2));
  return normalized(V3{std::cos(u1) * u3, u2, std::sin(u1) * u3});
}
// CosineSphericalSampler::getProbDensity (include/CosineSphericalSampler.h:26-37).
inline float cos_pdf(V3 n, V3 dir, float e) {
  float c = std::max(dot(n, dir), 0.0f);
  return std::pow(c, e) * (e + 1.0f) / (2.0f * kPi);
}

struct Scene {
  const rxo_tree* T;
  const uint32_t* tri_obj;
  const float* vnormals;  // per vertex, or null
  const rxo_pt_object* objs;
  uint32_t nobj;
  V3 cpos, front, right, up;
  float sight;
  int width, height;
};

// SimpleShape::getWorldNormal (src/SimpleShape.cpp:393-441): the normal interpolated
// from vertex normals at `p` (objects with vertex normals), else the face normal; with
// `flat` the face normal turned to the interpolated normal's side.
V3 world_normal(const Scene& S, uint32_t t, V3 p, bool flat = false) {
  const uint32_t* tv = &S.T->tris[3 * (size_t)t];
  V3 a = S.T->verts[tv[0]], b = S.T->verts[tv[1]], c = S.T->verts[tv[2]];
  V3 b1 = sub(b, a), b2 = sub(c, a);
  V3 fn = normalized(cross(b1, b2));
  if (!S.vnormals || !S.objs[S.tri_obj[t]].has_normals) return fn;
  V3 n0 = normalized(v3(S.vnormals + 3 * (size_t)tv[0])), n1 = normalized(v3(S.vnormals + 3 * (size_t)tv[1])),
     n2 = normalized(v3(S.vnormals + 3 * (size_t)tv[2]));
  V3 v = sub(p, a);
  float d12 = dot(b1, b2), l1 = len(b1), l2 = len(b2);
  float u2 = (dot(v, b1) * d12 - dot(v, b2) * l1 * l1) / (d12 * d12 - l1 * l1 * l2 * l2);
  float u1 = (dot(v, b1) - u2 * d12) / (l1 * l1);
  V3 n = normalized(add(add(mul(n0, 1.0f - u1 - u2), mul(n1, u1)), mul(n2, u2)));
  if (flat) return dot(n, fn) < 0 ? neg(fn) : fn;
  return n;
}

constexpr int kNone = -1, kCamera = -2;

// The fields of the reference's Ray record (include/Ray.h) the estimator reads.
struct PRay {
  V3 o{0, 0, 0}, d{0, 0, 0}, color{1, 1, 1};
  float dprob = 1, oprob = 1;
  int contact = kNone, ctri = -1, inside = kNone;
  int isect = kNone, itri = -1;
  float idist = -1;
};

V3 contact_normal(const Scene& S, const PRay& r, bool flat = false) {
  if (r.contact == kCamera) return S.front;
  if (r.contact >= 0) return world_normal(S, (uint32_t)r.ctri, r.o, flat);
  return {0, 0, 0};
}

// Ray::getCosineTerm (src/Ray.cpp:72-79); every surface object and the camera have one.
float cos_term(const Scene& S, const PRay& r) {
  float d = 1.0f;
  if (r.contact != kNone && len(r.d) > 0.5f) d = std::fabs(dot(contact_normal(S, r), r.d));
  return std::max(d, kCosTermMin);
}

// Ray::getRadianceDecay (src/Ray.cpp:67-70) for refractive insides.
V3 decay_of(const Scene& S, int inside, float dist) {
  if (inside < 0) return {1, 1, 1};
  const rxo_pt_object& o = S.objs[inside];
  if (o.kind != kRefractive) return {1, 1, 1};
  return {std::pow(o.decay[0], dist), std::pow(o.decay[1], dist), std::pow(o.decay[2], dist)};
}

float refr_coeff(const Scene& S, int obj) { return obj >= 0 && S.objs[obj].kind == kRefractive ? S.objs[obj].ior : 1.0f; }

// DiffuseMaterial::scatter (src/DiffuseMaterial.cpp:4-78).
PRay scatter_diffuse(const Scene& S, int obj, V3 col, const PRay& in, bool russian, Rng& rng) {
  PRay out;
  out.o = add(in.o, mul(in.d, in.idist));
  V3 n = world_normal(S, (uint32_t)in.itri, out.o);
  out.inside = in.inside;
  out.contact = obj;
  out.ctri = in.itri;
  if (dot(in.d, n) > 0) {  // leaving: pass straight through (DEFINITE)
    out.d = in.d;
    out.dprob = 1;
    out.color = {1, 1, 1};
    return out;
  }
  out.d = to_world(frame_from(n), hemi_cos(1.0f, rng));
  float p = maxc(col);
  if (!(dot(n, out.d) >= kCosTermMin)) {
    // a direction at the hemisphere's rim (u = 0 exactly, probability 2^-24 here, zero
    // for the continuous sampler): its density falls below the cosine clamp, so the
    // weight would blow up; the path ends (as the library's sampler does)
    out.d = {0, 0, 0};
    out.color = {0, 0, 0};
    out.dprob = 1;
    return out;
  }
  if (rng.next() < p || !russian) {
    bool front = dot(n, in.d) <= 0 && dot(n, out.d) >= 0;
    out.color = front ? mul(col, 1.0f / kPi) : V3{0, 0, 0};
    out.dprob = (russian ? p : 1.0f) * cos_pdf(n, out.d, 1.0f);
  } else {
    out.d = {0, 0, 0};
    out.color = {0, 0, 0};
    out.dprob = 1 - p;
  }
  return out;
}

// GlossyMaterial::scatter (src/GlossyMaterial.cpp:4-51) with GlossyBSDF::evaluate
// (include/GlossyBSDF.h:25-33). `russian` false skips the continuation roulette (the
// roulette-from-depth-3 variant; the reference always rolls it).
PRay scatter_glossy(const Scene& S, int obj, V3 col, float e, const PRay& in, bool russian, Rng& rng) {
  PRay out;
  out.o = add(in.o, mul(in.d, in.idist));
  V3 n = world_normal(S, (uint32_t)in.itri, out.o);
  out.inside = in.inside;
  out.contact = obj;
  out.ctri = in.itri;
  V3 refl = add(mul(n, -dot(n, in.d) * 2.0f), in.d);
  Frame lf = frame_from(refl);
  out.d = to_world(lf, hemi_cos(e, rng));
  V3 c{0, 0, 0};
  if (dot(n, in.d) <= 0 && dot(n, out.d) >= 0) {
    float rw = dot(refl, out.d);
    if (rw > 0) c = mul(col, std::pow(rw, e));
  }
  out.color = c;
  out.dprob = cos_pdf(lf.n, out.d, e);
  float p = maxc(col);
  if (len(c) == 0) {
    out.d = {0, 0, 0};
    out.color = {0, 0, 0};
    out.dprob = 1;
    return out;
  }
  if (!russian) return out;
  if (rng.next() < p) {
    out.dprob *= p;
  } else {
    out.d = {0, 0, 0};
    out.color = {0, 0, 0};
    out.dprob = 1 - p;
  }
  return out;
}

PRay scatter(const Scene& S, int obj, const PRay& in, bool russian, Rng& rng);

// RefractiveMaterial::scatter (src/RefractiveMaterial.cpp:132-269): a mirror for a
// negative index, else Fresnel choice between reflection and refraction (the
// refraction direction rotates the normal towards the incident direction by the Snell
// angle), total internal reflection ends the path, (n_i / n_t)^2 on eye paths.
PRay scatter_refractive(const Scene& S, int obj, const PRay& in, Rng& rng) {
  const rxo_pt_object& ob = S.objs[obj];
  PRay out;
  out.o = add(in.o, mul(in.d, in.idist));
  V3 n = world_normal(S, (uint32_t)in.itri, out.o);
  out.color = v3(ob.color);
  out.d = in.d;
  V3 refl = add(mul(n, -dot(n, in.d) * 2.0f), in.d);
  out.contact = obj;
  out.ctri = in.itri;
  if (ob.ior < 0) {  // mirror
    out.d = refl;
    out.inside = in.inside;
    out.dprob = 1;
    out.color = mul(out.color, 1.0f / cos_term(S, out));
    return out;
  }
  if (in.isect != obj && in.inside == obj) return scatter(S, in.isect, in, true, rng);  // hit another object inside
  float theta = std::acos(std::min(1.0f, std::max(-1.0f, dot(in.d, n))));
  int outside = obj;
  if (in.inside == obj) outside = kNone;  // objects do not nest: leaving goes to the outside
  float cn = refr_coeff(S, in.inside), nn = refr_coeff(S, outside);
  out.dprob = 1;
  float sin_phi = cn / nn * std::sin(theta);
  if (sin_phi >= 1) {  // total internal reflection ends the path
    out.d = {0, 0, 0};
    out.contact = kNone;
    out.ctri = -1;
    return out;
  }
  float phi = std::asin(sin_phi);
  if (theta > kPi / 2) phi = kPi - phi;
  V3 tang = normalized(cross(normalized(cross(n, in.d)), n));  // d's direction along the surface
  out.d = normalized(add(mul(n, std::cos(phi)), mul(tang, std::sin(phi))));
  float ct = std::fabs(std::cos(theta)), cp = std::fabs(std::cos(phi));
  float esr = std::pow(std::fabs(cn * ct - nn * cp) / (cn * ct + nn * cp), 2.0f);
  float epr = std::pow(std::fabs(nn * ct - cn * cp) / (nn * ct + cn * cp), 2.0f);
  float er = (esr + epr) / 2;
  float p = std::min(1.0f, std::max(0.0f, er));
  if (rng.next() < p) {
    out.d = refl;
    out.color = mul(out.color, er / cos_term(S, out));
    out.dprob = p;
    out.inside = in.inside;
  } else {
    out.color = mul(out.color, (cn * cn) / (nn * nn));  // eye path
    out.color = mul(out.color, (1 - er) / cos_term(S, out));
    out.dprob = 1 - p;
    out.inside = outside;
  }
  out.d = normalized(out.d);
  return out;
}

// SceneEmissiveObject::scatter (src/SceneEmissiveObject.cpp:4-19): the path ends; the
// emission counts on the front side.
PRay scatter_emissive(const Scene& S, int obj, const PRay& in) {
  PRay out;
  out.o = add(in.o, mul(in.d, in.idist));
  out.contact = obj;
  out.ctri = in.itri;
  out.d = {0, 0, 0};
  out.color = dot(in.d, contact_normal(S, out)) <= 0 ? v3(S.objs[obj].color) : V3{0, 0, 0};
  out.dprob = 1;
  return out;
}

// SceneObject::scatter (src/SceneObject.cpp:373-380): one of the object's materials at
// random (Phong: glossy or diffuse).
PRay scatter(const Scene& S, int obj, const PRay& in, bool russian, Rng& rng) {
  const rxo_pt_object& ob = S.objs[obj];
  if (in.isect < 0) {  // nothing hit (a ray inside an object that escaped it): the path ends
    PRay out;
    out.o = in.o;
    out.d = {0, 0, 0};
    out.color = {0, 0, 0};
    return out;
  }
  switch (ob.kind) {
    case kDiffuse: return scatter_diffuse(S, obj, v3(ob.color), in, russian, rng);
    case kGlossy: return scatter_glossy(S, obj, v3(ob.color), ob.coeff, in, russian, rng);
    case kPhong:
      return rng.next() < 0.5f ? scatter_glossy(S, obj, v3(ob.color), ob.coeff, in, russian, rng)
                               : scatter_diffuse(S, obj, v3(ob.diffuse_color), in, russian, rng);
    case kRefractive:
    case kReflective: return scatter_refractive(S, obj, in, rng);
    case kEmissive: return scatter_emissive(S, obj, in);
    default: {
      PRay out;
      out.d = {0, 0, 0};
      out.color = {0, 0, 0};
      return out;
    }
  }
}

// Scene::intersect with NoSelfIntersectionCondition (src/NoSelfIntersectionCondition.cpp:12-27)
// built from `r` (cond false: the camera's first query, which has none).
float intersect(const Scene& S, const PRay& r, bool cond, unsigned& tid) {
  if (!cond) return node_isect(S.T, 0, r.o, r.d, tid, AlwaysLegal{});
  const int contact = r.contact, inside = r.inside;
  auto legal = [&](uint32_t t, float dist) {
    int obj = (int)S.tri_obj[t];
    float d = dot(r.d, world_normal(S, t, add(r.o, mul(r.d, dist))));
    bool in = d <= 0, out = d >= 0;
    if (inside == contact) return !(in && contact == obj);
    return !(out && inside != obj);
  };
  return node_isect(S.T, 0, r.o, r.d, tid, legal);
}

// One eye path of PathTracer::renderPixels: the camera ray through the jittered pixel,
// the bounce loop of samplePathIter, and the path's contribution (product of colour over
// direction and origin pdfs, cosine and transmittance of every ray but the last) when it
// ends on an emitter, divided by the pixel-centre cosine (Camera::eliminateVignetting,
// src/Camera.cpp:78-96). Returns the contribution; `rays` counts intersection queries.
V3 trace_path(const Scene& S, int px, int py, uint32_t max_depth, uint32_t rr_mode, Rng& rng, uint64_t& rays) {
  // Camera::generateRay / generateRayBase (src/Camera.cpp:4-47)
  float xp = (float)px + rng.next() - S.width / 2.0f, yp = S.height / 2.0f - ((float)py + rng.next());
  PRay r;
  r.o = S.cpos;
  r.d = normalized(add(add(mul(S.front, S.sight), mul(S.right, xp)), mul(S.up, yp)));
  r.contact = kCamera;
  unsigned tid = 0;
  rays++;
  float dist = intersect(S, r, false, tid);
  if (dist >= 0) {
    r.isect = (int)S.tri_obj[tid];
    r.itri = (int)tid;
    r.idist = dist;
  }
  V3 color{1, 1, 1};
  bool emitted = false;
  for (uint32_t depth = 0;; depth++) {
    int so = r.inside >= 0 ? r.inside : r.isect;
    if (so < 0) break;  // nothing hit: the terminating ray
    bool russian = rr_mode == 0 || depth >= 3;
    PRay nx = scatter(S, so, r, russian, rng);
    // shading-normal light-leak check (src/MCRenderer.cpp:185-202)
    if (len(nx.d) > 0.5f && nx.inside == kNone && nx.contact >= 0) {
      V3 gn = contact_normal(S, nx, false), sn = contact_normal(S, nx, true);
      V3 wi = neg(r.d), wo = nx.d;
      if (dot(gn, wi) * dot(sn, wi) <= 0 || dot(gn, wo) * dot(sn, wo) <= 0) {
        nx.d = {0, 0, 0};
        nx.color = {0, 0, 0};
      }
    }
    // the contribution of ray r (not the last): colour / pdfs x cosine x transmittance
    color = mul(color, 1.0f / (r.dprob * r.oprob));
    color = mulv(color, r.color);
    color = mul(color, cos_term(S, r));
    color = mulv(color, decay_of(S, r.inside, len(sub(nx.o, r.o))));
    if (len(nx.d) < 0.5f) {  // the path ends with nx
      if (nx.contact >= 0 && S.objs[nx.contact].kind == kEmissive) {
        color = mulv(color, mul(nx.color, 1.0f / (nx.dprob * nx.oprob)));
        emitted = true;
      }
      break;
    }
    if (depth + 1 > max_depth) break;
    rays++;
    dist = intersect(S, nx, true, tid);
    if (dist < 0) break;
    nx.isect = (int)S.tri_obj[tid];
    nx.itri = (int)tid;
    nx.idist = dist;
    r = nx;
  }
  if (!emitted) return {0, 0, 0};
  V3 dc = normalized(add(add(mul(S.front, S.sight), mul(S.right, px + 0.5f - S.width / 2.0f)),
                         mul(S.up, S.height / 2.0f - 0.5f - py)));
  return mul(color, 1.0f / std::fabs(dot(dc, S.front)));
}

}  // namespace

extern "C" {

// PathTracer::renderPixels over the crop [x0, x0 + w) x [y0, y0 + h) of the camera's
// image: sum[(y * w + x) * 3 + c] = the sum over spp samples of the pixel's
// vignetting-corrected path contributions, sq the sum of their squares (may be null).
// rr_mode 0: the reference's Russian roulette at every bounce; 1: from depth 3 on.
// Returns the number of closest-hit queries traced.
uint64_t rxo_pt_render(const rxo_tree* T, const uint32_t* tri_obj, const float* vnormals, const rxo_pt_object* objs,
                       uint32_t nobj, const rxo_pt_camera* cam, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
                       uint32_t spp, uint32_t max_depth, uint32_t rr_mode, uint64_t seed, int nthreads, double* sum,
                       double* sq) {
  Scene S;
  S.T = T;
  S.tri_obj = tri_obj;
  S.vnormals = vnormals;
  S.objs = objs;
  S.nobj = nobj;
  S.cpos = v3(cam->position);
  S.front = normalized(sub(v3(cam->focus), S.cpos));
  S.right = normalized(cross(S.front, v3(cam->up)));
  S.up = cross(S.right, S.front);
  S.sight = (float)cam->sight_dist;
  S.width = (int)cam->width;
  S.height = (int)cam->height;
  uint64_t rays = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : rays)
#endif
  for (long q = 0; q < (long)w * h; q++) {
    int px = (int)(x0 + q % w), py = (int)(y0 + q / w);
    double acc[3] = {0, 0, 0}, acc2[3] = {0, 0, 0};
    Rng rng(seed, (uint64_t)py * cam->width + px);
    uint64_t r = 0;
    for (uint32_t s = 0; s < spp; s++) {
      V3 c = trace_path(S, px, py, max_depth, rr_mode, rng, r);
      const double v[3] = {c.x, c.y, c.z};
      for (int k = 0; k < 3; k++) {
        acc[k] += v[k];
        acc2[k] += v[k] * v[k];
      }
    }
    rays += r;
    for (int k = 0; k < 3; k++) {
      sum[3 * q + k] = acc[k];
      if (sq) sq[3 * q + k] = acc2[k];
    }
  }
  return rays;
}

}  // extern "C"
