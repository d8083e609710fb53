// The reference's Ray-level light-transport semantics as device functions over a path
// vertex record (reference include/Ray.h, src/Ray.cpp): scattering by every material of
// the path (SceneObject::scatter and its materials, SceneVPMObject::scatter), the BSDF
// and pdf queries the bidirectional estimators ask for (getBSDF,
// getDirectionSampleProbDensity, getOriginSampleProbDensity, getCosineTerm,
// getRadianceDecay), emission and camera rays, and Scene::findInsideObject.
#pragma once
#include "rx_pt.cuh"

namespace rx {

constexpr int kNone = -1;
constexpr int kCameraObj = -2;
enum : uint32_t { kDirRandom = 1u, kOrgRandom = 2u };

struct CamDev {
  F3 pos, front, right, up;
  float sight;
  int width, height;
};

// One reference Ray: a path vertex.
struct PV {
  F3 o, d, c;          // origin, direction (length 0: path end), colour (BSDF value)
  float dprob, oprob;  // directionProb, originProb
  int contact;         // contact object id, kNone, or kCameraObj
  int ctri;            // contact triangle (global id), -1 if none
  int inside;          // inside object id or kNone
  uint32_t flags;      // kDirRandom: directionSampleType RANDOM; kOrgRandom: originSampleType
  int pixel;
};

__device__ __forceinline__ PV pv_term(F3 origin) {
  PV t;
  t.o = origin;
  t.d = {0, 0, 0};
  t.c = {0, 0, 0};
  t.dprob = 1.0f;
  t.oprob = 1.0f;
  t.contact = kNone;
  t.ctri = -1;
  t.inside = kNone;
  t.flags = 0;  // DEFINITE, DEFINITE
  t.pixel = -1;
  return t;
}

__device__ __forceinline__ bool is_vpm(const DevScene& S, int obj) {
  return obj >= 0 && S.objects[obj].material == kVPM;
}
__device__ __forceinline__ bool is_emissive(const DevScene& S, int obj) {
  return obj >= 0 && S.objects[obj].material == kEmissive;
}
// SceneObject::getRefrCoeff: the dielectric's coefficient, the medium's IOR, else 1
__device__ __forceinline__ float refr_coeff(const DevScene& S, int obj) {
  if (obj < 0) return 1.0f;
  uint32_t m = S.objects[obj].material;
  return (m == kRefractive || m == kVPM) ? S.objects[obj].ior : 1.0f;
}
__device__ __forceinline__ F3 sigma_t(const DevObject& ob) {
  return {ob.sigma_s[0] + ob.sigma_a[0], ob.sigma_s[1] + ob.sigma_a[1], ob.sigma_s[2] + ob.sigma_a[2]};
}
// SceneVPMObject p_medium / P_surface (include/SceneVPMObject.h:34-47)
__device__ __forceinline__ float p_medium(const DevObject& ob, float s) {
  F3 t = sigma_t(ob);
  return lum({t.x * expf(-t.x * s), t.y * expf(-t.y * s), t.z * expf(-t.z * s)});
}
__device__ __forceinline__ float P_surface(const DevObject& ob, float d) {
  F3 t = sigma_t(ob);
  return lum({expf(-t.x * d), expf(-t.y * d), expf(-t.z * d)});
}
// HGPhaseFunc::evaluate / HGPhaseSampler::getProbDensity (include/HGPhaseFunc.h,
// include/HGPhaseSampler.h:63-69): the same value
__device__ __forceinline__ float hg(float g, float cos_theta) {
  float tmp = 1.0f + g * g - 2.0f * g * cos_theta;
  return (1.0f / (4.0f * RX_PI)) * (1.0f - g * g) / (tmp * sqrtf(tmp));
}
// HGPhaseSampler::genSample (include/HGPhaseSampler.h:13-34), right-handed frame about d
__device__ __forceinline__ F3 hg_sample(float g, F3 d, float e1, float e2) {
  float ct;
  if (fabsf(g) < 1e-5f) {
    ct = 1.0f - 2.0f * e1;
  } else {
    float sq = (1.0f - g * g) / (1.0f - g + 2.0f * g * e1);
    ct = (1.0f + g * g - sq * sq) / (2.0f * g);
  }
  float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  float sp, cp;
  sincosf(2.0f * RX_PI * e2, &sp, &cp);
  Frame f = frame_from(d);
  return to_world(f, F3{st * cp, ct, st * sp});
}

// COS_TERM_MIN (reference include/macros.h:9): the floor of Ray::getCosineTerm.
constexpr float kCosMin = 1e-6f;

// Ray::getContactNormal: the contact object's normal at the ray origin; the camera's is
// its viewing direction (Camera::getWorldNormal).
__device__ __forceinline__ F3 contact_normal(const DevScene& S, const CamDev& cam, const PV& r, bool flat = false) {
  if (r.contact == kCameraObj) return cam.front;
  if (r.contact < 0 || r.ctri < 0) return {0, 0, 0};
  TriGeom g = tri_geom(S, r.ctri);
  return world_normal(g, S.objects[g.obj].has_normals, r.o, flat);
}
// Ray::getCosineTerm (src/Ray.cpp:71-77)
__device__ __forceinline__ float cos_term(const DevScene& S, const CamDev& cam, const PV& r) {
  float d = 1.0f;
  bool has_cos = r.contact == kCameraObj || (r.contact >= 0 && !is_vpm(S, r.contact));
  if (has_cos && length(r.d) > 0.5f) d = fabsf(dot(contact_normal(S, cam, r), r.d));
  return fmaxf(d, kCosMin);
}
// Ray::getRadianceDecay: the inside object's transmittance over `dist`
__device__ __forceinline__ F3 decay_of(const DevScene& S, int inside, float dist) {
  if (inside < 0) return {1, 1, 1};
  const DevObject& ob = S.objects[inside];
  if (ob.material == kRefractive)
    return {powf(ob.decay[0], dist), powf(ob.decay[1], dist), powf(ob.decay[2], dist)};
  if (ob.material == kVPM) {
    F3 t = sigma_t(ob);
    return {expf(-t.x * dist), expf(-t.y * dist), expf(-t.z * dist)};
  }
  return {1, 1, 1};
}

// Scene::findInsideObject (src/Scene.cpp:354-390): the last volumetric object (other than
// `exclude`) that the +-d rays from o both leave through its surface.
__device__ __forceinline__ int find_inside(const DevScene& S, F3 o, F3 d, int exclude) {
  for (int i = (int)S.num_objects - 1; i >= 0; i--) {
    if (i == exclude || !is_vpm(S, i)) continue;
    bool ok = true;
    for (int side = 0; side < 2 && ok; side++) {
      F3 dd = side == 0 ? -d : d;
      PHit h = trace_cond<false>(S, o, dd, INFINITY, kNone, kNone, i);
      if (h.tid < 0 || h.t < 1e-6f) {
        ok = false;
        break;
      }
      TriGeom g = tri_geom(S, h.tid);
      F3 n = world_normal(g, S.objects[i].has_normals, o + dd * h.t);
      if (dot(n, dd) < 1e-6f) ok = false;
    }
    if (ok) return i;
  }
  return kNone;
}

// ---------------------------------------------------------------------------------------
// BSDF and pdf queries
// ---------------------------------------------------------------------------------------
// The getBSDF of a non-medium object `obj` (camera, emitter, surface materials).
static __device__ F3 bsdf_surface(const DevScene& S, const CamDev& cam, int obj, const PV& in, const PV& out) {
  if (obj == kCameraObj) return {1, 1, 1};  // Camera::getBSDF
  const DevObject& ob = S.objects[obj];
  if (ob.material == kEmissive) {  // SceneEmissiveObject::getBSDF
    if (dot(contact_normal(S, cam, out), out.d) < 0.0f) return {0, 0, 0};
    return f3v(ob.color);
  }
  F3 f = {0, 0, 0};
  if (out.contact == kNone || ob.material == kVPM) return f;  // material getBSDF needs a contact object
  F3 n = contact_normal(S, cam, out);
  bool front = dot(n, in.d) <= 0.0f && dot(n, out.d) >= 0.0f;
  if (ob.material == kDiffuse || ob.material == kPhong) {
    F3 c = ob.material == kPhong ? f3v(ob.diffuse_color) : f3v(ob.color);
    if (front) f = f + c * (1.0f / RX_PI);
  }
  if (ob.material == kGlossy || ob.material == kPhong) {  // GlossyMaterial::getBSDF, extra max(colour)
    F3 c = f3v(ob.color);
    if (front) {
      F3 r = n * (-dot(n, in.d) * 2.0f) + in.d;
      float rw = dot(r, out.d);
      if (rw > 0.0f) f = f + c * (maxc(c) * powf(rw, ob.coeff));
    }
  }
  return f;  // RefractiveMaterial has no getBSDF: 0
}

// in.getBSDF(out): Ray::getBSDF (src/Ray.cpp:14-25) -> the out ray's contact (or inside)
// object's getBSDF(in, out); a medium delegates to a contact surface
// (SceneVPMObject::getBSDF).
static __device__ F3 bsdf_of(const DevScene& S, const CamDev& cam, const PV& in, const PV& out) {
  int obj = out.contact != kNone ? out.contact : out.inside;
  if (obj == kNone) return {0, 0, 0};
  if (obj >= 0 && S.objects[obj].material == kVPM) {
    const DevObject& ob = S.objects[obj];
    if (out.contact == kNone) return f3v(ob.sigma_s) * hg(ob.g, dot(in.d, out.d));
    if (out.contact != obj) return bsdf_surface(S, cam, out.contact, in, out);
    return {0, 0, 0};
  }
  return bsdf_surface(S, cam, obj, in, out);
}

// The getDirectionSampleProbDensity of a non-medium object `obj`. `emitted`: the
// reference's &inRay == &outRay case (a ray asked about itself: its emission pdf).
static __device__ float dir_pdf_surface(const DevScene& S, const CamDev& cam, int obj, const PV& in, const PV& out,
                                 bool emitted) {
  if (obj == kCameraObj) return 1.0f;  // Camera::getDirectionSampleProbDensity
  const DevObject& ob = S.objects[obj];
  if (ob.material == kVPM) return 0.0f;
  if (emitted) return cos_lobe_pdf(contact_normal(S, cam, out), out.d, 1.0f);  // SceneObject.cpp:325-334
  if (ob.material == kEmissive) return 0.0f;  // no materials
  if (ob.material == kRefractive || ob.material == kReflective) return 1.0f;  // Material default
  if (out.contact == kNone) return 0.0f;
  F3 n = contact_normal(S, cam, out);
  float pdf = 0.0f;
  int nm = 0;
  if (ob.material == kDiffuse || ob.material == kPhong) {
    F3 c = ob.material == kPhong ? f3v(ob.diffuse_color) : f3v(ob.color);
    pdf += maxc(c) * cos_lobe_pdf(n, out.d, 1.0f);
    nm++;
  }
  if (ob.material == kGlossy || ob.material == kPhong) {
    F3 r = n * (-dot(n, in.d) * 2.0f) + in.d;
    pdf += cos_lobe_pdf(r, out.d, ob.coeff);
    nm++;
  }
  return nm > 1 ? pdf / (float)nm : pdf;
}

// in.getDirectionSampleProbDensity(out) (src/Ray.cpp:27-38) with the medium's
// SceneVPMObject::getDirectionSampleProbDensity (delegation to a contact surface, else
// albedo times the HG density).
static __device__ float dir_pdf(const DevScene& S, const CamDev& cam, const PV& in, const PV& out, bool emitted) {
  int obj = out.contact != kNone ? out.contact : out.inside;
  if (obj == kNone) return 0.0f;
  if (obj >= 0 && S.objects[obj].material == kVPM) {
    const DevObject& ob = S.objects[obj];
    if (!(out.flags & kDirRandom)) return 0.0f;
    if (out.contact != kNone) return out.contact == obj ? 0.0f : dir_pdf_surface(S, cam, out.contact, in, out, false);
    F3 t = sigma_t(ob);
    float albedo = lum(f3v(ob.sigma_s)) / lum(t);
    return albedo * hg(ob.g, dot(normalize(in.d), out.d));
  }
  return dir_pdf_surface(S, cam, obj, in, out, emitted);
}

// in.getOriginSampleProbDensity(out) (src/Ray.cpp:40-48): only a medium the in ray is
// inside makes it differ from 1.
__device__ __forceinline__ float origin_pdf(const DevScene& S, const PV& in, const PV& out) {
  if (!is_vpm(S, in.inside)) return 1.0f;
  const DevObject& ob = S.objects[in.inside];
  float dist = fmaxf(length(in.o - out.o), 1e-5f);
  return out.contact != kNone ? P_surface(ob, dist) : p_medium(ob, dist);
}

// ---------------------------------------------------------------------------------------
// Scattering: SceneObject::scatter (materialList[rand()%n]) and SceneVPMObject::scatter.
// `h_*`: the in ray's intersection (object, triangle, distance).
// ---------------------------------------------------------------------------------------
struct Hit3 {
  int obj, tri;
  float dist;
};

__device__ __forceinline__ float fresnel_er(float cur_n, float next_n, float ct, float cph) {
  float a = fabsf(cur_n * ct - next_n * cph) / (cur_n * ct + next_n * cph);
  float b = fabsf(next_n * ct - cur_n * cph) / (next_n * ct + cur_n * cph);
  return (a * a + b * b) * 0.5f;
}

static __device__ PV scatter_material(const DevScene& S, const CamDev& cam, int obj, const PV& in, Hit3 h,
                               bool fix_is_light, bool russian, Rng& rng);

// SceneVPMObject::scatter (src/SceneVPMObject.cpp:4-251)
static __device__ PV scatter_vpm(const DevScene& S, const CamDev& cam, int self, const PV& in, Hit3 h, bool fix_is_light,
                          bool russian, Rng& rng) {
  const DevObject& ob = S.objects[self];
  if (h.obj < 0 || h.tri < 0) {  // nothing hit: the path ends (the reference reports an error)
    PV t = pv_term(in.o);
    t.pixel = in.pixel;
    return t;
  }
  F3 st = sigma_t(ob);
  float samp = -logf(1.0f - rng.next()) / lum(st);
  bool go_in = h.obj == self && in.inside != self;
  bool be_in = in.inside == self;
  bool out_of_vol = samp >= h.dist;
  PV o = pv_term(in.o);
  o.flags = kDirRandom;
  o.pixel = in.pixel;
  if (go_in) {
    F3 x = in.o + in.d * h.dist;
    TriGeom g = tri_geom(S, h.tri);
    F3 n = world_normal(g, S.objects[g.obj].has_normals, x);
    o.o = x;
    o.d = in.d;
    F3 refl = normalize(n * (-dot(n, in.d) * 2.0f) + in.d);
    float theta = acosf(fminf(fmaxf(dot(in.d, n), -1.0f), 1.0f));
    float cur_n = refr_coeff(S, in.inside), next_n = refr_coeff(S, self);
    float sin_phi = cur_n / next_n * sinf(theta);
    o.c = {1, 1, 1};
    o.dprob = 1.0f;
    o.contact = self;
    o.ctri = h.tri;
    o.inside = in.inside;
    if (sin_phi >= 1.0f) {
      o.d = {0, 0, 0};
      o.contact = kNone;
      o.ctri = -1;
      o.flags = 0;
      return o;
    }
    float phi = asinf(sin_phi);
    if (theta > RX_PI * 0.5f) phi = RX_PI - phi;
    float cd = dot(in.d, n);
    F3 tp = normalize(in.d - n * cd);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    F3 wt = normalize(n * cp + tp * sp);
    float er = fresnel_er(cur_n, next_n, fabsf(cosf(theta)), fabsf(cp));
    float p = fminf(fmaxf(er, 0.0f), 1.0f);
    o.flags = 0;  // DEFINITE
    if (rng.next() < p) {
      o.d = refl;
      o.c = o.c * er;  // the medium's contact has no cosine term
      o.dprob = p;
    } else {
      if (!fix_is_light) o.c = o.c * ((cur_n * cur_n) / (next_n * next_n));
      o.c = o.c * (1.0f - er);
      o.dprob = 1.0f - p;
      o.contact = self;
      o.inside = self;
      o.d = wt;
    }
    return o;
  }
  if (be_in && !out_of_vol) {  // scattering inside the medium
    o.o = in.o + in.d * samp;
    o.d = hg_sample(ob.g, in.d, rng.next(), rng.next());
    o.c = F3{1, 1, 1} * hg(ob.g, dot(in.d, o.d));
    o.inside = self;
    o.ctri = h.tri;
    float albedo = lum(f3v(ob.sigma_s)) / lum(st);
    if (rng.next() < albedo || !russian) {
      o.contact = kNone;
      float pdf = hg(ob.g, dot(in.d, o.d));
      o.dprob = russian ? albedo * pdf : pdf;
      o.oprob = p_medium(ob, samp);
      o.flags = kDirRandom;
      o.c = o.c * f3v(ob.sigma_s);
    } else {
      o.d = {0, 0, 0};
      o.c = {0, 0, 0};
      o.dprob = 1.0f;
      o.oprob = p_medium(ob, samp);
      o.contact = kNone;
      o.flags = kDirRandom;
    }
    return o;
  }
  // leaving through, or hitting a surface inside, the medium
  F3 x = in.o + in.d * h.dist;
  if (h.obj == self) {
    TriGeom g = tri_geom(S, h.tri);
    F3 n = world_normal(g, S.objects[g.obj].has_normals, x);
    F3 refl = normalize(n * (-dot(n, in.d) * 2.0f) + in.d);
    float theta = acosf(fminf(fmaxf(dot(in.d, n), -1.0f), 1.0f));
    int outside = find_inside(S, x, in.d, self);
    float cur_n = refr_coeff(S, self), next_n = refr_coeff(S, outside);
    float sin_phi = cur_n / next_n * sinf(theta);
    o.o = x;
    o.contact = h.obj;
    o.ctri = h.tri;
    o.inside = self;
    o.dprob = 1.0f;
    o.c = {1, 1, 1};
    if (sin_phi >= 1.0f) {
      o.d = {0, 0, 0};
      o.contact = kNone;
      o.ctri = -1;
      o.flags = 0;
      return o;
    }
    float phi = asinf(sin_phi);
    if (theta > RX_PI * 0.5f) phi = RX_PI - phi;
    float cd = dot(in.d, n);
    F3 tp = normalize(in.d - n * cd);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    F3 wt = normalize(n * cp + tp * sp);
    float er = fresnel_er(cur_n, next_n, fabsf(cosf(theta)), fabsf(cp));
    float p = fminf(fmaxf(er, 0.0f), 1.0f);
    o.flags = 0;
    o.oprob = P_surface(ob, h.dist);
    if (rng.next() < p) {
      o.d = refl;
      o.c = o.c * er;
      o.dprob = p;
      o.inside = in.inside;
    } else {
      if (!fix_is_light) o.c = o.c * ((cur_n * cur_n) / (next_n * next_n));
      o.c = o.c * (1.0f - er);
      o.dprob = 1.0f - p;
      o.inside = outside;
      o.d = wt;
    }
    return o;
  }
  // a surface inside the medium scatters the ray (origin at the hit, distance 0)
  PV moved = in;
  moved.o = x;
  moved.contact = kNone;
  moved.inside = self;
  PV r = scatter_material(S, cam, h.obj, moved, Hit3{h.obj, h.tri, 0.0f}, fix_is_light, russian, rng);
  r.oprob *= P_surface(ob, h.dist);
  return r;
}

// SceneObject::scatter with the object's material(s): Diffuse, Glossy, Phong (one lobe
// picked uniformly, SceneObject.cpp:373-380), Refractive / Reflective, Emissive. A
// medium object is not handled here (scatter_vpm).
static __device__ PV scatter_material(const DevScene& S, const CamDev& cam, int obj, const PV& in, Hit3 h,
                               bool fix_is_light, bool russian, Rng& rng) {
  const DevObject& ob = S.objects[obj];
  F3 x = in.o + in.d * h.dist;
  PV o = pv_term(x);
  o.pixel = in.pixel;
  uint32_t kind = ob.material;
  if (kind == kVPM) {  // a medium inside a medium is not modelled: the path ends
    o.flags = 0;
    return o;
  }
  if (kind == kEmissive) {  // SceneEmissiveObject::scatter
    o.contact = obj;
    o.ctri = h.tri;
    F3 n = contact_normal(S, cam, o);
    o.c = dot(in.d, n) <= 0.0f ? f3v(ob.color) : F3{0, 0, 0};
    o.flags = kDirRandom;
    return o;
  }
  if (h.obj < 0 || h.tri < 0) {  // "error in ... scatter": nothing was hit
    o.flags = 0;
    return o;
  }
  TriGeom g = tri_geom(S, h.tri);
  F3 n = world_normal(g, S.objects[g.obj].has_normals, x);  // frame of the intersected object
  if (kind == kPhong) kind = rng.next() < 0.5f ? kGlossy : kDiffuse;
  o.contact = obj;
  o.ctri = h.tri;
  o.inside = in.inside;
  if (kind == kDiffuse) {  // DiffuseMaterial::scatter, src/DiffuseMaterial.cpp:4-77
    F3 c = ob.material == kPhong ? f3v(ob.diffuse_color) : f3v(ob.color);
    if (dot(in.d, n) > 0.0f) {  // leaving: pass through
      o.d = in.d;
      o.c = {1, 1, 1};
      o.dprob = 1.0f;
      o.flags = 0;
      return o;
    }
    Frame f = frame_from(n);
    float r1 = rng.next(), r2 = rng.next();
    o.d = to_world(f, hemi_cos(1.0f, r1, r2));
    float p = maxc(c);
    o.flags = kDirRandom;
    if (!(dot(n, o.d) >= kCosMin)) {
      // a direction at the hemisphere's rim (u = 0 exactly: probability 2^-24 for a
      // 24-bit generator, zero for the continuous sampler): its density cos / pi falls
      // below the cosine clamp of Ray::getCosineTerm (COS_TERM_MIN), so the reference's
      // weight (BSDF x clamped cosine / density) would blow up; the path ends instead
      o.d = {0, 0, 0};
      o.c = {0, 0, 0};
      o.dprob = 1.0f;
      return o;
    }
    if (rng.next() < p || !russian) {
      o.c = (dot(n, in.d) <= 0.0f && dot(n, o.d) >= 0.0f) ? c * (1.0f / RX_PI) : F3{0, 0, 0};
      float pdf = cos_lobe_pdf(n, o.d, 1.0f);
      o.dprob = russian ? p * pdf : pdf;
    } else {
      o.d = {0, 0, 0};
      o.c = {0, 0, 0};
      o.dprob = 1.0f - p;
    }
    return o;
  }
  if (kind == kGlossy) {  // GlossyMaterial::scatter, src/GlossyMaterial.cpp:4-57
    F3 c = f3v(ob.color);
    F3 r = n * (-dot(n, in.d) * 2.0f) + in.d;
    Frame f = frame_from(r);
    float r1 = rng.next(), r2 = rng.next();
    o.d = to_world(f, hemi_cos(ob.coeff, r1, r2));
    F3 val = {0, 0, 0};
    if (dot(n, in.d) <= 0.0f && dot(n, o.d) >= 0.0f) {
      float rw = dot(r, o.d);
      if (rw > 0.0f) val = c * powf(rw, ob.coeff);
    }
    o.c = val;
    o.dprob = cos_lobe_pdf(r, o.d, ob.coeff);
    o.flags = kDirRandom;
    float p = maxc(c);
    if (val.x == 0.0f && val.y == 0.0f && val.z == 0.0f) {
      o.d = {0, 0, 0};
      o.dprob = 1.0f;
      return o;
    }
    if (!russian) return o;
    if (rng.next() < p) {
      o.dprob *= p;
    } else {
      o.d = {0, 0, 0};
      o.c = {0, 0, 0};
      o.dprob = 1.0f - p;
    }
    return o;
  }
  // RefractiveMaterial::scatter (src/RefractiveMaterial.cpp:132-269)
  float ior = ob.material == kReflective ? -1.0f : ob.ior;
  F3 surf = f3v(ob.color);
  F3 r = n * (-dot(n, in.d) * 2.0f) + in.d;
  o.flags = 0;
  o.c = surf;
  if (ior < 0.0f) {
    o.d = r;
    o.inside = in.inside;
    o.dprob = 1.0f;
    o.c = surf * (1.0f / cos_term(S, cam, o));
    return o;
  }
  float cd = fminf(fmaxf(dot(in.d, n), -1.0f), 1.0f);
  float theta = acosf(cd);
  int outside = in.inside == obj ? find_inside(S, x, in.d, obj) : obj;
  float cur_n = refr_coeff(S, in.inside), next_n = refr_coeff(S, outside);
  o.dprob = 1.0f;
  float sin_phi = cur_n / next_n * sinf(theta);
  if (sin_phi >= 1.0f) {  // total internal reflection ends the path
    o.d = {0, 0, 0};
    o.contact = kNone;
    o.ctri = -1;
    return o;
  }
  float phi = asinf(sin_phi);
  if (theta > RX_PI * 0.5f) phi = RX_PI - phi;
  F3 tp = normalize(in.d - n * cd);
  float sp, cp;
  sincosf(phi, &sp, &cp);
  F3 wt = normalize(n * cp + tp * sp);
  float er = fresnel_er(cur_n, next_n, fabsf(cosf(theta)), fabsf(cp));
  float p = fminf(fmaxf(er, 0.0f), 1.0f);
  if (rng.next() < p) {
    o.d = normalize(r);
    o.c = o.c * (er / cos_term(S, cam, o));
    o.dprob = p;
    o.inside = in.inside;
  } else {
    o.d = wt;
    if (!fix_is_light) o.c = o.c * ((cur_n * cur_n) / (next_n * next_n));
    o.c = o.c * ((1.0f - er) / cos_term(S, cam, o));
    o.dprob = 1.0f - p;
    o.inside = outside;
  }
  return o;
}

// The object's scatter: a medium's (SceneVPMObject::scatter); a dielectric the ray is
// inside that hits another object hands the ray to that object
// (RefractiveMaterial.cpp:183-187); else the object's material.
static __device__ PV scatter_object(const DevScene& S, const CamDev& cam, int obj, const PV& in, Hit3 h, bool fix_is_light,
                             bool russian, Rng& rng) {
  const DevObject& ob = S.objects[obj];
  if (ob.material == kVPM) return scatter_vpm(S, cam, obj, in, h, fix_is_light, russian, rng);
  if (ob.material == kRefractive && h.obj != obj && in.inside == obj && h.obj >= 0 &&
      S.objects[h.obj].material != kVPM)
    return scatter_material(S, cam, h.obj, in, h, fix_is_light, russian, rng);
  return scatter_material(S, cam, obj, in, h, fix_is_light, russian, rng);
}

// One scatter of MCRenderer::samplePathIter (src/MCRenderer.cpp:169-217): the inside
// object scatters when there is one, else the intersected object; then the
// shading-normal light-leak kill.
// The bounce loop's shading-normal light-leak kill (src/MCRenderer.cpp:183-217).
__device__ __forceinline__ void leak_kill(const DevScene& S, const CamDev& cam, const PV& in, PV& o) {
  if (length(o.d) > 0.5f && o.inside == kNone && o.contact >= 0) {
    F3 ns = contact_normal(S, cam, o, false), nf = contact_normal(S, cam, o, true);
    F3 wi = -in.d;
    if (dot(ns, wi) * dot(nf, wi) <= 0.0f || dot(ns, o.d) * dot(nf, o.d) <= 0.0f) {
      o.d = {0, 0, 0};
      o.c = {0, 0, 0};
    }
  }
}

static __device__ PV scatter_step(const DevScene& S, const CamDev& cam, const PV& in, Hit3 h, bool fix_is_light, bool russian,
                           Rng& rng) {
  int obj = in.inside != kNone ? in.inside : h.obj;
  PV o = scatter_object(S, cam, obj, in, h, fix_is_light, russian, rng);
  leak_kill(S, cam, in, o);
  return o;
}

// SceneObject::emit(isUniformOrigin = true, isUniformDir = false) through
// Scene::SurfaceSampler (src/SceneObject.cpp:233-314, src/Scene.cpp:91-98): an emitter
// triangle by area, a uniform point, a cosine direction (the ray, not yet traced).
static __device__ PV emit_start(const DevScene& S, const CamDev& cam, Rng& rng) {
  float ru = rng.next() * S.light_area;
  int lo = 0, hi = (int)S.num_lights - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&S.light_cdf[mid]) < ru) lo = mid + 1;
    else hi = mid;
  }
  int lt = (int)__ldg(&S.light_tri[lo]);
  TriGeom g = tri_geom(S, lt);
  float u1 = rng.next(), u2 = rng.next();
  float su1 = sqrtf(u1);
  float bu = 1.0f - su1, bv = u2 * su1;
  PV r = pv_term(g.v0 * bu + g.v1 * bv + g.v2 * (1.0f - bu - bv));
  r.contact = g.obj;
  r.ctri = lt;
  r.oprob = 1.0f / S.light_area;
  F3 n = contact_normal(S, cam, r);
  Frame f = frame_from(n);
  float r1 = rng.next(), r2 = rng.next();
  r.d = to_world(f, hemi_cos(1.0f, r1, r2));
  if (dot(n, r.d) < 0.0f) r.d = -r.d;
  r.inside = find_inside(S, r.o, r.d, r.contact);
  r.c = is_emissive(S, r.contact) ? bsdf_of(S, cam, r, r) : F3{1, 1, 1};
  r.dprob = cos_lobe_pdf(n, r.d, 1.0f);
  r.flags = kDirRandom | kOrgRandom;
  return r;
}

// The first hit of an emitted ray (a hit at distance 0 counts as none).
__device__ __forceinline__ Hit3 emit_hit(const DevScene& S, const PV& r) {
  PHit h = trace_cond<false>(S, r.o, r.d, INFINITY, r.contact, r.inside);
  return (h.tid >= 0 && h.t > 0.0f) ? Hit3{(int)__ldg(&S.tri_obj[h.tid]), h.tid, h.t} : Hit3{kNone, -1, -1.0f};
}

// emit_start and its first hit.
static __device__ PV emit_ray(const DevScene& S, const CamDev& cam, Rng& rng, Hit3& hit) {
  PV r = emit_start(S, cam, rng);
  hit = emit_hit(S, r);
  return r;
}

}  // namespace rx
