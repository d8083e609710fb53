// Vertex connection and merging: the reference's VCMTracer (src/VCMTracer.cpp:6-639).
//
// Per iteration (VCMTracer.cpp:25-142):
//  1. Light subpaths (emission sample + the bounce loop of MCRenderer::samplePathIter,
//     with light-path scattering) on persistent warps that take the next subpath when
//     one ends (k_sub_run), their vertices stored; every non-specular
//     vertex after the first that is not on an emitter becomes a photon
//     (VCMTracer.cpp:64-95).
//  2. A sort-by-cell hash grid over the photons (cell = 2 r, SmallVCM's spatial hash
//     (x*73856093)^(y*19349663)^(z*83492791)): count per bucket, exclusive scan,
//     scatter (the counting-sort build of include/Hashgrid.h:21-91); it replaces the
//     per-iteration PointKDTree (include/PointKDTree.h), queried with the same strict
//     |p-x| < r test over the (up to) 8 cells the sphere touches.
//  3. Per pixel, the eye subpath (the same kernel, with light-path scattering, as
//     VCMTracer.cpp:107 does), then colorByMergingPaths (:566-636) and
//     colorByConnectingPaths (:430-562) with the full-path MIS of connectMergeWeight
//     (:321-428, double precision) and light-tracing splats through
//     Camera::transToPixel.
//  4. Vignetting correction of the iteration image and the running mean (FP64 film).
//
// The same pipeline without photons and merging is the reference's
// BidirectionalPathTracer (src/BidirectionalPathTracer.cpp:6-398): eye subpaths sampled
// as eye paths, the connection weight without merge techniques, and its own rule for
// the pure path-tracing technique (VcmParams::bpt).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "rx_bin.cuh"
#include "rx_walk.cuh"
#include "rx_internal.h"
#include "rx_material.cuh"

namespace rx {

constexpr int kMaxV = 24;  // vertices per stored subpath (max_depth <= kMaxV - 3)

struct VcmParams {
  CamDev cam;
  F3 focus;
  uint64_t seed;
  uint32_t iter;
  uint32_t max_depth;
  uint32_t maxv;       // vertices per stored subpath: max_depth + 3
  uint32_t n_light;    // light paths per iteration
  uint32_t n_pixels;
  float radius;
  float norm;          // light-path count normaliser (W*H in the reference)
  uint32_t bpt;        // 1: BidirectionalPathTracer (no merging), 0: VCMTracer
};

// ---- camera ----------------------------------------------------------------------------
__device__ __forceinline__ F3 cam_dir(const CamDev& c, float xp, float yp) {
  float x = xp - c.width * 0.5f, y = c.height * 0.5f - yp;
  return normalize(c.front * c.sight + c.right * x + c.up * y);
}

// Camera::generateRay + generateRayBase (src/Camera.cpp:4-47): the ray, not yet traced.
__device__ PV camera_start(const DevScene& S, const CamDev& c, uint32_t pixel, Rng& rng) {
  int x = pixel % c.width, y = pixel / c.width;
  float jx = rng.next(), jy = rng.next();
  PV r = pv_term(c.pos);
  r.d = cam_dir(c, x + jx, y + jy);
  r.c = {1, 1, 1};
  r.contact = kCameraObj;
  r.flags = kDirRandom;
  r.pixel = (int)pixel;
  r.inside = find_inside(S, r.o, r.d, kNone);
  return r;
}

// The first hit of a camera ray (no condition: the camera is no surface).
__device__ __forceinline__ Hit3 camera_hit(const DevScene& S, const PV& r) {
  PHit h = trace_cond<false>(S, r.o, r.d, INFINITY, kNone, kNone);
  return h.tid >= 0 ? Hit3{(int)__ldg(&S.tri_obj[h.tid]), h.tid, h.t} : Hit3{kNone, -1, -1.0f};
}

// camera_start and its first hit.
__device__ PV camera_ray(const DevScene& S, const CamDev& c, uint32_t pixel, Rng& rng, Hit3& hit) {
  PV r = camera_start(S, c, pixel, rng);
  hit = camera_hit(S, r);
  return r;
}

// MCRenderer::samplePath / samplePathIter (src/MCRenderer.cpp:151-273): the path's rays
// in order, ending with the ray that stopped it or a terminating ray. `light`: the
// isLightPath argument (light-path scattering).
// `put(i, ray)` receives the rays in order; returns their count.
template <class Put>
__device__ int sample_path(const DevScene& S, const CamDev& cam, PV start, Hit3 h, uint32_t max_depth, bool light,
                           Rng& rng, Put&& put) {
  int n = 0;
  PV prev = start;
  for (uint32_t depth = 0;; depth++) {
    put(n++, prev);
    if (prev.inside == kNone && h.obj == kNone) {
      put(n++, pv_term(prev.o));
      return n;
    }
    PV next = scatter_step(S, cam, prev, h, light, true, rng);
    if (length(next.d) < 0.5f) {
      put(n++, next);
      return n;
    }
    if (depth + 1 > max_depth) {
      put(n++, pv_term(prev.o));
      return n;
    }
    PHit hh = trace_cond<false>(S, next.o, next.d, INFINITY, next.contact, next.inside);
    if (hh.tid < 0) {
      put(n++, next);
      put(n++, pv_term(prev.o));
      return n;
    }
    h = Hit3{(int)__ldg(&S.tri_obj[hh.tid]), hh.tid, hh.t};
    prev = next;
  }
}

// ---- packed vertex storage (4 float4 per vertex) ---------------------------------------
__device__ __forceinline__ void store_pv(float4* p, const PV& v) {
  p[0] = make_float4(v.o.x, v.o.y, v.o.z, v.dprob);
  p[1] = make_float4(v.d.x, v.d.y, v.d.z, v.oprob);
  p[2] = make_float4(v.c.x, v.c.y, v.c.z, __int_as_float(v.pixel));
  p[3] = make_float4(__int_as_float(v.contact), __int_as_float(v.ctri), __int_as_float(v.inside),
                     __uint_as_float(v.flags));
}
__device__ __forceinline__ PV load_pv(const float4* p) {
  float4 a = p[0], b = p[1], c = p[2], e = p[3];
  PV v;
  v.o = f3(a);
  v.dprob = a.w;
  v.d = f3(b);
  v.oprob = b.w;
  v.c = f3(c);
  v.pixel = __float_as_int(c.w);
  v.contact = __float_as_int(e.x);
  v.ctri = __float_as_int(e.y);
  v.inside = __float_as_int(e.z);
  v.flags = __float_as_uint(e.w);
  return v;
}

// ---- the MIS weight of a join in O(1) ---------------------------------------------------
// connectMergeWeight sums, over every technique that could have made the joined path
// w[0..n-1] (light vertices 0..ci, eye vertices after), products pf[i] pb[i+1] of
// forward and backward pdf chains (C_i: connection at i, M_i: merge at i). For a join
// (connection or merge) of light vertex ci with eye vertex E = w[ci+1], connectRays
// changes only the two vertices' directions, colours, direction pdfs, sampling flags and
// inside objects, and VCMTracer::link reverses a vertex by its neighbours' positions
// only, so:
//  - pf[0..ci] and the ratios pb[i] / pb[ci-1] (i <= ci-1) depend on the light subpath
//    alone, pb[ci+1..n-1] and the ratios pf[i] / pf[ci+2] (i >= ci+2) on the eye
//    subpath alone;
//  - the techniques at i <= ci-2 add up to pb[ci-1] x (a light-only sum) and those at
//    i >= ci+2, with the merge at ci+1, to pf[ci+2] x (an eye-only sum), both built once
//    per subpath by a recursion over its vertices (light_mis, eye_mis);
//  - what is left (C and M at ci-1 and ci, C at ci+1, and the pdfs through the two
//    changed directions) is evaluated per pair (join_eval).
// The throughput and probability of connectColorProb split the same way.
struct alignas(16) MisL {  // per light vertex c, for a join at ci = c
  float sla;       // pb[c-1] / pb[c] x (C_i + M_i, i <= c-2) / pb[c-1] / pf[c], without the direction pdf at c
  float tla;       // (C_{c-1} + M_{c-1}) / (pb[c] pf[c])
  float prob;      // prod_{i<c} directionProb x originProb
  float pad;
  F3 thr;          // prod_{i<c} colour x transmittance x cosine
  float pad2;
};
struct alignas(16) MisE {  // per eye vertex k, for a join with E = eye vertex k
  double pb;       // pb at eye vertex k (pb[ci+1])
  float pbr;       // pb at eye vertex k-1 / pb at eye vertex k
  float sea;       // pf[ci+2] / pf[ci+1] x (M_{ci+1} + C_i + M_i, i >= ci+2) / pf[ci+2] / pb[ci+1], without the direction pdf at E
  F3 thr;          // prod_{m<k} colour x transmittance x cosine of the eye vertices
  float prob;      // prod_{m<k} directionProb x originProb
};

// link(w, n, ci, i, j) for a link against the subpath's own direction: vertex v aimed
// at u, with u's inside object.
__device__ __forceinline__ PV rev_to(const PV& v, const PV& u) {
  PV r = v;
  r.d = normalize(u.o - v.o);
  r.inside = u.inside;
  return r;
}
__device__ __forceinline__ float seg_len(const PV& a, const PV& b) { return fmaxf(length(b.o - a.o), 1e-5f); }
__device__ __forceinline__ bool rnd(const PV& v) { return (v.flags & kDirRandom) != 0u; }
// the merge technique's pdf factors of connectMergeWeight (VCMTracer.cpp:400-409) past pf, pb
__device__ __forceinline__ double merge_area(double p, const PV& v, float r, float norm) {
  p *= RX_PI * r * r;
  if (v.inside != kNone && v.contact == kNone) p *= 4.0 / 3.0 * r;
  return p * norm;
}

// Light-subpath records for c = 0 .. n-1, from the stored vertices of one light path
// (a window of four vertices, c - 2 .. c + 1, in registers).
__device__ void light_mis(const DevScene& S, const CamDev& cam, const float4* lb, int n, float r, float norm,
                          bool merges, MisL* out) {
  PV l2, l1, v = load_pv(lb), nx;  // vertices c - 2, c - 1, c, c + 1
  double pf = v.oprob, pf_prev = 0.0, sl = 0.0;
  F3 thr = {1, 1, 1};
  float prob = 1.0f;
  for (int c = 0; c < n; c++) {
    if (c + 1 < n) nx = load_pv(lb + 4 * (c + 1));
    MisL m;
    double al = 0.0, tl = 0.0;
    if (c >= 1) {
      const PV& a = l1;
      float d = seg_len(a, v);
      PV rv = rev_to(v, a);
      al = cos_term(S, cam, a);
      al /= (double)d * d;
      if (rnd(v)) al *= origin_pdf(S, rv, a);
      tl = rnd(a) && rnd(v) ? pf_prev : 0.0;
      if (merges && rnd(v)) {
        double p = pf_prev;
        if (rnd(a)) p *= c - 1 > 0 ? dir_pdf(S, cam, l2, a, false) : dir_pdf(S, cam, a, a, true);
        p *= origin_pdf(S, a, v);
        p *= cos_term(S, cam, rv);
        p /= (double)d * d;
        tl += merge_area(p, v, r, norm);
      }
    }
    m.sla = (float)(al * sl / pf);
    m.tla = (float)(tl / pf);
    m.prob = prob;
    m.pad = 0.0f;
    m.thr = thr;
    m.pad2 = 0.0f;
    out[c] = m;
    if (c + 1 >= n) break;
    // advance to c + 1
    float d = seg_len(v, nx);
    prob *= v.dprob * v.oprob;
    thr = thr * v.c;
    thr = thr * decay_of(S, v.inside, d);
    thr = thr * cos_term(S, cam, v);
    double pfn = pf * cos_term(S, cam, rev_to(nx, v));
    pfn /= (double)d * d;
    if (rnd(v)) {
      pfn *= c > 0 ? dir_pdf(S, cam, l1, v, false) : dir_pdf(S, cam, v, v, true);
      pfn *= origin_pdf(S, v, nx);
    }
    if (c >= 1) {
      double g = al;
      if (rnd(v)) g *= dir_pdf(S, cam, rev_to(nx, v), rev_to(v, l1), false);
      sl = sl * g + tl;
    }
    pf_prev = pf;
    pf = pfn;
    l2 = l1;
    l1 = v;
    v = nx;
  }
}

// Eye-subpath records for k = 0 .. n-1 (k >= 1 are merge vertices); e(k) gives vertex k.
template <class Get>
__device__ void eye_mis(const DevScene& S, const CamDev& cam, Get&& e, int n, float r, float norm, bool merges,
                        MisE* out) {
  double pb = e(0).oprob, pb_prev = 0.0, u = 0.0;
  F3 thr = {1, 1, 1};
  float prob = 1.0f;
  for (int k = 0; k < n; k++) {
    const PV v = e(k);
    MisE m;
    m.pb = pb;
    m.pbr = (float)(pb_prev / pb);
    m.sea = 0.0f;
    if (k >= 1) {
      const PV pe = e(k - 1);
      float d = seg_len(v, pe);
      double fe = cos_term(S, cam, pe);
      fe /= (double)d * d;
      fe *= origin_pdf(S, rev_to(v, pe), pe);
      double se = u + (merges && k >= 2 && rnd(pe) ? merge_area(pb_prev, pe, r, norm) : 0.0);
      m.sea = (float)(fe * se / pb);
    }
    m.thr = thr;
    m.prob = prob;
    out[k] = m;
    if (k + 1 >= n) break;
    // advance to k + 1
    const PV up = e(k + 1);
    float d = seg_len(v, up);
    thr = thr * v.c;
    thr = thr * decay_of(S, v.inside, d);
    thr = thr * cos_term(S, cam, v);
    prob *= v.dprob * v.oprob;
    double pbn = pb * cos_term(S, cam, rev_to(up, v));
    pbn /= (double)d * d;
    if (rnd(v)) {
      pbn *= k > 0 ? dir_pdf(S, cam, e(k - 1), v, false) : dir_pdf(S, cam, v, v, true);
      pbn *= origin_pdf(S, v, up);
    }
    if (k >= 1) {
      const PV pe = e(k - 1);
      float dd = seg_len(v, pe);
      PV rv = rev_to(v, pe);
      double g = cos_term(S, cam, pe);
      g /= (double)dd * dd;
      double opf = origin_pdf(S, rv, pe);
      if (rnd(v)) {
        g *= dir_pdf(S, cam, rev_to(up, v), rv, false);
        g *= opf;
      }
      double un = u * g;
      if (rnd(v) && rnd(pe)) un += pb_prev;
      if (merges && k >= 2 && rnd(pe)) un += merge_area(g * pb_prev * (rnd(v) ? 1.0 : opf), pe, r, norm);
      u = un;
    }
    pb_prev = pb;
    pb = pbn;
  }
}

// connectRays (MCRenderer.cpp:50-106) for light vertex L (w[ci]) and eye vertex E
// (w[ci+1]). Lm: the light vertex before L (null when ci = 0); pe: the eye vertex
// before E (null when E is the camera vertex, t = 1). Where the reference's neighbour
// index clamps onto the vertex itself (pl for ci = 0, pe for t = 1), the vertex is its
// own neighbour, already redirected. A merge changes only the directions and E.
__device__ __forceinline__ void join(const DevScene& S, const CamDev& cam, const PV& L, const PV* Lm, const PV& E,
                                     const PV* pe, bool merged, PV& Lp, PV& Ep) {
  Lp = L;
  Lp.d = normalize(E.o - L.o);
  Ep = E;
  Ep.d = -Lp.d;
  if (!merged) {
    Lp.dprob = 1.0f;
    Lp.c = bsdf_of(S, cam, Lm ? *Lm : Lp, Lp);
    Lp.flags |= kDirRandom;
    if (Lp.contact != kNone && Lm) {
      F3 n0 = contact_normal(S, cam, Lp);
      if (dot(n0, Lp.d) <= 0.0f) Lp.inside = Lp.contact;
      else if (dot(n0, Lm->d) <= 0.0f) Lp.inside = Lm->inside;
      else Lp.inside = find_inside(S, Lp.o, Lp.d, Lp.contact);
    }
  }
  Ep.dprob = 1.0f;
  Ep.c = bsdf_of(S, cam, pe ? *pe : Ep, Ep);
  Ep.flags |= kDirRandom;
  if (Ep.contact != kNone && pe) {
    F3 n0 = contact_normal(S, cam, Ep);
    if (dot(n0, Ep.d) <= 0.0f) Ep.inside = Ep.contact;
    else if (dot(n0, pe->d) <= 0.0f) Ep.inside = pe->inside;
    else Ep.inside = find_inside(S, Ep.o, Ep.d, Ep.contact);
  }
}

// connectColorProb (VCMTracer.cpp:248-306) and connectMergeWeight (:321-428) of the
// joined path from the two subpaths' records. Returns false where the reference drops
// the path (zero colour or probability); col / prob / wt as the reference's.
__device__ bool join_eval(const DevScene& S, const CamDev& cam, const PV& L, const PV* Lm, const PV& Lp, const PV& Ep,
                          const PV* pe, const MisL& ml, const MisE& me, bool merged, bool bpt, float r, float norm,
                          F3& col, float& prob, float& wt) {
  const float D = fmaxf(length(Ep.o - Lp.o), 1e-5f);
  const float cosL = cos_term(S, cam, Lp), cosE = cos_term(S, cam, Ep);
  const PV rE = pe ? rev_to(Ep, *pe) : Ep;  // link(ci+1, ci+2); for t = 1 only its origin is read
  const bool rl = rnd(Lp);
  const float opf = origin_pdf(S, Lp, rE);
  col = ml.thr * Lp.c;
  col = col * decay_of(S, Lp.inside, D);
  col = col * (cosL * cosE / (D * D));
  col = col * Ep.c;
  col = col * me.thr;
  prob = ml.prob * (Lp.dprob * Lp.oprob) * (Ep.dprob * Ep.oprob) * me.prob;
  if (merged) {
    prob *= RX_PI * r * r;
    prob *= cosE;
    prob /= D * D;
    prob *= opf;
    if (Ep.inside != kNone && Ep.contact == kNone) prob *= 4.0f / 3.0f * r;
  }
  if (!(prob > 0.0f) || !(length(col) > 0.0f)) return false;
  float dpf = 1.0f;
  if (rl) dpf = Lm ? dir_pdf(S, cam, *Lm, Lp, false) : dir_pdf(S, cam, Lp, Lp, true);
  // every term over pf[ci] pb[ci+1]
  const float g = 1.0f / (D * D);
  const float C = rl ? 1.0f : 0.0f;  // connection at ci
  float M = 0.0f;                     // merge at ci (needs an eye vertex after E; none without merging)
  if (pe && !bpt) {
    M = (rl ? dpf : 1.0f) * opf * cosE * g * (RX_PI * r * r) * norm;
    if (Ep.inside != kNone && Ep.contact == kNone) M *= 4.0f / 3.0f * r;
  }
  float sum = C + M;
  float pb0 = cosL * g * origin_pdf(S, Ep, L);  // pb[ci] / pb[ci+1]
  pb0 *= pe ? dir_pdf(S, cam, *pe, Ep, false) : dir_pdf(S, cam, Ep, Ep, true);
  if (Lm) sum += pb0 * ((rl ? dir_pdf(S, cam, Ep, rev_to(Lp, *Lm), false) : 1.0f) * ml.sla + ml.tla);
  if (pe) {
    const float pf1 = cosE * g * (rl ? dpf * opf : 1.0f);  // pf[ci+1] / pf[ci]
    if (rnd(*pe)) sum += pf1 * me.pbr;                      // connection at ci+1
    sum += pf1 * dir_pdf(S, cam, Lp, rE, false) * me.sea;
  }
  if (!pe && !Lm && !bpt) sum += pb0 / L.oprob;  // two-vertex path: VCM's mustUsePT adds pb[0] (pf[0] = originProb of L)
  const float res = (merged ? M : C) / sum;
  wt = res >= 0.0f ? res : 0.0f;
  return true;
}

// ---- light subpaths + photons ----------------------------------------------------------
// One light subpath per thread (the whole-path check mode, RX_VCM_FULL_PATH_MIS; the
// default samples them on persistent warps, k_sub_run below).
__global__ void __launch_bounds__(128) k_vcm_light(DevScene S, VcmParams P, float4* lv, int* llen,
                                                   float4* photon_pos, int* photon_ref, unsigned* n_photons,
                                                   unsigned photon_cap, unsigned long long* rays) {
  uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long nr = 0;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_light; p += stride) {
    Rng rng(P.seed, ((uint64_t)P.iter << 33) | (uint64_t)p, 0);
    Hit3 h;
    PV start = emit_ray(S, P.cam, rng, h);
    float4* out = lv + 4 * ((size_t)p * P.maxv);
    bool emitter_seen = false;  // photons stop at the first emitter after the origin
    int n = sample_path(S, P.cam, start, h, P.max_depth, true, rng, [&](int i, const PV& v) {
      store_pv(out + 4 * i, v);
      if (P.bpt || i == 0 || emitter_seen) return;  // no photons without merging
      if (is_emissive(S, v.contact)) {
        emitter_seen = true;
        return;
      }
      if (!(v.flags & kDirRandom)) return;
      unsigned slot = atomicAdd(n_photons, 1u);
      if (slot < photon_cap) {
        photon_pos[slot] = make_float4(v.o.x, v.o.y, v.o.z, 0.0f);
        photon_ref[slot] = (int)(p * P.maxv + i);
      }
    });
    nr += (unsigned long long)n;
    llen[p] = n;
  }
  if (nr) atomicAdd(rays, nr);
}

// ---- subpaths on persistent warps --------------------------------------------------------
// The bounce loop of sample_path with the subpaths spread over persistent warps: a lane
// whose subpath has ended takes the next one from a counter (one atomic per warp and
// refill), so a warp's lanes stay busy until every subpath is sampled, and one slow
// bounce holds only its own lane (a ray that finds no legal hit walks most of the tree)
// instead of the whole GPU at every depth, as it would with one launch per depth. Every
// iteration of the loop traces one ray per busy lane: a new subpath's first ray, or the
// ray the lane's last scatter made; then the lane stores the vertex, scatters again or
// ends. The random numbers, and so the subpaths, are sample_path's.
// Where a subpath's vertices go: the vertex store, and for VCM light subpaths the photons
// (random vertices after the origin, up to the first emitter: k_vcm_light's rule).
struct SubSink {
  float4* verts;
  int* len;
  bool photons;
  float4* photon_pos;
  int* photon_ref;
  unsigned* n_photons;
  unsigned photon_cap;
  __device__ void put(const DevScene& S, const VcmParams& P, uint32_t p, int i, const PV& v, bool& seen) const {
    store_pv(verts + 4 * ((size_t)p * P.maxv + i), v);
    if (!photons || i == 0 || seen) return;
    if (is_emissive(S, v.contact)) {
      seen = true;
      return;
    }
    if (!(v.flags & kDirRandom)) return;
    unsigned slot = atomicAdd(n_photons, 1u);
    if (slot < photon_cap) {
      photon_pos[slot] = make_float4(v.o.x, v.o.y, v.o.z, 0.0f);
      photon_ref[slot] = (int)(p * P.maxv + i);
    }
  }
};

// Light subpaths from emit_start (k_vcm_light's stream) or eye subpaths from
// camera_start (k_vcm_eye_full's), each subpath's vertices in the store; `light`: the
// isLightPath argument of the scattering. cursor: subpaths handed out (zero at launch).
template <bool LIGHT>
__global__ void __launch_bounds__(128) k_sub_run(DevScene S, VcmParams P, SubSink out, bool light_scatter,
                                                 unsigned* cursor, unsigned long long* rays) {
  constexpr unsigned FULL = 0xffffffffu;
  const uint32_t n = LIGHT ? P.n_light : P.n_pixels;
  const int lane = threadIdx.x & 31;
  bool active = false, exhausted = false, first = false, seen = false;
  uint32_t p = 0, depth = 0;
  int m = 0;
  Rng rng(0, 0, 0);
  PV prev, next;  // the last stored vertex; the vertex whose ray is traced next
  unsigned long long nr = 0;
  while (true) {
    const unsigned want = __ballot_sync(FULL, !active && !exhausted);
    if (want) {
      const int leader = __ffs(want) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(cursor, (unsigned)__popc(want));
      base = __shfl_sync(FULL, base, leader);
      if (!active && !exhausted) {
        const unsigned r = base + (unsigned)__popc(want & ((1u << lane) - 1));
        if (r < n) {
          p = r;
          rng = Rng(LIGHT ? P.seed : P.seed ^ 0x5bd1e995ull, ((uint64_t)P.iter << 33) | (uint64_t)p, 0);
          next = LIGHT ? emit_start(S, P.cam, rng) : camera_start(S, P.cam, p, rng);
          seen = false;
          m = 0;
          out.put(S, P, p, m++, next, seen);
          depth = 0;
          first = true;
          active = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, active)) break;
    if (!active) continue;
    // the one trace of this iteration
    Hit3 h;
    if (first) {
      h = LIGHT ? emit_hit(S, next) : camera_hit(S, next);
    } else {
      const PHit hh = trace_cond<false>(S, next.o, next.d, INFINITY, next.contact, next.inside);
      h = hh.tid >= 0 ? Hit3{(int)__ldg(&S.tri_obj[hh.tid]), hh.tid, hh.t} : Hit3{kNone, -1, -1.0f};
    }
    bool end = false;
    if (first) {  // the subpath's origin is stored; nothing to scatter from ends it
      if (next.inside == kNone && h.obj == kNone) {
        out.put(S, P, p, m++, pv_term(next.o), seen);
        end = true;
      }
      prev = next;
      first = false;
    } else {
      out.put(S, P, p, m++, next, seen);
      if (h.obj == kNone) {
        out.put(S, P, p, m++, pv_term(prev.o), seen);
        end = true;
      } else {
        prev = next;
        depth++;
      }
    }
    if (!end) {  // scatter from the last vertex: the next ray, or the end of the subpath
      next = scatter_step(S, P.cam, prev, h, light_scatter, true, rng);
      if (length(next.d) < 0.5f) {
        out.put(S, P, p, m++, next, seen);
        end = true;
      } else if (depth + 1 > P.max_depth) {
        out.put(S, P, p, m++, pv_term(prev.o), seen);
        end = true;
      }
    }
    if (end) {
      out.len[p] = m;
      nr += (unsigned long long)m;
      active = false;
    }
  }
  if (nr) atomicAdd(rays, nr);
}

// The light subpaths' records, one thread per path, from the stored vertices (apart from
// the sampling kernel, whose traversal stack and divergent bounce loop would hold them).
__global__ void __launch_bounds__(128) k_light_mis(DevScene S, VcmParams P, const float4* lv, const int* llen,
                                                   MisL* lmis) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_light; p += gridDim.x * blockDim.x)
    light_mis(S, P.cam, lv + 4 * ((size_t)p * P.maxv), llen[p], P.radius, P.norm, !P.bpt, lmis + (size_t)p * P.maxv);
}

// ---- hash grid ---------------------------------------------------------------------------
struct Grid {
  float cell;          // 2 * radius
  unsigned mask;       // buckets - 1
  const unsigned* start;  // bucket -> first sorted photon (exclusive scan), buckets + 1 entries
  const float4* pos;      // photon positions in bucket order
  const int* ref;         // photon light vertices (path * maxv + index) in bucket order
  const float4* join;     // per photon in bucket order, kJoin float4: the light side of a merge
};
// The light side of a merge with a photon at light vertex ci + 1, gathered once per
// photon into bucket order: vertex ci (L, 4 float4), vertex ci - 1 (Lm, 4 float4, zero
// when ci = 0) and L's record (2 float4; MisL::pad carries ci).
constexpr int kJoin = 10;
__device__ __forceinline__ unsigned cell_hash(int x, int y, int z, unsigned mask) {
  return ((unsigned)(x * 73856093) ^ (unsigned)(y * 19349663) ^ (unsigned)(z * 83492791)) & mask;
}
__global__ void k_grid_count(const float4* pos, const unsigned* n_photons, unsigned cap, float cell, unsigned mask,
                             unsigned* count, unsigned* key) {
  unsigned n = min(*n_photons, cap);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 p = pos[i];
    unsigned k = cell_hash((int)floorf(p.x / cell), (int)floorf(p.y / cell), (int)floorf(p.z / cell), mask);
    key[i] = k;
    atomicAdd(&count[k], 1u);
  }
}
__global__ void k_grid_scatter(const unsigned* key, const float4* pos, const int* ref, const unsigned* n_photons,
                               unsigned cap, unsigned* cursor, float4* pos_out, int* ref_out, const float4* lv,
                               const MisL* lmis, uint32_t maxv, float4* join) {
  unsigned n = min(*n_photons, cap);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned slot = atomicAdd(&cursor[key[i]], 1u);
    const int r = ref[i];
    pos_out[slot] = pos[i];
    ref_out[slot] = r;
    const uint32_t lp = (uint32_t)r / maxv, ci = (uint32_t)r % maxv - 1;
    const float4* L = lv + 4 * ((size_t)lp * maxv + ci);
    float4* out = join + (size_t)kJoin * slot;
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = L[k];
    if (ci > 0) {
      const float4* Lm = L - 4;
#pragma unroll
      for (int k = 0; k < 4; k++) out[4 + k] = Lm[k];
    } else {
#pragma unroll
      for (int k = 0; k < 4; k++) out[4 + k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    MisL m = lmis[(size_t)lp * maxv + ci];
    out[8] = make_float4(m.sla, m.tla, m.prob, __int_as_float((int)ci));
    out[9] = make_float4(m.thr.x, m.thr.y, m.thr.z, 0.0f);
  }
}

// ---- the reference's bidirectional machinery over a whole path ----------------------
// VCMTracer::link (src/VCMTracer.cpp:308-319)
__device__ __forceinline__ PV link(const PV* w, int n, int ci, int i, int j) {
  const PV& src = w[min(max(i, 0), n - 1)];
  const PV& dst = w[min(max(j, 0), n - 1)];
  PV r = src;
  if ((j > i && i <= ci) || (j < i && i > ci)) return r;
  r.d = normalize(dst.o - src.o);
  r.inside = dst.inside;
  return r;
}

// MCRenderer::connectRays (src/MCRenderer.cpp:50-106)
__device__ bool connect_rays(const DevScene& S, const CamDev& cam, PV* w, int n, int ci, bool merged) {
  PV& L = w[ci];
  PV& E = w[ci + 1];
  if (!merged && (!(L.flags & kDirRandom) || !(E.flags & kDirRandom))) return false;
  if (merged && !(E.flags & kDirRandom)) return false;
  const PV& pl = w[ci - 1 > 0 ? ci - 1 : 0];
  const PV& pe = w[ci + 2 < n - 1 ? ci + 2 : n - 1];
  L.d = normalize(E.o - L.o);
  E.d = -L.d;
  if (!merged) {
    L.dprob = 1.0f;
    L.c = bsdf_of(S, cam, pl, L);
    L.flags |= kDirRandom;
    if (L.contact != kNone && ci > 0) {
      F3 n0 = contact_normal(S, cam, L);
      if (dot(n0, L.d) <= 0.0f) L.inside = L.contact;
      else if (dot(n0, pl.d) <= 0.0f) L.inside = pl.inside;
      else L.inside = find_inside(S, L.o, L.d, L.contact);
    }
  }
  E.dprob = 1.0f;
  E.c = bsdf_of(S, cam, pe, E);
  E.flags |= kDirRandom;
  if (E.contact != kNone && ci < n - 2) {
    F3 n0 = contact_normal(S, cam, E);
    if (dot(n0, E.d) <= 0.0f) E.inside = E.contact;
    else if (dot(n0, pe.d) <= 0.0f) E.inside = pe.inside;
    else E.inside = find_inside(S, E.o, E.d, E.contact);
  }
  return true;
}

// VCMTracer::connectColorProb (src/VCMTracer.cpp:248-306)
__device__ void connect_color_prob(const DevScene& S, const CamDev& cam, const PV* w, int n, int ci, bool merged,
                                   float r, F3& color, float& prob) {
  color = {1, 1, 1};
  prob = 1.0f;
  for (int i = 0; i < n; i++) {
    color = color * w[i].c;
    float dist = 1e-5f;
    if (i <= ci) {
      dist = fmaxf(length(w[i + 1].o - w[i].o), 1e-5f);
      color = color * decay_of(S, w[i].inside, dist);
    } else if (i > ci + 1) {
      dist = fmaxf(length(w[i - 1].o - w[i].o), 1e-5f);
      color = color * decay_of(S, w[i].inside, dist);
    }
    if (i == ci && i < n - 1) color = color * (cos_term(S, cam, w[i]) * cos_term(S, cam, w[i + 1]) / (dist * dist));
    if (i != ci && i != ci + 1) color = color * cos_term(S, cam, w[i]);
    prob *= w[i].dprob * w[i].oprob;
    if (merged && i == ci) {
      prob *= RX_PI * r * r;
      prob *= cos_term(S, cam, link(w, n, ci, i + 1, i));
      prob /= dist * dist;
      prob *= origin_pdf(S, link(w, n, ci, i, i + 1), link(w, n, ci, i + 1, i + 2));
      if (w[i + 1].inside != kNone && w[i + 1].contact == kNone) prob *= 4.0f / 3.0f * r;
    }
  }
}

__device__ __forceinline__ bool must_use_pt(const PV* w, int n) {
  for (int i = 1; i < n - 1; i++)
    if (w[i].flags & kDirRandom) return false;
  return true;
}
// BidirectionalPathTracer::mustUsePT (src/BidirectionalPathTracer.cpp:115-122): no two
// consecutive vertices sampled at random.
__device__ __forceinline__ bool bpt_must_use_pt(const PV* w, int n) {
  for (int i = 0; i < n - 1; i++)
    if ((w[i].flags & kDirRandom) && (w[i + 1].flags & kDirRandom)) return false;
  return true;
}

// VCMTracer::connectMergeWeight (src/VCMTracer.cpp:321-428), power 1, double precision
// With bpt, BidirectionalPathTracer::connectWeight (src/BidirectionalPathTracer.cpp:198-276,
// exponent 1): no merge techniques and its own mustUsePT.
__device__ float connect_merge_weight(const DevScene& S, const CamDev& cam, const PV* w, int n, int ci, bool merged,
                                      bool bpt, float r, float norm) {
  double pf[2 * kMaxV], pb[2 * kMaxV];
  float dist[2 * kMaxV];
  pf[0] = w[0].oprob;
  for (int i = 0; i < n - 1; i++) {
    pf[i + 1] = pf[i] * cos_term(S, cam, link(w, n, ci, i + 1, i));
    dist[i] = fmaxf(length(w[i + 1].o - w[i].o), 1e-5f);
    pf[i + 1] /= (double)dist[i] * dist[i];
    if (w[i].flags & kDirRandom) {
      if (i > 0) {
        pf[i + 1] *= dir_pdf(S, cam, link(w, n, ci, i - 1, i), link(w, n, ci, i, i + 1), false);
      } else {
        PV ray = link(w, n, ci, i, i + 1);
        pf[i + 1] *= dir_pdf(S, cam, ray, ray, true);
      }
      pf[i + 1] *= origin_pdf(S, link(w, n, ci, i, i + 1), link(w, n, ci, i + 1, i + 2));
    }
  }
  pb[n - 1] = w[n - 1].oprob;
  for (int i = n - 1; i > 0; i--) {
    pb[i - 1] = pb[i] * cos_term(S, cam, link(w, n, ci, i - 1, i));
    pb[i - 1] /= (double)dist[i - 1] * dist[i - 1];
    if (w[i].flags & kDirRandom) {
      if (i < n - 1) {
        pb[i - 1] *= dir_pdf(S, cam, link(w, n, ci, i + 1, i), link(w, n, ci, i, i - 1), false);
      } else {
        PV ray = link(w, n, ci, i, i - 1);
        pb[i - 1] *= dir_pdf(S, cam, ray, ray, true);
      }
      pb[i - 1] *= origin_pdf(S, link(w, n, ci, i, i - 1), link(w, n, ci, i - 1, i - 2));
    }
  }
  double self = ci == -1 ? pb[0] : pf[ci] * pb[ci + 1];
  double sum = 0.0;
  for (int i = 0; i < n - 1; i++) {
    if ((w[i].flags & kDirRandom) && (w[i + 1].flags & kDirRandom)) sum += pf[i] * pb[i + 1];
    if (!bpt && i < n - 2 && (w[i + 1].flags & kDirRandom)) {
      double p = pf[i] * pb[i + 1];
      if (w[i].flags & kDirRandom) {
        if (i > 0) {
          p *= dir_pdf(S, cam, link(w, n, ci, i - 1, i), link(w, n, ci, i, i + 1), false);
        } else {
          PV ray = link(w, n, ci, i, i + 1);
          p *= dir_pdf(S, cam, ray, ray, true);
        }
      }
      p *= origin_pdf(S, link(w, n, ci, i, i + 1), link(w, n, ci, i + 1, i + 2));
      p *= RX_PI * r * r;
      p *= cos_term(S, cam, link(w, n, ci, i + 1, i));
      p /= (double)dist[i] * dist[i];
      if (w[i + 1].inside != kNone && w[i + 1].contact == kNone) p *= 4.0 / 3.0 * r;
      p *= norm;
      sum += p;
      if (merged && ci == i) self = p;
    }
  }
  if (bpt ? bpt_must_use_pt(w, n) : must_use_pt(w, n)) sum += pb[0];
  double res = self / sum;
  if (!(res >= 0.0)) return 0.0f;
  return (float)res;
}

// Camera::transToPixel (src/Camera.cpp:136-152)
__device__ __forceinline__ void trans_to_pixel(const CamDev& c, F3 point, float& px, float& py) {
  F3 v = point - c.pos;
  float fd = dot(v, c.front);
  float ratio = c.sight / fd;
  px = dot(v, c.right) * ratio + c.width / 2.0f - 0.5f;
  py = c.height / 2.0f - dot(v, c.up) * ratio - 0.5f;
}

__device__ __forceinline__ void img_add(float* img, int pixel, F3 c) {
  atomicAdd(img + 3 * pixel, c.x);
  atomicAdd(img + 3 * pixel + 1, c.y);
  atomicAdd(img + 3 * pixel + 2, c.z);
}

// ---- eye subpaths and connections ---------------------------------------------------------
// colorByConnectingPaths (VCMTracer.cpp:430-562) joins every light vertex ci of the
// pixel's light path with every eye vertex k (s = ci + 1, t = k + 1), plus the pure
// eye path (s = 0). k_sub_run samples and stores the eye subpath; k_eye_post
// builds its records, adds the s = 0 technique, and lists which vertices can take part
// in a connection (sampled
// at random, not on an emitter past the light's own vertex); the (k, ci) pairs are then
// evaluated one per lane with their shadow rays (k_conn_eval).

// Per pixel, from its stored eye subpath: the records, the s = 0 technique (the eye
// path ends on an emitter and the reference's mustUsePT holds: VCM, no interior vertex
// sampled at random, weight pb[0] / (pb[0] + the two-vertex connection);
// BidirectionalPathTracer, no two consecutive random vertices, weight pb[0] / pb[0]),
// and the lists of eye and light vertices that can take part in a connection.
__global__ void __launch_bounds__(128) k_eye_post(DevScene S, VcmParams P, const float4* lv, const int* llen,
                                                  const float4* ev, const int* elen, MisE* emis, uint2* cmask,
                                                  unsigned long long* ccount, float* img) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_pixels; p += gridDim.x * blockDim.x) {
    const float4* eb = ev + 4 * ((size_t)p * P.maxv);
    const int ne = elen[p];
    MisE* me = emis + (size_t)p * P.maxv;
    eye_mis(S, P.cam, [&](int k) { return load_pv(eb + 4 * k); }, ne, P.radius, P.norm, !P.bpt, me);
    F3 acc = {0, 0, 0};
    uint32_t em = 0;
    bool rand_interior = false, rand_pair = false, prev_rand = false, first_rand = false, open = true;
    for (int k = 0; k < ne; k++) {
      const PV v = load_pv(eb + 4 * k);
      const bool rv = rnd(v);
      if (k == 0) first_rand = rv;
      if (k >= 1) rand_pair |= prev_rand && rv;  // pairs within e[0..k]
      if (rv && !is_emissive(S, v.contact)) em |= 1u << k;
      if (k >= 1 && open) {  // s = 0 with t = k + 1 (interior e[1..k-1], pairs within e[0..k])
        if (P.bpt ? rand_pair : rand_interior) {
          open = false;
        } else if (is_emissive(S, v.contact)) {
          const MisE m = me[k];
          F3 col = v.c * m.thr;
          float prob = (v.dprob * v.oprob) * m.prob;
          if (prob > 0.0f && length(col) > 0.0f) {
            float wt = m.pb > 0.0 && m.pb < INFINITY ? 1.0f : 0.0f;      // pb[0] / pb[0]
            if (!P.bpt && wt > 0.0f && k == 1 && rv && first_rand) {  // pb[0] / (pb[0] + pf[0] pb[1])
              float res = 1.0f / (1.0f + v.oprob * m.pbr);
              wt = res >= 0.0f ? res : 0.0f;
            }
            F3 c = col * (wt / prob);
            if (length(c) > 0.0f) acc = acc + c;
          }
        }
      }
      if (k >= 1) rand_interior |= rv;  // e[k] is interior for every longer path
      prev_rand = rv;
    }
    img_add(img, (int)p, acc);
    uint32_t lm = 0;
    const uint32_t lp = p % P.n_light;
    const int nl = llen[lp];
    for (int ci = 0; ci < nl; ci++) {
      float4 t4 = lv[4 * ((size_t)lp * P.maxv + ci) + 3];
      int contact = __float_as_int(t4.x);
      uint32_t flags = __float_as_uint(t4.w);
      if ((flags & kDirRandom) && (ci == 0 || !is_emissive(S, contact))) lm |= 1u << ci;
    }
    cmask[p] = make_uint2(em, lm);
    ccount[p] = (unsigned long long)(__popc(em) * __popc(lm));
  }
}

// Pairs [win0, win0 + cap) of the scanned order: pixel and eye vertex (q = p * maxv + k)
// and light vertex of each.
__global__ void k_conn_fill(VcmParams P, const uint2* cmask, const unsigned long long* coff, unsigned long long win0,
                            uint32_t cap, uint32_t* pair_q, int* pair_c) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_pixels; p += gridDim.x * blockDim.x) {
    uint2 m = cmask[p];
    unsigned long long idx = coff[p];
    for (uint32_t em = m.x; em; em &= em - 1) {
      int k = __ffs(em) - 1;
      for (uint32_t lm = m.y; lm; lm &= lm - 1) {
        if (idx >= win0 && idx - win0 < cap) {
          pair_q[idx - win0] = p * P.maxv + (uint32_t)k;
          pair_c[idx - win0] = __ffs(lm) - 1;
        }
        idx++;
      }
    }
  }
}

// A connection's shadow ray (testVisibility) and what it adds when nothing blocks it:
// origin and length, direction and contact object, colour and inside object, pixel.
struct ShadowQ {
  float4 o_len;
  float4 d_contact;
  float4 col_inside;
  int4 pixel;
};

// One connection per lane (runs of kConnRun per thread): the joined path's colour,
// probability and MIS weight from the records; a contribution that is not zero queues its
// shadow ray (testVisibility) in `sq` (one slot per connection at most), and the shadow
// kernel that follows adds it to its pixel when nothing blocks it.
constexpr int kConnRun = 4;
__global__ void __launch_bounds__(128) k_conn_eval(DevScene S, VcmParams P, const float4* lv, const float4* ev,
                                                   const MisL* lmis, const MisE* emis, const uint32_t* pair_q,
                                                   const int* pair_c, uint32_t npairs, float* img,
                                                   unsigned long long* rays, ShadowQ* sq, unsigned* sq_n) {
  const float r = P.radius;
  uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long nrays = 0;
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * kConnRun; base < npairs;
       base += stride * kConnRun) {
    for (uint32_t j = base; j < base + kConnRun && j < npairs; j++) {
      uint32_t q = pair_q[j];
      int ci = pair_c[j];
      int p = (int)(q / P.maxv), k = (int)(q % P.maxv);
      uint32_t lp = (uint32_t)p % P.n_light;
      const float4* lb = lv + 4 * ((size_t)lp * P.maxv);
      const float4* eb = ev + 4 * ((size_t)p * P.maxv);
      const PV L = load_pv(lb + 4 * ci);
      const PV E = load_pv(eb + 4 * k);
      PV Lm, pe, Lp, Ep;
      if (ci > 0) Lm = load_pv(lb + 4 * (ci - 1));
      if (k > 0) pe = load_pv(eb + 4 * (k - 1));
      const MisL ml = lmis[(size_t)lp * P.maxv + ci];
      const MisE me = emis[(size_t)p * P.maxv + k];
      join(S, P.cam, L, ci > 0 ? &Lm : nullptr, E, k > 0 ? &pe : nullptr, false, Lp, Ep);
      F3 col;
      float prob, wt;
      if (!join_eval(S, P.cam, L, ci > 0 ? &Lm : nullptr, Lp, Ep, k > 0 ? &pe : nullptr, ml, me, false, P.bpt, r, P.norm,
                     col, prob, wt))
        continue;
      F3 c = col * (wt / prob);
      if (!(length(c) > 0.0f)) continue;
      float len = length(Ep.o - Lp.o);
      nrays++;
      int target = p;
      if (k == 0) {  // light tracing: splat onto the pixel the light vertex projects to
        F3 dir = normalize(Lp.o - Ep.o);
        float ca = fabsf(dot(P.cam.front, dir));
        float to_solid = P.cam.sight * P.cam.sight / (ca * ca * ca);
        float to_surface = to_solid / ca;
        c = c * (to_surface / (float)P.n_pixels) * ca;
        float px, py;
        trans_to_pixel(P.cam, Lp.o, px, py);
        int ix = (int)px, iy = (int)py;
        target = ix >= 0 && ix < P.cam.width && iy >= 0 && iy < P.cam.height ? iy * P.cam.width + ix : -1;
      }
      if (target < 0) continue;
      // queue the shadow ray (testVisibility): the lanes here take their slots with one
      // atomic
      const unsigned m = __activemask();
      const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
      unsigned slot = 0;
      if (lane == leader) slot = atomicAdd(sq_n, (unsigned)__popc(m));
      slot = __shfl_sync(m, slot, leader) + __popc(m & ((1u << lane) - 1));
      sq[slot] = ShadowQ{make_float4(Ep.o.x, Ep.o.y, Ep.o.z, len - 1e-5f),
                         make_float4(Ep.d.x, Ep.d.y, Ep.d.z, __int_as_float(Ep.contact)),
                         make_float4(c.x, c.y, c.z, __int_as_float(Ep.inside)), make_int4(target, 0, 0, 0)};
    }
  }
  if (nrays) atomicAdd(rays, nrays);
}

// The queued shadow rays on persistent warps over the scene's 4-wide BVH (rx_walk.cuh):
// any legal hit shorter than the connection (NoSelfIntersectionCondition, as trace_cond)
// blocks it; an unblocked connection adds its colour to its pixel.
struct ShadowLane {
  const DevScene& S;
  const ShadowQ* __restrict__ q;
  uint32_t n;
  float* img;
  int contact = kNone, inside = kNone, target = 0;
  bool cond = false, blocked = false;
  float lim = 0.0f;
  F3 col{};

  __device__ bool begin(uint32_t r, F3& o, F3& d) {
    if (r >= n) return false;
    const ShadowQ e = q[r];
    o = F3{e.o_len.x, e.o_len.y, e.o_len.z};
    d = F3{e.d_contact.x, e.d_contact.y, e.d_contact.z};
    lim = e.o_len.w;
    contact = __float_as_int(e.d_contact.w);
    inside = __float_as_int(e.col_inside.w);
    col = F3{e.col_inside.x, e.col_inside.y, e.col_inside.z};
    target = e.pixel.x;
    cond = !(contact == kNone && inside == kNone);
    blocked = false;
    return true;
  }
  __device__ const float4* nodes() const { return S.accel.bvh4; }
  __device__ float limit() const { return lim; }
  __device__ void leaf(int first, int count, F3 o, F3 d) {
    PHit b{-1, lim};
    if (leaf_test<true>(S, first, count, o, d, cond, contact, inside, b)) {
      blocked = true;
      lim = -INFINITY;  // every remaining box and stack entry is pruned
    }
  }
  __device__ void end() {
    if (!blocked) img_add(img, target, col);
  }
};
__global__ void __launch_bounds__(128, 8) k_shadow_wide(DevScene S, const ShadowQ* q, const unsigned* qn, float* img,
                                                        unsigned long long* cursor) {
  ShadowLane L{S, q, *qn, img};
  walk_persistent<4, kShortStack, 64>(L, cursor);
}
// The same, one thread per queued ray over the binary BVH (when the 4-wide tree is too
// deep for the persistent walk's stack).
__global__ void __launch_bounds__(128) k_shadow_thread(DevScene S, const ShadowQ* q, const unsigned* qn, float* img) {
  const uint32_t n = *qn;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ShadowQ e = q[i];
    PHit sh = trace_cond<true>(S, F3{e.o_len.x, e.o_len.y, e.o_len.z}, F3{e.d_contact.x, e.d_contact.y, e.d_contact.z},
                               e.o_len.w, __float_as_int(e.d_contact.w), __float_as_int(e.col_inside.w));
    if (sh.tid < 0) img_add(img, e.pixel.x, F3{e.col_inside.x, e.col_inside.y, e.col_inside.z});
  }
}

// Per pixel: the eye subpath and colorByConnectingPaths by the reference's loops over each
// whole joined path, a shadow ray per connection in the same thread. Kept as the check of
// k_sub_run + k_eye_post + k_conn_eval (RX_VCM_FULL_PATH_MIS, which also samples the
// light subpaths one per thread, k_vcm_light: the same random numbers, so the same
// subpaths as k_sub_run).
__global__ void __launch_bounds__(128) k_vcm_eye_full(DevScene S, VcmParams P, const float4* lv, const int* llen,
                                                 float4* ev, int* elen, MisE* emis, float* img,
                                                 unsigned long long* rays) {
  uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long nrays = 0, nshadow = 0;
  const float r = P.radius;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_pixels; p += stride) {
    Rng rng(P.seed ^ 0x5bd1e995ull, ((uint64_t)P.iter << 33) | (uint64_t)p, 0);
    PV eye[kMaxV];
    PV w[2 * kMaxV];
    Hit3 h;
    PV start = camera_ray(S, P.cam, p, rng, h);
    int ne = sample_path(S, P.cam, start, h, P.max_depth, !P.bpt, rng, [&](int i, const PV& v) { eye[i] = v; });
    nrays += (unsigned long long)ne;
    for (int k = 0; k < ne; k++) store_pv(ev + 4 * ((size_t)p * P.maxv + k), eye[k]);
    elen[p] = ne;
    eye_mis(S, P.cam, [&](int k) { return eye[k]; }, ne, r, P.norm, !P.bpt, emis + (size_t)p * P.maxv);
    F3 acc = {0, 0, 0};
    uint32_t lp = p % P.n_light;
    int nl = llen[lp];
    for (int whole = 2; whole <= ne + nl; whole++) {
      int s0 = whole - ne > 0 ? whole - ne : 0;
      int s1 = whole - 1 < nl ? whole - 1 : nl;
      for (int s = s0; s <= s1; s++) {
        int t = whole - s;
        int n = 0;
        for (int k = 0; k < s; k++) w[n++] = load_pv(lv + 4 * ((size_t)lp * P.maxv + k));
        for (int k = t - 1; k >= 0; k--) w[n++] = eye[k];
        int ci = s - 1;
        if (s == 0 && !is_emissive(S, w[0].contact)) continue;
        if (s == 0 && !(P.bpt ? bpt_must_use_pt(w, n) : must_use_pt(w, n))) continue;
        if (s > 0) {
          if (s > 1 && is_emissive(S, w[ci].contact)) continue;
          if (is_emissive(S, w[ci + 1].contact)) continue;
          if (!connect_rays(S, P.cam, w, n, ci, false)) continue;
          const PV& E = w[ci + 1];
          const PV& L = w[ci];
          float len = length(E.o - L.o);
          nshadow++;
          PHit sh = trace_cond<true>(S, E.o, E.d, len - 1e-5f, E.contact, E.inside);  // testVisibility
          if (sh.tid >= 0) continue;
        }
        F3 col;
        float prob;
        connect_color_prob(S, P.cam, w, n, ci, false, r, col, prob);
        if (!(prob > 0.0f)) continue;
        if (!(length(col) > 0.0f)) continue;
        float wt = connect_merge_weight(S, P.cam, w, n, ci, false, P.bpt, r, P.norm);
        F3 c = col * (wt / prob);
        if (!(length(c) > 0.0f)) continue;
        if (t == 1) {  // light tracing: splat onto the pixel the light vertex projects to
          F3 dir = normalize(w[ci].o - w[ci + 1].o);
          float ca = fabsf(dot(P.cam.front, dir));
          float to_solid = P.cam.sight * P.cam.sight / (ca * ca * ca);
          float to_surface = to_solid / ca;
          c = c * (to_surface / (float)P.n_pixels) * ca;
          float px, py;
          trans_to_pixel(P.cam, w[n - 2].o, px, py);
          int ix = (int)px, iy = (int)py;
          if (ix >= 0 && ix < P.cam.width && iy >= 0 && iy < P.cam.height) img_add(img, iy * P.cam.width + ix, c);
        } else {
          acc = acc + c;
        }
      }
    }
    img_add(img, (int)p, acc);
  }
  if (nrays) atomicAdd(rays, nrays);
  if (nshadow) atomicAdd(rays + 1, nshadow);
}

// ---- merging as a wavefront: queries, (query, photon) pairs, one pair per lane -------
// colorByMergingPaths (VCMTracer.cpp:566-636): eye vertex ei of pixel p (query
// q = p * maxv + ei) merges with every photon closer than r, for ei >= 1 up to the first
// emitter, at vertices sampled at random. The grid walk visits every cell the sphere
// touches (two per axis in exact arithmetic, up to three after rounding of the cell
// divisions), each bucket once.
// Calls range(begin, end) for each distinct bucket of the cells around q.
template <class F>
__device__ __forceinline__ void merge_buckets(const Grid& G, F3 q, float r, F&& range) {
  int x0 = (int)floorf((q.x - r) / G.cell), y0 = (int)floorf((q.y - r) / G.cell), z0 = (int)floorf((q.z - r) / G.cell);
  int x1 = min((int)floorf((q.x + r) / G.cell), x0 + 2), y1 = min((int)floorf((q.y + r) / G.cell), y0 + 2);
  int z1 = min((int)floorf((q.z + r) / G.cell), z0 + 2);
  unsigned seen[27];
  int nseen = 0;
  for (int cx = x0; cx <= x1; cx++)
    for (int cy = y0; cy <= y1; cy++)
      for (int cz = z0; cz <= z1; cz++) {
        unsigned b = cell_hash(cx, cy, cz, G.mask);
        bool dup = false;
        for (int k = 0; k < nseen; k++) dup |= seen[k] == b;
        if (dup || nseen >= 27) continue;
        seen[nseen++] = b;
        range(G.start[b], G.start[b + 1]);
      }
}
template <class F>
__device__ __forceinline__ void merge_walk(const Grid& G, F3 q, float r, F&& visit) {
  merge_buckets(G, q, r, [&](unsigned b0, unsigned b1) {
    for (unsigned i = b0; i < b1; i++)
      if (length(q - f3(G.pos[i])) < r) visit(G.ref[i]);
  });
}

// The merge position of query q, or false if the eye vertex does not merge.
__device__ __forceinline__ bool merge_query(const DevScene& S, const VcmParams& P, const float4* ev, const int* elen,
                                            uint32_t q, F3& pos) {
  uint32_t p = q / P.maxv;
  int ei = (int)(q % P.maxv);
  if (p >= P.n_pixels || ei < 1 || ei >= elen[p]) return false;
  for (int k = 1; k <= ei; k++) {
    PV v = load_pv(ev + 4 * ((size_t)p * P.maxv + k));
    if (is_emissive(S, v.contact)) return false;  // the loop stops at the first emitter
    if (k == ei) {
      if (!(v.flags & kDirRandom)) return false;
      pos = v.o;
    }
  }
  return true;
}

__global__ void k_merge_count(DevScene S, VcmParams P, const float4* ev, const int* elen, Grid G,
                              unsigned long long* qcount, uint32_t nq) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    F3 pos;
    unsigned long long c = 0;
    if (merge_query(S, P, ev, elen, q, pos)) merge_walk(G, pos, P.radius, [&](int) { c++; });
    qcount[q] = c;
  }
}

// Pairs [win0, win0 + cap) of the scanned order: query and photon of each.
__global__ void k_merge_fill(DevScene S, VcmParams P, const float4* ev, const int* elen, Grid G,
                             const unsigned long long* qoff, uint32_t nq, unsigned long long win0, uint32_t cap,
                             uint32_t* pair_q, int* pair_ref) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    F3 pos;
    if (!merge_query(S, P, ev, elen, q, pos)) continue;
    unsigned long long idx = qoff[q];
    merge_walk(G, pos, P.radius, [&](int ref) {
      if (idx >= win0 && idx - win0 < cap) {
        pair_q[idx - win0] = q;
        pair_ref[idx - win0] = ref;
      }
      idx++;
    });
  }
}

// The contribution of merging eye vertex E (pe before it, records me) with the photon
// whose light side is `jd` (kJoin float4): the photon's predecessor L = w[ci] is joined
// with E as connectRays does for a merge, then colour, probability and MIS weight from
// the records (zero where the reference drops the path).
__device__ __forceinline__ F3 merge_pair(const DevScene& S, const VcmParams& P, const float4* jd, const PV& E,
                                         const PV& pe, const MisE& me) {
  const PV L = load_pv(jd);
  const float4 m0 = jd[8], m1 = jd[9];
  const int ci = __float_as_int(m0.w);
  MisL ml;
  ml.sla = m0.x;
  ml.tla = m0.y;
  ml.prob = m0.z;
  ml.thr = f3(m1);
  PV Lm, Lp, Ep;
  if (ci > 0) Lm = load_pv(jd + 4);
  join(S, P.cam, L, ci > 0 ? &Lm : nullptr, E, &pe, true, Lp, Ep);
  F3 col;
  float prob, wt;
  if (!join_eval(S, P.cam, L, ci > 0 ? &Lm : nullptr, Lp, Ep, &pe, ml, me, true, false, P.radius, P.norm, col, prob,
                 wt))
    return F3{0, 0, 0};
  return col * (wt / prob) * (1.0f / P.norm);
}

// The iteration's merge queries in spatial order. A query is an eye vertex that merges
// (colorByMergingPaths, VCMTracer.cpp:566-636: vertex ei >= 1 of the pixel's eye path,
// sampled at random, before the first emitter); its key is the Morton code of its
// position on a 64^3 grid over the scene bounds, so that the counting sort by key
// (k_ray_scatter) puts queries that gather the same photons next to each other.
__device__ __forceinline__ uint32_t spread6(uint32_t v) {  // 6 bits -> every third bit
  uint32_t r = 0;
#pragma unroll
  for (int b = 0; b < 6; b++) r |= ((v >> b) & 1u) << (3 * b);
  return r;
}
__global__ void __launch_bounds__(128) k_merge_queries(DevScene S, VcmParams P, const float4* ev, const int* elen,
                                                       uint32_t* qlist, uint32_t* qkey, uint32_t* hist,
                                                       unsigned* count) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const DevAccel& A = S.accel;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t iters = (P.n_pixels + stride - 1) / stride;
  for (uint32_t it = 0; it < iters; it++) {
    const uint32_t p = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const int ne = p < P.n_pixels ? elen[p] : 0;
    int nmax = ne;
    for (int s2 = 16; s2 > 0; s2 >>= 1) nmax = max(nmax, __shfl_xor_sync(FULL, nmax, s2));
    bool stop = false;
    for (int k = 1; k < nmax; k++) {
      bool valid = false;
      F3 x{};
      if (k < ne && !stop) {
        const float4* eb = ev + 4 * ((size_t)p * P.maxv + k);
        const float4 o4 = eb[0], t4 = eb[3];
        if (is_emissive(S, __float_as_int(t4.x))) stop = true;  // the merge loop stops at the first emitter
        else if (__float_as_uint(t4.w) & kDirRandom) valid = true, x = f3(o4);
      }
      const unsigned m = __ballot_sync(FULL, valid);
      if (!m) continue;
      const int leader = __ffs(m) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (valid) {
        const float xs[3] = {x.x, x.y, x.z};
        uint32_t key = 0;
#pragma unroll
        for (int a2 = 0; a2 < 3; a2++) {
          const float u = (xs[a2] - A.lo[a2]) / fmaxf(A.hi[a2] - A.lo[a2], 1e-20f) * 64.0f;
          key |= spread6((uint32_t)fminf(fmaxf(u, 0.0f), 63.0f)) << a2;
        }
        const unsigned slot = base + __popc(m & lt);
        qlist[slot] = p * P.maxv + (uint32_t)k;
        qkey[slot] = key;
        atomicAdd(&hist[key], 1u);
      }
    }
  }
}

// Merge pairs (colorByMergingPaths, VCMTracer.cpp:566-636), one warp per query of the
// spatially sorted list, positions [j0, j1): the 32 lanes hash the cells the sphere
// touches, and the warp walks each distinct bucket 128 sorted photons per step
// (coalesced positions, the strict |p - x| < r test), appending the photons inside as
// (query, photon slot in bucket order) pairs with one atomic per step. Pairs past `cap`
// are counted, not written (the host then grows the list or splits the range). Queries
// taken in spatial order make the pairs that follow one another gather the same photons.
__global__ void __launch_bounds__(256) k_merge_walk(VcmParams P, const float4* ev, Grid G, const uint32_t* qlist,
                                                    const uint32_t* order, uint32_t j0, uint32_t j1,
                                                    unsigned long long cap, uint32_t* pair_q, int* pair_ref,
                                                    unsigned long long* npairs) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const float r = P.radius;
  for (uint32_t j = j0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); j < j1; j += nw) {
    {
      const uint32_t q = __ldg(&qlist[__ldg(&order[j])]);
      const F3 x = f3(ev[4 * (size_t)q]);  // vertex q % maxv of pixel q / maxv
      // the cells the sphere touches (as merge_buckets), one per lane; equal buckets are
      // walked once, by the lowest lane that holds them
      const int x0 = (int)floorf((x.x - r) / G.cell), y0 = (int)floorf((x.y - r) / G.cell);
      const int z0 = (int)floorf((x.z - r) / G.cell);
      const int nx = min((int)floorf((x.x + r) / G.cell), x0 + 2) - x0 + 1;
      const int ny = min((int)floorf((x.y + r) / G.cell), y0 + 2) - y0 + 1;
      const int nz = min((int)floorf((x.z + r) / G.cell), z0 + 2) - z0 + 1;
      const bool cell_lane = lane < nx * ny * nz;
      unsigned bucket = 0xffffffffu, b0 = 0, b1 = 0;
      if (cell_lane) {
        const int cz = lane % nz, cy = (lane / nz) % ny, cx = lane / (nz * ny);
        bucket = cell_hash(x0 + cx, y0 + cy, z0 + cz, G.mask);
      }
      const unsigned peers = __match_any_sync(0xffffffffu, bucket);
      const bool leader = cell_lane && (unsigned)(__ffs(peers) - 1) == (unsigned)lane;
      if (leader) {
        b0 = G.start[bucket];
        b1 = G.start[bucket + 1];
      }
      for (unsigned lead = __ballot_sync(0xffffffffu, leader && b1 > b0); lead; lead &= lead - 1) {
        const int src = __ffs(lead) - 1;
        const unsigned r0 = __shfl_sync(0xffffffffu, b0, src), r1 = __shfl_sync(0xffffffffu, b1, src);
        for (unsigned i0 = r0; i0 < r1; i0 += 128) {
          bool h[4];
          unsigned m[4], n = 0;
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const unsigned i = i0 + 32 * u + lane;
            h[u] = i < r1 && length(x - f3(G.pos[i])) < r;
          }
#pragma unroll
          for (int u = 0; u < 4; u++) {
            m[u] = __ballot_sync(0xffffffffu, h[u]);
            n += __popc(m[u]);
          }
          if (n == 0) continue;
          unsigned long long base = 0;
          if (lane == 0) base = atomicAdd(npairs, (unsigned long long)n);
          base = __shfl_sync(0xffffffffu, base, 0);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            if (h[u]) {
              const unsigned long long slot = base + __popc(m[u] & lt);
              if (slot < cap) {
                pair_q[slot] = q;
                pair_ref[slot] = (int)(i0 + 32 * u + lane);
              }
            }
            base += __popc(m[u]);
          }
        }
      }
    }
  }
}

// One merge pair per lane, kRun consecutive pairs per thread (pairs of one query are
// appended together, so the eye vertex and its records are loaded once per query and
// contributions summed per pixel before the image atomics).
constexpr int kRun = 8;
__global__ void __launch_bounds__(128) k_merge_eval(DevScene S, VcmParams P, const float4* ev, const MisE* emis,
                                                    const float4* join, const uint32_t* pair_q, const int* pair_slot,
                                                    uint32_t npairs, float* img) {
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * kRun; base < npairs; base += stride * kRun) {
    F3 acc = {0, 0, 0};
    uint32_t cur = 0xffffffffu;
    PV E, pe;
    MisE me;
    for (uint32_t j = base; j < base + kRun && j < npairs; j++) {
      const uint32_t q = pair_q[j];
      if (q != cur) {
        if (cur != 0xffffffffu) img_add(img, (int)(cur / P.maxv), acc);
        acc = {0, 0, 0};
        cur = q;
        const uint32_t p = q / P.maxv, k = q % P.maxv;
        const float4* eb = ev + 4 * ((size_t)p * P.maxv);
        E = load_pv(eb + 4 * k);
        pe = load_pv(eb + 4 * (k - 1));
        me = emis[q];
      }
      acc = acc + merge_pair(S, P, join + (size_t)kJoin * pair_slot[j], E, pe, me);
    }
    if (cur != 0xffffffffu) img_add(img, (int)(cur / P.maxv), acc);
  }
}

// Merge pairs evaluated by the reference's loops over the whole joined path
// (connectRays, connectColorProb, connectMergeWeight): O(path length) per pair, with the
// path in a per-thread array. Kept as the check of k_merge_eval (RX_VCM_FULL_PATH_MIS).
__global__ void __launch_bounds__(128) k_merge_eval_full(DevScene S, VcmParams P, const float4* lv, const float4* ev,
                                                         const uint32_t* pair_q, const int* pair_ref, uint32_t npairs,
                                                         float* img) {
  const float r = P.radius;
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * kRun; base < npairs; base += stride * kRun) {
    F3 acc = {0, 0, 0};
    int acc_pixel = -1;
    for (uint32_t j = base; j < base + kRun && j < npairs; j++) {
      uint32_t q = pair_q[j];
      int ref = pair_ref[j];
      int p = (int)(q / P.maxv), ei = (int)(q % P.maxv);
      int lp = ref / (int)P.maxv, li = ref % (int)P.maxv;
      PV w[2 * kMaxV];
      int n = 0;
      for (int k = 0; k < li; k++) w[n++] = load_pv(lv + 4 * ((size_t)lp * P.maxv + k));
      for (int k = ei; k >= 0; k--) w[n++] = load_pv(ev + 4 * ((size_t)p * P.maxv + k));
      int ci = li - 1;
      if (!connect_rays(S, P.cam, w, n, ci, true)) continue;
      F3 col;
      float prob;
      connect_color_prob(S, P.cam, w, n, ci, true, r, col, prob);
      if (length(col) == 0.0f || prob == 0.0f) continue;
      float wt = connect_merge_weight(S, P.cam, w, n, ci, true, false, r, P.norm);
      F3 c = col * (wt / prob) * (1.0f / P.norm);
      if (p != acc_pixel) {
        if (acc_pixel >= 0) img_add(img, acc_pixel, acc);
        acc = {0, 0, 0};
        acc_pixel = p;
      }
      acc = acc + c;
    }
    if (acc_pixel >= 0) img_add(img, acc_pixel, acc);
  }
}

// MCRenderer::eliminateVignetting on the iteration image, then the running mean's sum.
__global__ void k_vcm_accumulate(VcmParams P, const float* img, double* film) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_pixels; p += gridDim.x * blockDim.x) {
    int x = p % P.cam.width, y = p / P.cam.width;
    F3 dc = cam_dir(P.cam, x + 0.5f, y + 0.5f);
    float v = fabsf(dot(dc, P.cam.front));
    for (int c = 0; c < 3; c++) {
      const double a = (double)(img[3 * p + c] / v);
      if (isfinite(a)) film[3 * p + c] += a;  // a non-finite value (a zero-density sample) is dropped
    }
  }
}

// ---- PhotonMap (src/Photonmap.cpp) --------------------------------------------------------
// Progressive photon mapping with ray marching through media, as PhotonMap::renderPixels
// runs it (rayMarching is always on there): per iteration W x H light paths deposit
// photons at their random vertices up to the first emitter (surface photons, OUTVOL, and
// in-medium photons, INVOL); each eye path (sampleMergePath: eye-path scattering, at most
// MERGE_LEN bounces, passing straight through media) gathers at its first random surface
// vertex and, along every segment inside a homogeneous medium, at ray-marching steps of
// the medium's stepSize, with the kernel 3 (1 - d^2/r^2)^2 / pi over N r^2 (surface) or
// N r^3 (medium). Photons share the VCM hash grid.
constexpr int kPmMergeLen = 10;           // MERGE_LEN (Photonmap.cpp:7)
constexpr int kPmMaxV = kPmMergeLen + 3;  // rays of an eye merge path, with its terminator
constexpr uint32_t kOutVol = 0u, kInVol = 1u;  // Ray::PhotonType OUTVOL / INVOL
constexpr int kPmData = 5;                // per photon: the photon ray (4 float4), its power
__device__ __forceinline__ F3 fdiv(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }

// Light paths and photons (Photonmap.cpp:55-86): the photon at light vertex i carries
// prod_{k<i} colour_k / directionProb_k / originProb_k x cosine_k x transmittance_k over
// originProb_i (Photonmap.cpp:229-236), and its ray with the arriving direction.
__global__ void __launch_bounds__(128) k_pm_light(DevScene S, VcmParams P, float4* ph_pos, float4* ph_data,
                                                  unsigned* n_photons, unsigned cap, unsigned long long* rays) {
  uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long nr = 0;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P.n_light; p += stride) {
    Rng rng(P.seed, ((uint64_t)P.iter << 33) | (uint64_t)p, 0);
    Hit3 h;
    PV start = emit_ray(S, P.cam, rng, h);
    PV prev = start;
    F3 thr = {1, 1, 1};
    bool stop = false;
    int n = sample_path(S, P.cam, start, h, P.max_depth, true, rng, [&](int i, const PV& v) {
      if (i > 0) {
        thr = thr * fdiv(fdiv(prev.c, prev.dprob), prev.oprob);
        thr = thr * cos_term(S, P.cam, prev);
        thr = thr * decay_of(S, prev.inside, length(prev.o - v.o));
        if (!stop && is_emissive(S, v.contact)) stop = true;  // light is not reflective
        if (!stop && (v.flags & kDirRandom)) {
          unsigned slot = atomicAdd(n_photons, 1u);
          if (slot < cap) {
            const bool in_vol = v.contact == kNone && is_vpm(S, v.inside);
            ph_pos[slot] = make_float4(v.o.x, v.o.y, v.o.z, __uint_as_float(in_vol ? kInVol : kOutVol));
            PV ray = v;
            ray.d = prev.d;
            store_pv(ph_data + (size_t)kPmData * slot, ray);
            F3 pw = fdiv(thr, v.oprob);
            ph_data[(size_t)kPmData * slot + 4] = make_float4(pw.x, pw.y, pw.z, 0.0f);
          }
        }
      }
      prev = v;
    });
    nr += (unsigned long long)n;
  }
  if (nr) atomicAdd(rays, nr);
}

__global__ void k_pm_scatter(const unsigned* key, const float4* pos, const float4* data, const unsigned* n_photons,
                             unsigned cap, unsigned* cursor, float4* pos_out, float4* data_out) {
  unsigned n = min(*n_photons, cap);
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned slot = atomicAdd(&cursor[key[i]], 1u);
    pos_out[slot] = pos[i];
#pragma unroll
    for (int k = 0; k < kPmData; k++) data_out[(size_t)kPmData * slot + k] = data[(size_t)kPmData * i + k];
  }
}

// Bounding boxes of the surface and the medium photons (HashGrid::Build): a query
// outside its grid's box finds nothing (Hashgrid.h Process). Floats as order-preserving
// integers for the atomics; box = {min xyz, max xyz} per type.
__device__ __forceinline__ int ordered(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unordered(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }
__global__ void k_pm_box_init(int* box) {
  if (threadIdx.x < 12) box[threadIdx.x] = (threadIdx.x % 6) < 3 ? INT_MAX : INT_MIN;
}
__global__ void k_pm_box(const float4* pos, const unsigned* n_photons, unsigned cap, int* box) {
  unsigned n = min(*n_photons, cap);
  int m[12];
#pragma unroll
  for (int k = 0; k < 12; k++) m[k] = (k % 6) < 3 ? INT_MAX : INT_MIN;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 q = pos[i];
    const int t = __float_as_uint(q.w) == kInVol ? 6 : 0;
    const int v[3] = {ordered(q.x), ordered(q.y), ordered(q.z)};
#pragma unroll
    for (int k = 0; k < 3; k++) {  // per type, unrolled so that m stays in registers
      if (t == 0) {
        m[k] = min(m[k], v[k]);
        m[3 + k] = max(m[3 + k], v[k]);
      } else {
        m[6 + k] = min(m[6 + k], v[k]);
        m[9 + k] = max(m[9 + k], v[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 12; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      const int w = __shfl_xor_sync(0xffffffffu, m[k], o);
      m[k] = (k % 6) < 3 ? min(m[k], w) : max(m[k], w);
    }
    if ((threadIdx.x & 31) == 0) {
      if ((k % 6) < 3) atomicMin(box + k, m[k]);
      else atomicMax(box + k, m[k]);
    }
  }
}

// The density estimate at x of the photons of one type (Photonmap.cpp:211-259), for the
// out ray `out` (the eye side), by the whole warp: lane j hashes the j-th cell the sphere
// touches (as merge_buckets), equal buckets are walked once (by their lowest lane), and
// the lanes split each bucket's photons. Every lane returns its partial sum.
__device__ F3 pm_gather(const DevScene& S, const CamDev& cam, const Grid& G, const float4* pdata, const int* box,
                        F3 x, const PV& out, uint32_t type, float r, float nph, int lane) {
  const int* b = box + 6 * type;
  if (x.x < unordered(b[0]) || x.y < unordered(b[1]) || x.z < unordered(b[2]) || x.x > unordered(b[3]) ||
      x.y > unordered(b[4]) || x.z > unordered(b[5]))
    return F3{0, 0, 0};
  const int x0 = (int)floorf((x.x - r) / G.cell), y0 = (int)floorf((x.y - r) / G.cell);
  const int z0 = (int)floorf((x.z - r) / G.cell);
  const int nx = min((int)floorf((x.x + r) / G.cell), x0 + 2) - x0 + 1;
  const int ny = min((int)floorf((x.y + r) / G.cell), y0 + 2) - y0 + 1;
  const int nz = min((int)floorf((x.z + r) / G.cell), z0 + 2) - z0 + 1;
  const bool cell_lane = lane < nx * ny * nz;
  unsigned bucket = 0xffffffffu, b0 = 0, b1 = 0;
  if (cell_lane) bucket = cell_hash(x0 + lane / (nz * ny), y0 + (lane / nz) % ny, z0 + lane % nz, G.mask);
  const unsigned peers = __match_any_sync(0xffffffffu, bucket);
  const bool leader = cell_lane && (unsigned)(__ffs(peers) - 1) == (unsigned)lane;
  if (leader) {
    b0 = G.start[bucket];
    b1 = G.start[bucket + 1];
  }
  F3 contrib = {0, 0, 0};
  const float r2 = r * r;
  const float norm = type == kInVol ? nph * r * r * r : nph * r * r;
  for (unsigned lead = __ballot_sync(0xffffffffu, leader && b1 > b0); lead; lead &= lead - 1) {
    const int src = __ffs(lead) - 1;
    const unsigned r0 = __shfl_sync(0xffffffffu, b0, src), r1 = __shfl_sync(0xffffffffu, b1, src);
    for (unsigned i = r0 + (unsigned)lane; i < r1; i += 32) {
      const float4 q = G.pos[i];
      if (__float_as_uint(q.w) != type) continue;
      const float dist = length(x - f3(q));
      const float d2 = dist * dist;
      if (!(d2 <= r2)) continue;
      const float4* pd = pdata + (size_t)kPmData * i;
      const PV ray = load_pv(pd);
      const F3 color = f3(pd[4]) * bsdf_of(S, cam, ray, out);
      if (lum(color) < 1e-6f) continue;
      const float sk = fmaxf(0.0f, 1.0f - d2 / r2);
      const float kernel = 3.0f * sk * sk / RX_PI;
      contrib = contrib + color * (kernel / norm);
    }
  }
  return contrib;
}

// The same estimate by one lane alone (the medium gathers, one ray-marching step per
// lane: their spheres hold few photons each).
__device__ F3 pm_gather_lane(const DevScene& S, const CamDev& cam, const Grid& G, const float4* pdata, const int* box,
                             F3 x, const PV& out, uint32_t type, float r, float nph) {
  const int* b = box + 6 * type;
  if (x.x < unordered(b[0]) || x.y < unordered(b[1]) || x.z < unordered(b[2]) || x.x > unordered(b[3]) ||
      x.y > unordered(b[4]) || x.z > unordered(b[5]))
    return F3{0, 0, 0};
  F3 contrib = {0, 0, 0};
  const float r2 = r * r;
  const float norm = type == kInVol ? nph * r * r * r : nph * r * r;
  merge_buckets(G, x, r, [&](unsigned b0, unsigned b1) {
    for (unsigned i = b0; i < b1; i++) {
      const float4 q = G.pos[i];
      if (__float_as_uint(q.w) != type) continue;
      const float dist = length(x - f3(q));
      const float d2 = dist * dist;
      if (!(d2 <= r2)) continue;
      const float4* pd = pdata + (size_t)kPmData * i;
      const PV ray = load_pv(pd);
      const F3 color = f3(pd[4]) * bsdf_of(S, cam, ray, out);
      if (lum(color) < 1e-6f) continue;
      const float sk = fmaxf(0.0f, 1.0f - d2 / r2);
      const float kernel = 3.0f * sk * sk / RX_PI;
      contrib = contrib + color * (kernel / norm);
    }
  });
  return contrib;
}

// One warp per pixel: lane 0 samples the eye merge path into shared memory, then the
// lanes share the ray-marching steps of each medium segment (one gather per lane) and
// split the photons of the gather at the first random surface vertex.
__global__ void __launch_bounds__(128) k_pm_eye(DevScene S, VcmParams P, Grid G, const float4* pdata, const int* box,
                                                float* img, unsigned long long* rays) {
  __shared__ float4 paths[4][kPmMaxV * 4];
  const int lane = threadIdx.x & 31;
  float4* sp = paths[threadIdx.x >> 5];
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  const float r = P.radius;
  unsigned long long nr = 0;
  for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < P.n_pixels; p += nw) {
    Rng rng(P.seed ^ 0x5bd1e995ull, ((uint64_t)P.iter << 33) | (uint64_t)p, 0);
    int n = 0;
    if (lane == 0) {  // PhotonMap::sampleMergePath (Photonmap.cpp:142-187)
      Hit3 h;
      PV prev = camera_ray(S, P.cam, p, rng, h);
      for (int depth = 0;; depth++) {
        store_pv(sp + 4 * n++, prev);
        PV next;
        if (prev.inside != kNone && !is_vpm(S, prev.inside)) {
          next = scatter_object(S, P.cam, prev.inside, prev, h, false, true, rng);
        } else if (h.obj != kNone) {
          PV in = prev;
          Hit3 hh = h;
          if (is_vpm(S, h.obj) && prev.contact >= 0 && is_vpm(S, prev.contact)) {  // straight through the medium
            in.o = prev.o + prev.d * h.dist;
            hh.dist = 0.0f;
          }
          next = scatter_object(S, P.cam, h.obj, in, hh, false, true, rng);
        } else {
          store_pv(sp + 4 * n++, pv_term(prev.o));
          break;
        }
        if (length(next.d) < 0.5f) {
          store_pv(sp + 4 * n++, next);
          break;
        }
        if (depth + 1 > kPmMergeLen) {
          store_pv(sp + 4 * n++, pv_term(prev.o));
          break;
        }
        PHit t = trace_cond<false>(S, next.o, next.d, INFINITY, next.contact, next.inside);
        if (t.tid < 0) {
          store_pv(sp + 4 * n++, next);
          store_pv(sp + 4 * n++, pv_term(prev.o));
          break;
        }
        h = Hit3{(int)__ldg(&S.tri_obj[t.tid]), t.tid, t.t};
        prev = next;
      }
      nr += (unsigned long long)n;
    }
    n = __shfl_sync(0xffffffffu, n, 0);
    __syncwarp();
    // PhotonMap::throughputByDensityEstimation (Photonmap.cpp:262-386), rayMarching on
    F3 Tr = {1, 1, 1}, surf = {0, 0, 0}, vol = {0, 0, 0};
    for (int i = 1; i < n; i++) {
      const PV a = load_pv(sp + 4 * (i - 1)), b = load_pv(sp + 4 * i);
      const float dist = fmaxf(length(a.o - b.o), 1e-5f);
      if (is_vpm(S, a.inside)) {
        const float step_size = S.objects[a.inside].step_size;
        int N = (int)(dist / step_size);
        if (N == 0) N++;
        const float step = dist / (float)N;
        float u = 0.0f;
        if (lane == 0) u = rng.next();
        const float offset = step * __shfl_sync(0xffffffffu, u, 0);
        Tr = Tr * decay_of(S, a.inside, offset);
        for (int j = lane; j < N; j += 32) {  // one step per lane; Tr after step j in closed form
          PV out = a;
          out.d = -a.d;
          out.o = a.o + a.d * (offset + step * (float)j);
          out.contact = kNone;
          const F3 c = pm_gather_lane(S, P.cam, G, pdata, box, out.o, out, kInVol, r, P.norm);
          vol = vol + c * (Tr * decay_of(S, a.inside, step * (float)(j + 1))) * step;
        }
        Tr = Tr * decay_of(S, a.inside, step * (float)N);
      } else if (a.inside != kNone) {
        Tr = Tr * decay_of(S, a.inside, dist);
      }
      if (is_emissive(S, b.contact)) {  // the eye path hit a light: its radiance (lane 0's share)
        surf = lane == 0 ? b.c : F3{0, 0, 0};
        break;
      }
      if (b.contact != kNone && rnd(b)) {
        if (is_vpm(S, b.contact)) continue;
        PV out = b;
        out.d = -a.d;
        surf = pm_gather(S, P.cam, G, pdata, box, b.o, out, kOutVol, r, P.norm, lane);
        break;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      vol.x += __shfl_xor_sync(0xffffffffu, vol.x, o);
      vol.y += __shfl_xor_sync(0xffffffffu, vol.y, o);
      vol.z += __shfl_xor_sync(0xffffffffu, vol.z, o);
      surf.x += __shfl_xor_sync(0xffffffffu, surf.x, o);
      surf.y += __shfl_xor_sync(0xffffffffu, surf.y, o);
      surf.z += __shfl_xor_sync(0xffffffffu, surf.z, o);
    }
    if (lane == 0) {
      const PV e0 = load_pv(sp);
      F3 color = Tr * surf + vol;
      color = color * fdiv(fdiv(cos_term(S, P.cam, e0) * e0.c, e0.dprob), e0.oprob);
      img[3 * p] = color.x;
      img[3 * p + 1] = color.y;
      img[3 * p + 2] = color.z;
    }
    __syncwarp();
  }
  if (lane == 0 && nr) atomicAdd(rays, nr);
}

// ---- host driver -----------------------------------------------------------------------
// The camera frame of Camera (src/Camera.cpp): front, right and up from position, focus
// and up, integer sightDist.
static VcmParams camera_params(const rx_camera& cam) {
  VcmParams P{};
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
  P.focus = foc;
  P.n_pixels = cam.width * cam.height;
  return P;
}

// Photons stored in this iteration's grid (the stored count, clipped to the capacity),
// added to a running total.
__global__ void k_count_photons(const unsigned* nph, unsigned cap, unsigned long long* total) {
  *total += (unsigned long long)min(*nph, cap);
}

cudaError_t render_vcm(rx_context* c, const rx_camera& cam, const rx_vcm_options& opt, double* film,
                       rx_render_stats* stats, cudaStream_t s) {
  const DevScene& S = c->scene;
  VcmParams P = camera_params(cam);
  P.seed = opt.seed;
  P.max_depth = opt.max_depth;
  P.maxv = opt.max_depth + 3;
  P.n_pixels = cam.width * cam.height;
  P.bpt = (opt.flags & kVcmBidirectional) ? 1u : 0u;
  P.n_light = opt.light_paths && !P.bpt ? opt.light_paths : P.n_pixels;  // BPT: one light path per pixel
  P.norm = (float)P.n_light;
  const unsigned cap = P.bpt ? 1u : P.n_light * P.maxv;  // photon capacity (none without merging)
  unsigned buckets = 1u << 16;
  while (buckets < cap && buckets < (1u << 26)) buckets <<= 1;
  std::vector<DevBuf> bufs(33);
  cudaError_t e;
  auto al = [&](int k, size_t bytes) { return bufs[k].alloc(bytes); };
  if ((e = al(26, 16)) != cudaSuccess) return e;  // subpath cursors
  if ((e = al(0, (size_t)P.n_light * P.maxv * 4 * sizeof(float4))) != cudaSuccess) return e;  // light vertices
  if ((e = al(1, (size_t)P.n_light * sizeof(int))) != cudaSuccess) return e;
  if ((e = al(2, (size_t)cap * sizeof(float4))) != cudaSuccess) return e;                      // photon positions
  if ((e = al(3, (size_t)cap * sizeof(int))) != cudaSuccess) return e;
  if ((e = al(4, (size_t)cap * sizeof(unsigned))) != cudaSuccess) return e;                     // photon keys
  if ((e = al(5, (size_t)cap * sizeof(int))) != cudaSuccess) return e;                          // sorted ids
  if ((e = al(6, (size_t)(buckets + 1) * sizeof(unsigned))) != cudaSuccess) return e;           // counts
  if ((e = al(7, (size_t)(buckets + 1) * sizeof(unsigned))) != cudaSuccess) return e;           // start
  if ((e = al(8, (size_t)(buckets + 1) * sizeof(unsigned))) != cudaSuccess) return e;           // cursor
  if ((e = al(9, ((buckets + 1) / 1024 + 2) * sizeof(unsigned))) != cudaSuccess) return e;      // block sums
  if ((e = al(10, (size_t)P.n_pixels * 3 * sizeof(float))) != cudaSuccess) return e;            // iteration image
  if ((e = al(11, 64 * sizeof(unsigned long long))) != cudaSuccess) return e;                   // counters
  const uint32_t nq = P.n_pixels * P.maxv;                                                       // merge queries
  const unsigned nqblk = (nq + 1023) / 1024;
  if ((e = al(12, (size_t)P.n_pixels * P.maxv * 4 * sizeof(float4))) != cudaSuccess) return e;  // eye vertices
  if ((e = al(13, (size_t)P.n_pixels * sizeof(int))) != cudaSuccess) return e;                   // eye lengths
  if ((e = al(14, (size_t)nq * sizeof(unsigned long long))) != cudaSuccess) return e;            // query counts
  if ((e = al(15, (size_t)nq * sizeof(unsigned long long))) != cudaSuccess) return e;            // query offsets
  if ((e = al(16, ((size_t)nqblk + 2) * sizeof(unsigned long long))) != cudaSuccess) return e;  // block sums
  if ((e = al(19, (size_t)P.n_light * P.maxv * sizeof(MisL))) != cudaSuccess) return e;         // light MIS records
  if ((e = al(20, (size_t)P.n_pixels * P.maxv * sizeof(MisE))) != cudaSuccess) return e;        // eye MIS records
  if ((e = al(21, (size_t)P.n_pixels * sizeof(uint2))) != cudaSuccess) return e;                // connection masks
  if ((e = al(22, (size_t)cap * sizeof(float4))) != cudaSuccess) return e;                      // sorted photon positions
  if ((e = al(23, (size_t)cap * kJoin * sizeof(float4))) != cudaSuccess) return e;              // photon join data
  if (!P.bpt) {  // merge queries in spatial order: list, keys, sorted order, key counts, count
    if ((e = al(27, (size_t)nq * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = al(28, (size_t)nq * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = al(29, (size_t)nq * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = al(30, ((size_t)kRayBins + 1024) * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = al(31, 16)) != cudaSuccess) return e;
  }
  const bool full_mis = (opt.flags & RX_VCM_FULL_PATH_MIS) != 0;
  constexpr uint32_t kMergeCap = 1u << 30;  // merge pairs per evaluation (8 GB of pair list)
  uint32_t q_chunk = nq;                     // sorted queries per merge walk
  const uint32_t pair_cap = 1u << 27;  // pairs per evaluation window
  uint32_t pair_alloc = 1u << 20;      // grows with demand up to pair_cap
  if ((e = al(17, (size_t)pair_alloc * sizeof(uint32_t))) != cudaSuccess) return e;
  if ((e = al(18, (size_t)pair_alloc * sizeof(int))) != cudaSuccess) return e;
  unsigned long long* ctr = bufs[11].as<unsigned long long>();
  unsigned* nph = reinterpret_cast<unsigned*>(ctr + 8);
  cudaMemsetAsync(ctr, 0, 64 * sizeof(unsigned long long), s);
  int grid = c->trace_cfg.sms * 4;
  // shadow rays on the persistent 4-wide walk when the tree fits its stack
  const bool wide_shadow = c->d_bvh4.p && 3 * c->bvh4.max_depth + 1 <= 64;
  int sub_grid[2] = {0, 0};  // resident blocks of k_sub_run<false>, <true>
  {
    int per = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sub_run<false>, 128, 0)) != cudaSuccess) return e;
    sub_grid[0] = c->trace_cfg.sms * std::max(per, 1);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sub_run<true>, 128, 0)) != cudaSuccess) return e;
    sub_grid[1] = c->trace_cfg.sms * std::max(per, 1);
  }
  Event e0, e1, m0, m1;  // render; merge gather of an iteration (with stats)
  if ((e = e0.create()) != cudaSuccess || (e = e1.create()) != cudaSuccess) return e;
  if (stats && ((e = m0.create()) != cudaSuccess || (e = m1.create()) != cudaSuccess)) return e;
  cudaEventRecord(e0, s);
  float radius = opt.radius;
  unsigned long long merges = 0, queries = 0;
  float merge_ms = 0;
  unsigned nscan = buckets + 1;
  unsigned nblk = (nscan + 1023) / 1024;
  const auto t_start = std::chrono::steady_clock::now();
  uint32_t done = 0;
  Snapshots snaps(c);
  for (uint32_t it = 0; it < opt.iterations; it++) {
    radius *= powf(((float)it + opt.alpha) / ((float)it + 1.0f), 1.0f / 3.0f);  // VCMTracer.cpp:29-30
    P.radius = radius;
    P.iter = it;
    cudaMemsetAsync(nph, 0, sizeof(unsigned), s);
    cudaMemsetAsync(bufs[26].p, 0, bufs[26].bytes, s);  // subpath cursors
    // the subpaths on persistent warps (the whole-path check mode keeps one thread per
    // subpath): one launch per side, as many blocks as stay resident
    auto subpaths = [&](bool light_side) {
      const SubSink out = light_side ? SubSink{bufs[0].as<float4>(), bufs[1].as<int>(), !P.bpt, bufs[2].as<float4>(),
                                               bufs[3].as<int>(), nph, cap}
                                     : SubSink{bufs[12].as<float4>(), bufs[13].as<int>(), false, nullptr, nullptr,
                                               nullptr, 0u};
      unsigned* cursor = bufs[26].as<unsigned>() + (light_side ? 0 : 1);
      unsigned long long* rc = ctr + (light_side ? 0 : 1);
      const bool light_scatter = light_side || !P.bpt;  // VCM samples eye paths with light-path scattering
      if (light_side) k_sub_run<true><<<sub_grid[1], 128, 0, s>>>(S, P, out, light_scatter, cursor, rc);
      else k_sub_run<false><<<sub_grid[0], 128, 0, s>>>(S, P, out, light_scatter, cursor, rc);
    };
    if (full_mis)
      k_vcm_light<<<grid * 4, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[1].as<int>(), bufs[2].as<float4>(),
                                       bufs[3].as<int>(), nph, cap, ctr);
    else
      subpaths(true);
    k_light_mis<<<grid, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[1].as<int>(), bufs[19].as<MisL>());
    const float cell = 2.0f * radius;
    Grid G{cell, buckets - 1, bufs[7].as<unsigned>(), bufs[22].as<float4>(), bufs[5].as<int>(), bufs[23].as<float4>()};
    if (!P.bpt) {  // the photon grid
      cudaMemsetAsync(bufs[6].p, 0, bufs[6].bytes, s);
      k_grid_count<<<grid, 256, 0, s>>>(bufs[2].as<float4>(), nph, cap, cell, buckets - 1, bufs[6].as<unsigned>(),
                                        bufs[4].as<unsigned>());
      k_scan_blocks<unsigned><<<nblk, 1024, 0, s>>>(bufs[6].as<unsigned>(), bufs[7].as<unsigned>(),
                                                      bufs[9].as<unsigned>(), nscan);
      k_scan_sums<unsigned><<<1, 1024, 0, s>>>(bufs[9].as<unsigned>(), nblk);
      k_scan_add<unsigned><<<nblk, 1024, 0, s>>>(bufs[7].as<unsigned>(), bufs[9].as<unsigned>(), nscan,
                                                  bufs[8].as<unsigned>());
      k_grid_scatter<<<grid, 256, 0, s>>>(bufs[4].as<unsigned>(), bufs[2].as<float4>(), bufs[3].as<int>(), nph, cap,
                                          bufs[8].as<unsigned>(), bufs[22].as<float4>(), bufs[5].as<int>(),
                                          bufs[0].as<float4>(), bufs[19].as<MisL>(), P.maxv, bufs[23].as<float4>());
      k_count_photons<<<1, 1, 0, s>>>(nph, cap, ctr + 6);
    }
    cudaMemsetAsync(bufs[10].p, 0, bufs[10].bytes, s);
    unsigned long long* qc = bufs[14].as<unsigned long long>();
    unsigned long long* qo = bufs[15].as<unsigned long long>();
    // exclusive scan of n 64-bit counts into qo; returns the total (synchronises)
    auto scan_total = [&](uint32_t n, unsigned long long& total) -> cudaError_t {
      const unsigned nb = (n + 1023) / 1024;
      k_scan_blocks<unsigned long long><<<nb, 1024, 0, s>>>(qc, qo, bufs[16].as<unsigned long long>(), n);
      k_scan_sums<unsigned long long><<<1, 1024, 0, s>>>(bufs[16].as<unsigned long long>(), nb);
      k_scan_add<unsigned long long><<<nb, 1024, 0, s>>>(qo, bufs[16].as<unsigned long long>(), n, nullptr);
      unsigned long long tail[2] = {0, 0};
      cudaMemcpyAsync(&tail[0], qo + (n - 1), sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(&tail[1], qc + (n - 1), sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
      cudaError_t err = cudaStreamSynchronize(s);
      total = tail[0] + tail[1];
      if (err == cudaSuccess && total > pair_alloc && pair_alloc < pair_cap) {
        pair_alloc = (uint32_t)std::min<unsigned long long>(pair_cap, std::max<unsigned long long>(total, 2ull * pair_alloc));
        if ((err = bufs[17].alloc((size_t)pair_alloc * sizeof(uint32_t))) != cudaSuccess) return err;
        err = bufs[18].alloc((size_t)pair_alloc * sizeof(int));
      }
      return err;
    };
    unsigned long long total = 0;
    if (full_mis) {
      k_vcm_eye_full<<<grid, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[1].as<int>(), bufs[12].as<float4>(),
                                          bufs[13].as<int>(), bufs[20].as<MisE>(), bufs[10].as<float>(), ctr + 1);
    } else {
      subpaths(false);
      k_eye_post<<<grid * 2, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[1].as<int>(), bufs[12].as<float4>(),
                                          bufs[13].as<int>(), bufs[20].as<MisE>(), bufs[21].as<uint2>(), qc,
                                          bufs[10].as<float>());
      if ((e = scan_total(P.n_pixels, total)) != cudaSuccess) return e;
      // the shadow-ray queue: at most one ray per connection of a window
      const size_t sq_bytes = (size_t)std::min<unsigned long long>(pair_alloc, std::max(total, 1ull)) * sizeof(ShadowQ);
      if (bufs[32].bytes < sq_bytes && (e = bufs[32].alloc(sq_bytes)) != cudaSuccess) return e;
      unsigned* sq_n = reinterpret_cast<unsigned*>(ctr + 13);
      unsigned long long* sq_cursor = ctr + 12;
      for (unsigned long long w0 = 0; w0 < total; w0 += pair_alloc) {
        uint32_t np = (uint32_t)std::min<unsigned long long>(pair_alloc, total - w0);
        k_conn_fill<<<grid * 4, 128, 0, s>>>(P, bufs[21].as<uint2>(), qo, w0, pair_alloc, bufs[17].as<uint32_t>(),
                                             bufs[18].as<int>());
        cudaMemsetAsync(sq_n, 0, sizeof(unsigned), s);
        k_conn_eval<<<grid * 2, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[12].as<float4>(), bufs[19].as<MisL>(),
                                             bufs[20].as<MisE>(), bufs[17].as<uint32_t>(), bufs[18].as<int>(), np,
                                             bufs[10].as<float>(), ctr + 2, bufs[32].as<ShadowQ>(), sq_n);
        if (wide_shadow) {  // persistent: the blocks that stay resident (8 per SM)
          cudaMemsetAsync(sq_cursor, 0, sizeof(unsigned long long), s);
          k_shadow_wide<<<c->trace_cfg.sms * 8, 128, 0, s>>>(S, bufs[32].as<ShadowQ>(), sq_n, bufs[10].as<float>(),
                                                            sq_cursor);
        } else {
          k_shadow_thread<<<grid * 2, 128, 0, s>>>(S, bufs[32].as<ShadowQ>(), sq_n, bufs[10].as<float>());
        }
      }
    }
    if (P.bpt) {
      // BidirectionalPathTracer: connections only
    } else if (full_mis) {  // merging as (query, photon) pair lists: count per query, scan, windows
      k_merge_count<<<grid * 4, 128, 0, s>>>(S, P, bufs[12].as<float4>(), bufs[13].as<int>(), G, qc, nq);
      if ((e = scan_total(nq, total)) != cudaSuccess) return e;
      merges += total;
      for (unsigned long long w0 = 0; w0 < total; w0 += pair_alloc) {
        uint32_t np = (uint32_t)std::min<unsigned long long>(pair_alloc, total - w0);
        k_merge_fill<<<grid * 4, 128, 0, s>>>(S, P, bufs[12].as<float4>(), bufs[13].as<int>(), G, qo, nq, w0, pair_alloc,
                                              bufs[17].as<uint32_t>(), bufs[18].as<int>());
        k_merge_eval_full<<<grid * 2, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[12].as<float4>(),
                                                   bufs[17].as<uint32_t>(), bufs[18].as<int>(), np,
                                                   bufs[10].as<float>());
      }
    } else {  // the queries in spatial order, one walk appending pairs, then one pair per lane
      if (m0) cudaEventRecord(m0, s);
      uint32_t* qlist = bufs[27].as<uint32_t>();
      uint32_t* qkey = bufs[28].as<uint32_t>();
      uint32_t* qorder = bufs[29].as<uint32_t>();
      uint32_t* qhist = bufs[30].as<uint32_t>();
      unsigned* qcount = bufs[31].as<unsigned>();
      cudaMemsetAsync(qcount, 0, sizeof(unsigned), s);
      cudaMemsetAsync(qhist, 0, (size_t)kRayBins * sizeof(uint32_t), s);
      k_merge_queries<<<grid, 128, 0, s>>>(S, P, bufs[12].as<float4>(), bufs[13].as<int>(), qlist, qkey, qhist, qcount);
      scan_bins(qhist, qhist + kRayBins, s);
      k_ray_scatter<<<grid * 2, 256, 0, s>>>(qkey, 0, qcount, qhist, qorder);
      unsigned nqv = 0;
      cudaMemcpyAsync(&nqv, qcount, sizeof nqv, cudaMemcpyDeviceToHost, s);
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
      queries += nqv;
      for (uint32_t j0 = 0; j0 < nqv;) {
        const uint32_t j1 = (uint32_t)std::min<uint64_t>(nqv, (uint64_t)j0 + q_chunk);
        unsigned long long* np_dev = ctr + 4;  // [4] pairs of this query range
        cudaMemsetAsync(np_dev, 0, sizeof(unsigned long long), s);
        k_merge_walk<<<grid * 2, 256, 0, s>>>(P, bufs[12].as<float4>(), G, qlist, qorder, j0, j1, pair_alloc,
                                              bufs[17].as<uint32_t>(), bufs[18].as<int>(), np_dev);
        unsigned long long np = 0;
        cudaMemcpyAsync(&np, np_dev, sizeof np, cudaMemcpyDeviceToHost, s);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (np > pair_alloc) {  // grow the pair list, or split the query range once it is at its cap
          if (pair_alloc < kMergeCap) {
            pair_alloc = (uint32_t)std::min<unsigned long long>(kMergeCap, np + np / 4);
            if ((e = bufs[17].alloc((size_t)pair_alloc * sizeof(uint32_t))) != cudaSuccess) return e;
            if ((e = bufs[18].alloc((size_t)pair_alloc * sizeof(int))) != cudaSuccess) return e;
            continue;
          }
          if (j1 - j0 > 1) {
            q_chunk = (j1 - j0) / 2;
            continue;
          }
          np = pair_alloc;  // one query beyond the cap: its first kMergeCap pairs
        }
        merges += np;
        if (np)
          k_merge_eval<<<grid * 2, 128, 0, s>>>(S, P, bufs[12].as<float4>(), bufs[20].as<MisE>(), bufs[23].as<float4>(),
                                                bufs[17].as<uint32_t>(), bufs[18].as<int>(), (uint32_t)np,
                                                bufs[10].as<float>());
        j0 = j1;
      }
      if (m1) {  // device time of this iteration's merge gather (walk + pair evaluation)
        cudaEventRecord(m1, s);
        if ((e = cudaEventSynchronize(m1)) != cudaSuccess) return e;
        float mms = 0;
        cudaEventElapsedTime(&mms, m0, m1);
        merge_ms += mms;
      }
    }
    k_vcm_accumulate<<<grid, 256, 0, s>>>(P, bufs[10].as<float>(), film);
    done = it + 1;
    if (snaps.due()) {
      const double n = done;
      if ((e = snaps.take(film, cam.width, cam.height, n, [&](size_t) { return n; }, s)) != cudaSuccess) return e;
    }
    if (opt.time_budget_s > 0) {  // the reference's runtime check after each iteration
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
      if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() >= opt.time_budget_s)
        break;
    }
  }
  cudaEventRecord(e1, s);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (stats) {
    unsigned long long h[8];
    cudaMemcpy(h, ctr, sizeof h, cudaMemcpyDeviceToHost);
    stats->extension_rays = h[0] + h[1];
    stats->shadow_rays = h[2];
    stats->merges = merges;
    stats->paths = (uint64_t)P.n_pixels * done;
    stats->ms = ms;
    stats->merge_ms = merge_ms;
    stats->merge_queries = queries;
    stats->photons = h[6];
  }
  return cudaSuccess;
}

// PhotonMap::renderPixels (src/Photonmap.cpp:12-138): per iteration s the radius
// max(r0 ((s+1)^(alpha-1))^(1/3), EPSILON), light paths and photons, the hash grid over
// all photons with a box per photon type, the eye pass, and the running mean of the
// vignetting-corrected images.
cudaError_t render_pm(rx_context* c, const rx_camera& cam, const rx_pm_options& opt, double* film,
                      rx_render_stats* stats, cudaStream_t s) {
  const DevScene& S = c->scene;
  VcmParams P = camera_params(cam);
  P.seed = opt.seed;
  P.max_depth = opt.max_depth;
  P.maxv = opt.max_depth + 3;
  P.n_light = opt.light_paths ? opt.light_paths : P.n_pixels;  // mPhotonsNum = W * H
  P.norm = (float)P.n_light;
  const float alpha = opt.alpha > 0.0f ? opt.alpha : 2.0f / 3.0f;  // mAlpha
  const unsigned cap = P.n_light * P.maxv;
  unsigned buckets = 1u << 16;
  while (buckets < cap && buckets < (1u << 26)) buckets <<= 1;
  const unsigned nscan = buckets + 1, nblk = (nscan + 1023) / 1024;
  std::vector<DevBuf> bufs(12);
  cudaError_t e;
  auto al = [&](int k, size_t bytes) { return bufs[k].alloc(bytes); };
  if ((e = al(0, (size_t)cap * sizeof(float4))) != cudaSuccess) return e;            // photon positions (+ type)
  if ((e = al(1, (size_t)cap * kPmData * sizeof(float4))) != cudaSuccess) return e;  // photon rays, powers
  if ((e = al(2, (size_t)cap * sizeof(unsigned))) != cudaSuccess) return e;          // bucket keys
  if ((e = al(3, (size_t)cap * sizeof(float4))) != cudaSuccess) return e;            // positions, bucket order
  if ((e = al(4, (size_t)cap * kPmData * sizeof(float4))) != cudaSuccess) return e;  // data, bucket order
  if ((e = al(5, (size_t)nscan * sizeof(unsigned))) != cudaSuccess) return e;        // counts
  if ((e = al(6, (size_t)nscan * sizeof(unsigned))) != cudaSuccess) return e;        // start
  if ((e = al(7, (size_t)nscan * sizeof(unsigned))) != cudaSuccess) return e;        // cursor
  if ((e = al(8, ((size_t)nblk + 2) * sizeof(unsigned))) != cudaSuccess) return e;   // block sums
  if ((e = al(9, (size_t)P.n_pixels * 3 * sizeof(float))) != cudaSuccess) return e;  // iteration image
  if ((e = al(10, 16 * sizeof(unsigned long long))) != cudaSuccess) return e;        // counters
  if ((e = al(11, 12 * sizeof(int))) != cudaSuccess) return e;                       // photon boxes
  unsigned long long* ctr = bufs[10].as<unsigned long long>();
  unsigned* nph = reinterpret_cast<unsigned*>(ctr + 8);
  cudaMemsetAsync(ctr, 0, 16 * sizeof(unsigned long long), s);
  const int grid = c->trace_cfg.sms * 4;
  Event e0, e1;
  if ((e = e0.create()) != cudaSuccess || (e = e1.create()) != cudaSuccess) return e;
  cudaEventRecord(e0, s);
  unsigned long long photons = 0;
  const auto t_start = std::chrono::steady_clock::now();
  uint32_t done = 0;
  Snapshots snaps(c);
  for (uint32_t it = 0; it < opt.iterations; it++) {
    P.iter = it;
    P.radius = fmaxf(opt.radius * powf(powf((float)(it + 1), alpha - 1.0f), 1.0f / 3.0f), 1e-5f);
    cudaMemsetAsync(nph, 0, sizeof(unsigned), s);
    k_pm_light<<<grid * 4, 128, 0, s>>>(S, P, bufs[0].as<float4>(), bufs[1].as<float4>(), nph, cap, ctr);
    const float cell = 2.0f * P.radius;
    cudaMemsetAsync(bufs[5].p, 0, bufs[5].bytes, s);
    k_grid_count<<<grid, 256, 0, s>>>(bufs[0].as<float4>(), nph, cap, cell, buckets - 1, bufs[5].as<unsigned>(),
                                      bufs[2].as<unsigned>());
    k_scan_blocks<unsigned><<<nblk, 1024, 0, s>>>(bufs[5].as<unsigned>(), bufs[6].as<unsigned>(),
                                                    bufs[8].as<unsigned>(), nscan);
    k_scan_sums<unsigned><<<1, 1024, 0, s>>>(bufs[8].as<unsigned>(), nblk);
    k_scan_add<unsigned><<<nblk, 1024, 0, s>>>(bufs[6].as<unsigned>(), bufs[8].as<unsigned>(), nscan,
                                                bufs[7].as<unsigned>());
    k_pm_scatter<<<grid, 256, 0, s>>>(bufs[2].as<unsigned>(), bufs[0].as<float4>(), bufs[1].as<float4>(), nph, cap,
                                      bufs[7].as<unsigned>(), bufs[3].as<float4>(), bufs[4].as<float4>());
    k_pm_box_init<<<1, 32, 0, s>>>(bufs[11].as<int>());
    k_pm_box<<<grid, 256, 0, s>>>(bufs[0].as<float4>(), nph, cap, bufs[11].as<int>());
    Grid G{cell, buckets - 1, bufs[6].as<unsigned>(), bufs[3].as<float4>(), nullptr, nullptr};
    cudaMemsetAsync(bufs[9].p, 0, bufs[9].bytes, s);
    k_pm_eye<<<grid * 2, 128, 0, s>>>(S, P, G, bufs[4].as<float4>(), bufs[11].as<int>(), bufs[9].as<float>(), ctr + 1);
    k_vcm_accumulate<<<grid, 256, 0, s>>>(P, bufs[9].as<float>(), film);
    unsigned np = 0;
    cudaMemcpyAsync(&np, nph, sizeof np, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    photons += std::min(np, cap);
    done = it + 1;
    if (snaps.due()) {
      const double n = done;
      if ((e = snaps.take(film, cam.width, cam.height, n, [&](size_t) { return n; }, s)) != cudaSuccess) return e;
    }
    if (opt.time_budget_s > 0 &&
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() >= opt.time_budget_s)
      break;
  }
  cudaEventRecord(e1, s);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (stats) {
    unsigned long long h[2];
    cudaMemcpy(h, ctr, sizeof h, cudaMemcpyDeviceToHost);
    stats->extension_rays = h[0] + h[1];
    stats->shadow_rays = 0;
    stats->merges = photons;
    stats->photons = photons;
    stats->paths = (uint64_t)P.n_pixels * done;
    stats->ms = ms;
  }
  return cudaSuccess;
}

}  // namespace rx
