// Device building blocks of the light-transport kernels: vector math, the counter-based
// random numbers, shading normals, the reference's materials and the condition-aware
// closest-hit / occlusion queries.
//
// Sampling semantics follow the reference (cited per function); arithmetic here is
// ordinary fast FP32 with FMA (statistical parity, not bit parity).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rx_accel.h"
#include "rx_exact.cuh"
#include "rx_scene.h"

namespace rx {

#define RX_PI 3.14159265358979323846f

__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator-(F3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 operator*(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 l, F3 r) {
  return {l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x};
}
__device__ __forceinline__ float length(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ F3 normalize(F3 a) {
  float l = length(a);
  return l > 0.0f ? a * (1.0f / l) : a;
}
__device__ __forceinline__ float maxc(F3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
// luminance weights of smallFuncs.h y()/intensity()
__device__ __forceinline__ float lum(F3 a) { return 0.212671f * a.x + 0.715160f * a.y + 0.072169f * a.z; }
__device__ __forceinline__ F3 f3v(const float* p) { return {p[0], p[1], p[2]}; }

// ---- random numbers ------------------------------------------------------------------
// Counter-based: value k of path `path` under `seed` is a 64-bit mix (splitmix64
// finaliser) of (seed, path, k), 24-bit floats in [0,1) like RNG::randFloat
// (reference src/RandGenerator.cpp:21-25). Paths are independent and reproducible,
// with no shared state (the reference's single global MT19937 is raced by all its
// OpenMP threads, RandGenerator.cpp:9).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t key;
  uint32_t k;
  __device__ __forceinline__ Rng(uint64_t seed, uint64_t path, uint32_t start)
      : key(mix64(seed ^ mix64(path + 0x9e3779b97f4a7c15ull))), k(start) {}
  __device__ __forceinline__ float next() {
    uint64_t h = mix64(key + 0x9e3779b97f4a7c15ull * (uint64_t)(++k));
    return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
  }
};

// ---- local frames and samplers ---------------------------------------------------------
// LocalFrame::buildFromNormal / toWorld, reference include/LocalFrame.h:13-33.
struct Frame {
  F3 s, t, n;
};
__device__ __forceinline__ Frame frame_from(F3 n) {
  F3 tmp = fabsf(n.z) > 0.99f ? F3{1, 0, 0} : F3{0, 0, 1};
  Frame f;
  f.n = n;
  f.s = normalize(cross(n, tmp));
  f.t = normalize(cross(f.s, f.n));
  return f;
}
__device__ __forceinline__ F3 to_world(const Frame& f, F3 a) { return f.s * a.x + f.n * a.y + f.t * a.z; }
// RandGenerator::genHemiCosDirection, src/RandGenerator.cpp:152-167 (cos^exp lobe
// around the frame's n; exp = 1 is cosine sampling).
__device__ __forceinline__ F3 hemi_cos(float e, float r1, float r2) {
  float u1 = 2.0f * RX_PI * r1;
  float u2 = e == 1.0f ? sqrtf(r2) : powf(r2, 1.0f / (e + 1.0f));
  float u3 = sqrtf(fmaxf(0.0f, 1.0f - u2 * u2));
  float s, c;
  sincosf(u1, &s, &c);
  return normalize(F3{c * u3, u2, s * u3});
}
// CosineSphericalSampler::getProbDensity, include/CosineSphericalSampler.h:292-303
__device__ __forceinline__ float cos_lobe_pdf(F3 n, F3 dir, float e) {
  float ct = fmaxf(dot(n, dir), 0.0f);
  float p = e == 1.0f ? ct : powf(ct, e);
  return p * (e + 1.0f) / (2.0f * RX_PI);
}

// ---- normals -------------------------------------------------------------------------
struct TriGeom {
  F3 v0, v1, v2, n0, n1, n2;
  int obj;
};
__device__ __forceinline__ TriGeom tri_geom(const DevScene& S, int tid) {
  TriGeom g;
  const float4* v = S.tri_v + 3 * (size_t)tid;
  const float4* n = S.tri_n + 3 * (size_t)tid;
  g.v0 = f3(__ldg(v));
  g.v1 = f3(__ldg(v + 1));
  g.v2 = f3(__ldg(v + 2));
  g.n0 = f3(__ldg(n));
  g.n1 = f3(__ldg(n + 1));
  g.n2 = f3(__ldg(n + 2));
  g.obj = (int)__ldg(&S.tri_obj[tid]);
  return g;
}
// SimpleShape::getWorldNormal (src/SimpleShape.cpp:393-441): face normal without vertex
// normals, else the vertex normals interpolated with the barycentric coordinates of
// `p` (same u1, u2 formula); flat = face normal turned toward the interpolated one.
__device__ __forceinline__ F3 world_normal(const TriGeom& g, bool has_normals, F3 p, bool flat = false) {
  F3 b1 = g.v1 - g.v0, b2 = g.v2 - g.v0;
  F3 fn = normalize(cross(b1, b2));
  if (!has_normals) return fn;
  F3 v = p - g.v0;
  float d12 = dot(b1, b2), l1s = dot(b1, b1), l2s = dot(b2, b2);
  float u2 = (dot(v, b1) * d12 - dot(v, b2) * l1s) / (d12 * d12 - l1s * l2s);
  float u1 = (dot(v, b1) - u2 * d12) / l1s;
  F3 n = normalize(g.n0 * (1.0f - u1 - u2) + g.n1 * u1 + g.n2 * u2);
  if (flat) return dot(n, fn) < 0.0f ? -fn : fn;
  return n;
}

// ---- self-intersection condition + closest hit ---------------------------------------
// NoSelfIntersectionCondition::legal (src/NoSelfIntersectionCondition.cpp:12-27),
// evaluated on every candidate before the closest one is chosen (KDTree.cpp:290):
// the sign of the direction against the candidate's shading normal decides.
__device__ __forceinline__ bool legal_hit(int contact, int inside, int obj, float dn) {
  bool in = dn <= 0.0f, out = dn >= 0.0f;
  if (inside == contact) return !(in && contact == obj);
  return !(out && inside != obj);
}

struct PHit {
  int tid;
  float t;
};

// Closest legal hit with t < tmax (ANY: stop at the first legal one). contact, inside:
// object ids, -1 for none (-1/-1: no condition, as the camera ray's first query),
// -2 for the camera as contact object. only_obj >= 0: closest hit among that object's
// triangles only, no condition (the per-object trees of Scene::findInsideObject).
template <bool ANY, int STACK = kStackDepth>
__device__ __forceinline__ PHit trace_cond(const DevScene& S, F3 o, F3 d, float tmax, int contact, int inside,
                                           int only_obj = -1) {
  const DevAccel& A = S.accel;
  F3 inv = {fabsf(d.x) > 1e-30f ? 1.0f / d.x : copysignf(1e30f, d.x),
            fabsf(d.y) > 1e-30f ? 1.0f / d.y : copysignf(1e30f, d.y),
            fabsf(d.z) > 1e-30f ? 1.0f / d.z : copysignf(1e30f, d.z)};
  F3 ood = {o.x * inv.x, o.y * inv.y, o.z * inv.z};
  PHit best{-1, tmax};
  int stack[STACK];
  int sp = 0, cur = 0, cnt = 0;
  const bool cond = only_obj < 0 && !(contact == -1 && inside == -1);
  while (true) {
    if (cur >= 0) {
      const float4* np = A.bvh + 4 * (size_t)cur;
      float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
      int4 n3 = __ldg(reinterpret_cast<const int4*>(np + 3));
      float a0 = fmaf(n0.x, inv.x, -ood.x), b0 = fmaf(n0.y, inv.x, -ood.x);
      float a1 = fmaf(n0.z, inv.y, -ood.y), b1 = fmaf(n0.w, inv.y, -ood.y);
      float a2 = fmaf(n2.x, inv.z, -ood.z), b2 = fmaf(n2.y, inv.z, -ood.z);
      float tn0 = fmaxf(max3f(fminf(a0, b0), fminf(a1, b1), fminf(a2, b2)), 0.0f);
      float tf0 = fminf(min3f(fmaxf(a0, b0), fmaxf(a1, b1), fmaxf(a2, b2)), best.t);
      float c0 = fmaf(n1.x, inv.x, -ood.x), d0 = fmaf(n1.y, inv.x, -ood.x);
      float c1 = fmaf(n1.z, inv.y, -ood.y), d1 = fmaf(n1.w, inv.y, -ood.y);
      float c2 = fmaf(n2.z, inv.z, -ood.z), d2 = fmaf(n2.w, inv.z, -ood.z);
      float tn1 = fmaxf(max3f(fminf(c0, d0), fminf(c1, d1), fminf(c2, d2)), 0.0f);
      float tf1 = fminf(min3f(fmaxf(c0, d0), fmaxf(c1, d1), fmaxf(c2, d2)), best.t);
      bool h0 = tn0 <= tf0 * 1.0000005f, h1 = tn1 <= tf1 * 1.0000005f;
      if (h0 && h1) {
        bool first0 = tn0 <= tn1;
        int far_ref = first0 ? n3.y : n3.x, far_cnt = first0 ? n3.w : n3.z;
        if (sp < STACK) stack[sp++] = far_ref < 0 ? ~((~far_ref) << 3 | (far_cnt - 1)) : far_ref;
        cur = first0 ? n3.x : n3.y;
        cnt = first0 ? n3.z : n3.w;
        continue;
      } else if (h0) {
        cur = n3.x;
        cnt = n3.z;
        continue;
      } else if (h1) {
        cur = n3.y;
        cnt = n3.w;
        continue;
      }
    } else {
      int first = ~cur;
      for (int k = 0; k < cnt; k++) {
        const float4* tp = A.tris + 3 * (size_t)(first + k);
        float4 w0 = __ldg(tp), w1 = __ldg(tp + 1), w2 = __ldg(tp + 2);
        F3 v0 = f3(w0), e1 = f3(w1) - v0, e2 = f3(w2) - v0;
        F3 pv = cross(d, e2);
        float det = dot(e1, pv);
        if (fabsf(det) < 1e-30f) continue;
        float idet = 1.0f / det;
        F3 sv = o - v0;
        float u = dot(sv, pv) * idet;
        if (u < -1e-7f || u > 1.0000001f) continue;
        F3 qv = cross(sv, e1);
        float v = dot(d, qv) * idet;
        if (v < -1e-7f || u + v > 1.0000001f) continue;
        float t = dot(e2, qv) * idet;
        if (!(t >= 0.0f) || !(t < best.t)) continue;
        if (only_obj >= 0) {
          if (__float_as_int(__ldg(&S.slot_n[3 * (size_t)(first + k)]).w) != only_obj) continue;
        } else if (cond) {
          const float4* nn = S.slot_n + 3 * (size_t)(first + k);
          float4 q0 = __ldg(nn), q1 = __ldg(nn + 1), q2 = __ldg(nn + 2);
          int obj = __float_as_int(q0.w);
          F3 n = normalize(f3(q0) * (1.0f - u - v) + f3(q1) * u + f3(q2) * v);
          if (!legal_hit(contact, inside, obj, dot(d, n))) continue;
        }
        best = {__float_as_int(w0.w), t};
        if (ANY) return best;
      }
    }
    if (sp == 0) break;
    int r = stack[--sp];
    if (r < 0) {
      int packed = ~r;
      cur = ~(packed >> 3);
      cnt = (packed & 7) + 1;
    } else {
      cur = r;
    }
  }
  return best;
}

// The same query over the 4-wide BVH (rx_accel.h layout): four child boxes per
// 128-byte node, nearest hit child next, the others stacked far to near with their entry
// distance so that popped subtrees beyond the current best are skipped. The stack holds
// at most 3 entries per level: callers use it only when 3 * bvh4_depth + 1 <= 64.
constexpr int kWalk4 = 4;   // walk selector: the 4-wide BVH
constexpr int kWalk4S = 5;  // the 4-wide BVH, first kShortStack stack entries in shared memory
constexpr int kWalk4P = 6;  // kWalk4S on persistent warps that refill finished lanes (extension rays)
constexpr int kShortStack = 16;
// The cnt triangles of the 4-wide tree's leaf at slot `first` (Moller-Trumbore, the
// NoSelfIntersectionCondition when cond): lowers best to the nearest legal hit; with ANY,
// returns true at the first one.
template <bool ANY>
__device__ __forceinline__ bool leaf_test(const DevScene& S, int first, int cnt, F3 o, F3 d, bool cond, int contact,
                                          int inside, PHit& best) {
  const DevAccel& A = S.accel;
  for (int k = 0; k < cnt; k++) {
    const float4* tp = A.tris + 3 * (size_t)(first + k);
    float4 w0 = __ldg(tp), w1 = __ldg(tp + 1), w2 = __ldg(tp + 2);
    F3 v0 = f3(w0), e1 = f3(w1) - v0, e2 = f3(w2) - v0;
    F3 pv = cross(d, e2);
    float det = dot(e1, pv);
    if (fabsf(det) < 1e-30f) continue;
    float idet = 1.0f / det;
    F3 sv = o - v0;
    float u = dot(sv, pv) * idet;
    if (u < -1e-7f || u > 1.0000001f) continue;
    F3 qv = cross(sv, e1);
    float v = dot(d, qv) * idet;
    if (v < -1e-7f || u + v > 1.0000001f) continue;
    float t = dot(e2, qv) * idet;
    if (!(t >= 0.0f) || !(t < best.t)) continue;
    if (cond) {
      const float4* nn = S.slot_n + 3 * (size_t)(first + k);
      float4 q0 = __ldg(nn), q1 = __ldg(nn + 1), q2 = __ldg(nn + 2);
      int obj = __float_as_int(q0.w);
      F3 n = normalize(f3(q0) * (1.0f - u - v) + f3(q1) * u + f3(q2) * v);
      if (!legal_hit(contact, inside, obj, dot(d, n))) continue;
    }
    best = {__float_as_int(w0.w), t};
    if (ANY) return true;
  }
  return false;
}

// SH > 0: the first SH stack entries of each thread sit in shared memory, one column
// per thread (callers are kernels of at most kShortCols threads per block).
constexpr int kShortCols = 128;
template <bool ANY, int SH = 0>
__device__ __forceinline__ PHit trace_cond4(const DevScene& S, F3 o, F3 d, float tmax, int contact, int inside) {
  const DevAccel& A = S.accel;
  constexpr int kSHN = SH > 0 ? SH : 1;
  __shared__ int s_ref[kSHN][kShortCols];
  __shared__ float s_tn[kSHN][kShortCols];
  const int tx = threadIdx.x;
  F3 inv = {fabsf(d.x) > 1e-30f ? 1.0f / d.x : copysignf(1e30f, d.x),
            fabsf(d.y) > 1e-30f ? 1.0f / d.y : copysignf(1e30f, d.y),
            fabsf(d.z) > 1e-30f ? 1.0f / d.z : copysignf(1e30f, d.z)};
  F3 ood = {o.x * inv.x, o.y * inv.y, o.z * inv.z};
  // the near plane of each axis: the lower bound where the inverse direction is positive
  // (it is never zero), else the upper one; fma(x, inv, -ood) is monotonic in x, so the
  // near plane gives the smaller slab value, as ordering both with min / max would
  const int ox = inv.x < 0.0f ? 1 : 0, oy = inv.y < 0.0f ? 1 : 0, oz = inv.z < 0.0f ? 1 : 0;
  PHit best{-1, tmax};
  constexpr int kS = 64;
  int stack_ref[kS - SH];
  float stack_tn[kS - SH];
  int sp = 0, cur = 0;  // an inner node or a packed leaf (rx_accel.h)
  const bool cond = !(contact == -1 && inside == -1);
  while (true) {
    if (cur >= 0) {
      const float4* np = A.bvh4 + 8 * (size_t)cur;
      float4 lx = __ldg(np + ox), hx = __ldg(np + 1 - ox), ly = __ldg(np + 2 + oy), hy = __ldg(np + 3 - oy);
      float4 lz = __ldg(np + 4 + oz), hz = __ldg(np + 5 - oz);  // near (l) and far (h) planes
      int4 cr = __ldg(reinterpret_cast<const int4*>(np + 6));
      const float lxa[4] = {lx.x, lx.y, lx.z, lx.w}, hxa[4] = {hx.x, hx.y, hx.z, hx.w};
      const float lya[4] = {ly.x, ly.y, ly.z, ly.w}, hya[4] = {hy.x, hy.y, hy.z, hy.w};
      const float lza[4] = {lz.x, lz.y, lz.z, lz.w}, hza[4] = {hz.x, hz.y, hz.z, hz.w};
      int r[4] = {cr.x, cr.y, cr.z, cr.w};
      float tn[4];
      int nh = 0;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        float a0 = fmaf(lxa[j], inv.x, -ood.x), b0 = fmaf(hxa[j], inv.x, -ood.x);
        float a1 = fmaf(lya[j], inv.y, -ood.y), b1 = fmaf(hya[j], inv.y, -ood.y);
        float a2 = fmaf(lza[j], inv.z, -ood.z), b2 = fmaf(hza[j], inv.z, -ood.z);
        float t0 = fmaxf(max3f(a0, a1, a2), 0.0f);
        float t1 = fminf(min3f(b0, b1, b2), best.t);
        bool h = t0 <= t1 * 1.0000005f;  // an empty slot's inverted box gives t0 = +inf, t1 = -inf
        tn[j] = h ? t0 : INFINITY;
        nh += h ? 1 : 0;
      }
      auto cs = [&](int a, int b) {
        if (tn[b] < tn[a]) {
          float t = tn[a];
          tn[a] = tn[b];
          tn[b] = t;
          int q = r[a];
          r[a] = r[b];
          r[b] = q;
        }
      };
      cs(0, 1);
      cs(2, 3);
      cs(0, 2);
      cs(1, 3);
      cs(1, 2);
      if (nh > 0) {
#pragma unroll
        for (int k = 3; k >= 1; k--)
          if (k < nh && sp < kS) {
            if (SH > 0 && sp < SH) {  // packed refs go on the stack as they are
              s_ref[sp][tx] = r[k];
              s_tn[sp][tx] = tn[k];
            } else {
              stack_ref[sp - SH] = r[k];
              stack_tn[sp - SH] = tn[k];
            }
            sp++;
          }
        cur = r[0];
        continue;
      }
    } else if (leaf_test<ANY>(S, leaf_first(cur), leaf_count(cur), o, d, cond, contact, inside, best)) {
      return best;
    }
    bool found = false;
    while (sp > 0) {
      sp--;
      const bool sh = SH > 0 && sp < SH;
      if ((sh ? s_tn[sp][tx] : stack_tn[sp - SH]) <= best.t) {
        cur = sh ? s_ref[sp][tx] : stack_ref[sp - SH];
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return best;
}

// Closest / any legal hit with the walk WALK selects: kWalk4 = the 4-wide BVH, kWalk4S =
// the same with its first kShortStack stack entries in shared memory, else the binary
// BVH with a stack of WALK entries.
template <bool ANY, int WALK>
__device__ __forceinline__ PHit trace_walk(const DevScene& S, F3 o, F3 d, float tmax, int contact, int inside) {
  if constexpr (WALK == kWalk4) return trace_cond4<ANY, 0>(S, o, d, tmax, contact, inside);
  else if constexpr (WALK == kWalk4S || WALK == kWalk4P)
    return trace_cond4<ANY, kShortStack>(S, o, d, tmax, contact, inside);
  else return trace_cond<ANY, WALK>(S, o, d, tmax, contact, inside);
}

}  // namespace rx
