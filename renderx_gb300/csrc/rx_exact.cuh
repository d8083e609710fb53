// Device restatement of the reference's parity-critical float arithmetic, one IEEE
// single-precision operation per reference operation, round-to-nearest, never fused:
//  * vector ops of nvVector.h:491-527 (cross; dot accumulated from 0; normalize by
//    the correctly rounded sqrt of the accumulated square norm),
//  * the ray/triangle test of KDTree.cpp:267-293,
//  * the node box test of KDTree.cpp:34-52.
// __f*_rn intrinsics are never contracted into FMAs, so the results match the
// reference built with -ffp-contract=off on the host bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rx {

struct F3 {
  float x, y, z;
};

__device__ __forceinline__ F3 f3(float4 v) { return {v.x, v.y, v.z}; }

// Not parity arithmetic: the BVH walks' slab tests (their boxes only pick candidates).
// Three-input float minimum and maximum (one instruction each on sm_100 and later; the
// same values as two fminf / fmaxf, NaN operands aside, which the walk never forms).
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
// The slab tests' inverse direction: finite and never zero (+-1e30 for components
// within 1e-30 of zero).
__device__ __forceinline__ F3 safe_inv(F3 d) {
  auto iv = [](float x) { return fabsf(x) > 1e-30f ? 1.0f / x : copysignf(1e30f, x); };
  return {iv(d.x), iv(d.y), iv(d.z)};
}
__device__ __forceinline__ float comp(F3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

__device__ __forceinline__ F3 xsub(F3 a, F3 b) {
  return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
// vec3::cross, nvVector.h:491-499
__device__ __forceinline__ F3 xcross(F3 l, F3 r) {
  return {__fsub_rn(__fmul_rn(l.y, r.z), __fmul_rn(l.z, r.y)), __fsub_rn(__fmul_rn(l.z, r.x), __fmul_rn(l.x, r.z)),
          __fsub_rn(__fmul_rn(l.x, r.y), __fmul_rn(l.y, r.x))};
}
// vec3::dot, nvVector.h:502-508: r = 0; r += l[i]*r[i]
__device__ __forceinline__ float xdot(F3 a, F3 b) {
  float r = __fadd_rn(0.0f, __fmul_rn(a.x, b.x));
  r = __fadd_rn(r, __fmul_rn(a.y, b.y));
  return __fadd_rn(r, __fmul_rn(a.z, b.z));
}
// vec3::normalize, nvVector.h:511-527
__device__ __forceinline__ F3 xnormalize(F3 v) {
  float r = __fsqrt_rn(xdot(v, v));
  if (r > 0.0f) v = {__fdiv_rn(v.x, r), __fdiv_rn(v.y, r), __fdiv_rn(v.z, r)};
  return v;
}

// KDTree::intersect(ray, triangle) without a condition (KDTree.cpp:267-293). Returns
// true when the reference accepts the triangle (distance >= 0; NaN never passes the
// caller's `dist >= 0`), and the distance.
// `normal(l0, l1)` gives the triangle's unit normal, xnormalize(xcross(l0, l1)): formed
// here, or read from the triangle's slot, where the same functions formed it once
// (k_slot_normals) with the same bits.
template <class Normal>
__device__ __forceinline__ bool tri_exact_with(F3 v0, F3 v1, F3 v2, F3 o, F3 d, float& t, Normal normal) {
  F3 l0 = xsub(v1, v0), l1 = xsub(v2, v1), l2 = xsub(v0, v2);
  F3 r0 = xsub(v0, o), r1 = xsub(v1, o), r2 = xsub(v2, o);
  float s0 = xdot(d, xcross(l0, r0));
  float s1 = xdot(d, xcross(l1, r1));
  float s2 = xdot(d, xcross(l2, r2));
  bool pos = (s0 >= 0.0f) & (s1 >= 0.0f) & (s2 >= 0.0f);
  bool neg = (s0 <= 0.0f) & (s1 <= 0.0f) & (s2 <= 0.0f);
  if (!(pos | neg)) return false;
  F3 n = normal(l0, l1);
  float od = xdot(n, r2);
  float dd = xdot(n, d);
  if (dd == 0.0f) return false;
  float q = __fdiv_rn(od, dd);
  if (!(q >= 0.0f)) return false;
  t = q;
  return true;
}
__device__ __forceinline__ bool tri_exact(F3 v0, F3 v1, F3 v2, F3 o, F3 d, float& t) {
  return tri_exact_with(v0, v1, v2, o, d, t, [](F3 l0, F3 l1) { return xnormalize(xcross(l0, l1)); });
}
// The same test with the unit normal read from the triangle's slot (loaded only for
// rays that pass the edge tests).
__device__ __forceinline__ bool tri_exact_n(F3 v0, F3 v1, F3 v2, const float4* nrm, F3 o, F3 d, float& t) {
  return tri_exact_with(v0, v1, v2, o, d, t, [nrm](F3, F3) { return f3(__ldg(nrm)); });
}

// KDTree::Node::BoundingBox::intersect (KDTree.cpp:34-52) reduced to pass/fail:
// some face at non-negative distance whose intersection point lies within the other
// two slabs, inclusive, no epsilon. Faces are skipped when the direction component is
// exactly zero.
__device__ __forceinline__ bool box_exact(F3 mn, F3 mx, F3 o, F3 d) {
#pragma unroll
  for (int i = 0; i < 6; i++) {
    int a = i % 3;
    float da = comp(d, a);
    if (da == 0.0f) continue;
    float b = i < 3 ? comp(mn, a) : comp(mx, a);
    float dist = __fdiv_rn(__fsub_rn(b, comp(o, a)), da);
    if (!(dist >= 0.0f)) continue;
    int a1 = (i + 1) % 3, a2 = (i + 2) % 3;
    float p1 = __fadd_rn(comp(o, a1), __fmul_rn(dist, comp(d, a1)));
    float p2 = __fadd_rn(comp(o, a2), __fmul_rn(dist, comp(d, a2)));
    if (comp(mn, a1) <= p1 && comp(mx, a1) >= p1 && comp(mn, a2) <= p2 && comp(mx, a2) >= p2) return true;
  }
  return false;
}

// The margins of box_clear_pass for one ray: per axis 4e-6 (1 + |o|) and 4e-6 |d|, so
// that the margin at distance t, 4e-6 (1 + |o| + t |d|), is one fused multiply-add (its
// rounding moves it by about 1e-7 of itself; the margin is four times the bound it must
// exceed).
struct ClearMargins {
  F3 mo, md;
};
__device__ __forceinline__ ClearMargins clear_margins(F3 o, F3 d) {
  return {{4e-6f * (1.0f + fabsf(o.x)), 4e-6f * (1.0f + fabsf(o.y)), 4e-6f * (1.0f + fabsf(o.z))},
          {4e-6f * fabsf(d.x), 4e-6f * fabsf(d.y), 4e-6f * fabsf(d.z)}};
}

// Decides the reference box test cheaply when the answer is clear: the ray's entry
// (or exit) face point lies inside that face with a margin that exceeds the
// reference's rounding error (< 8 ulp of |o|+|t d| per coordinate); the sign of the
// face distance is exact because both sides form fl(b - o) and divide by d's sign.
// Returns 1 = passes, 0 = undecided (caller runs box_exact).
__device__ __forceinline__ int box_clear_pass(F3 mn, F3 mx, F3 o, F3 d, F3 inv, const ClearMargins& m) {
  float t0x = __fmul_rn(__fsub_rn(mn.x, o.x), inv.x), t1x = __fmul_rn(__fsub_rn(mx.x, o.x), inv.x);
  float t0y = __fmul_rn(__fsub_rn(mn.y, o.y), inv.y), t1y = __fmul_rn(__fsub_rn(mx.y, o.y), inv.y);
  float t0z = __fmul_rn(__fsub_rn(mn.z, o.z), inv.z), t1z = __fmul_rn(__fsub_rn(mx.z, o.z), inv.z);
  const float nx = fminf(t0x, t1x), ny = fminf(t0y, t1y), nz = fminf(t0z, t1z);
  const float fx = fmaxf(t0x, t1x), fy = fmaxf(t0y, t1y), fz = fmaxf(t0z, t1z);
  const float te = max3f(nx, ny, nz), tx = min3f(fx, fy, fz);  // entry and exit faces
#pragma unroll
  for (int f = 0; f < 2; f++) {
    const float t = f == 0 ? te : tx;
    if (!(t >= 0.0f)) continue;
    // the face's axis (any axis that attains t: each is a face the ray meets at t), then
    // the point on it inside the other two slabs with the margin, all three axes at once
    const int a = f == 0 ? (nx == t ? 0 : (ny == t ? 1 : 2)) : (fx == t ? 0 : (fy == t ? 1 : 2));
    const float px = o.x + t * d.x, py = o.y + t * d.y, pz = o.z + t * d.z;
    const float dx = fmaf(t, m.md.x, m.mo.x), dy = fmaf(t, m.md.y, m.mo.y), dz = fmaf(t, m.md.z, m.mo.z);
    const bool inx = (px >= mn.x + dx) && (px <= mx.x - dx), iny = (py >= mn.y + dy) && (py <= mx.y - dy);
    const bool inz = (pz >= mn.z + dz) && (pz <= mx.z - dz);
    if ((inx || a == 0) && (iny || a == 1) && (inz || a == 2)) return 1;
  }
  return 0;
}

}  // namespace rx
