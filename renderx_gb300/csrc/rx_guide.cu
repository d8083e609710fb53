// Learned path guiding on the fifth-generation tensor cores: a BF16 MLP (FP32
// accumulation in tensor memory) mapping a surface point, its normal and the outgoing
// direction to a mixture of von Mises-Fisher lobes over incident directions, trained
// online by the renderer's own radiance samples. No counterpart in the reference: it is
// the learned proposal that the path tracer combines with BSDF sampling by one-sample MIS.
//
// Network: 80 inputs (12-frequency sin/cos encoding of the position normalised to the
// scene box, the shading normal, the outgoing direction, a constant 1) -> 4 hidden
// layers of 64 ReLU units -> 64 outputs of which 40 are used: 8 lobes x (weight logit,
// log-concentration, 3 mean coordinates). Weights and activations BF16, accumulation
// FP32 in tensor memory. One CTA of 128 threads owns a tile of 128 samples; thread s owns
// sample s (tensor-memory lane s of the M = 128 accumulators).
//
// Training minimises the cross entropy of the mixture against the renderer's integrand
// samples, -sum_s w_s log q(wi_s) / sum_s w_s, with w_s = (BSDF x cosine x incident
// radiance) / (sampling density) of sample s. The training kernel runs forward and
// backward per tile and accumulates every layer's weight gradient in tensor memory
// across all tiles a CTA processes; one flush per CTA adds them to the FP32 gradient.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "rx_guide.h"
#include "rx_internal.h"
#include "rx_tc.cuh"

namespace rx {

constexpr uint32_t kDiagARegion = 96u << 10;   // A operand region (bytes)
constexpr uint32_t kDiagBRegion = 100u << 10;  // B operand region
constexpr uint32_t kDiagSmem = kDiagARegion + kDiagBRegion + 64;

// D = A * B^T on one CTA of 128 threads. A: M x K, B: N x K (row-major bf16 in global
// memory), placed in shared memory in the K-major or MN-major core-matrix view. Every
// TMEM lane (128) x N columns is zeroed first and written out, so rows >= M show where an
// M = 64 accumulator lands.
__global__ void __launch_bounds__(128) k_diag_umma(const uint16_t* A, const uint16_t* B, float* D, uint32_t M,
                                                   uint32_t N, uint32_t K, int a_mn, int b_mn, int* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  unsigned char* sa = smem;
  unsigned char* sb = smem + kDiagARegion;
  const int tid = threadIdx.x, warp = tid >> 5;
  // stage operands
  for (uint32_t i = tid; i < M * K; i += blockDim.x) {
    uint32_t m = i / K, k = i % K;
    uint32_t off = a_mn ? tc::core_off(k, m, M) : tc::core_off(m, k, K);
    *reinterpret_cast<uint16_t*>(sa + off) = A[i];
  }
  for (uint32_t i = tid; i < N * K; i += blockDim.x) {
    uint32_t n = i / K, k = i % K;
    uint32_t off = b_mn ? tc::core_off(k, n, N) : tc::core_off(n, k, K);
    *reinterpret_cast<uint16_t*>(sb + off) = B[i];
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  float z[16];
#pragma unroll
  for (int i = 0; i < 16; i++) z[i] = 0.0f;
  for (uint32_t c = 0; c < N; c += 16) tc::tmem_st16(tbase + lane_base + c, z);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (tid == 0) {
    uint32_t idesc = tc::idesc_bf16(M, N, a_mn != 0, b_mn != 0);
    uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
    for (uint32_t k0 = 0; k0 < K; k0 += 16) {
      uint64_t ad = a_mn ? tc::sdesc(a0 + tc::core_off(k0, 0, M), (M >> 3) * 128u, 128u)
                         : tc::sdesc(a0 + tc::core_off(0, k0, K), 128u, (K >> 3) * 128u);
      uint64_t bd = b_mn ? tc::sdesc(b0 + tc::core_off(k0, 0, N), (N >> 3) * 128u, 128u)
                         : tc::sdesc(b0 + tc::core_off(0, k0, K), 128u, (K >> 3) * 128u);
      tc::mma_bf16(tbase, ad, bd, idesc, k0 > 0);
    }
    tc::mma_commit(&bar);
  }
  bool ok = tc::mbar_wait(&bar, 0);
  tc::tc_fence_after();
  if (!ok) {
    if ((tid & 31) == 0) atomicExch(status, 1);
  } else {
    for (uint32_t c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(tbase + lane_base + c, v);
#pragma unroll
      for (int i = 0; i < 16; i++) D[(size_t)tid * N + c + i] = v[i];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 128);
}

// Back-to-back tcgen05.mma issue from one thread: `count` MMAs of M = 128, K = 16 and the
// given N (BF16, FP32 accumulation, operands in shared memory), timed with the SM clock
// from the first issue to the last issue and to the completion of all. Shared memory
// holds A (128 x 64) and B (256 x 64) BF16 tiles; each MMA reads one K = 16 slice.
constexpr uint32_t kRateSmem = (128 + 256) * 64 * 2;
__global__ void __launch_bounds__(128, 1) k_diag_umma_rate(uint32_t N, uint32_t count, unsigned long long* clk,
                                                           int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  for (uint32_t i = threadIdx.x; i < kRateSmem / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(sm)[i] = make_uint4(0x3f803f80u, 0u, 0x3f803f80u, 0u);  // 1.0 / 0.0 pairs
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&tbase, 256);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (threadIdx.x == 0) {
    const uint32_t id = tc::idesc_bf16(128, N, false, false);
    const uint32_t a0 = tc::smem_u32(sm), b0 = tc::smem_u32(sm + 128 * 64 * 2);
    const uint32_t sbo = 8u * 128u;  // K = 64: the next 8 rows
    const long long t0 = clock64();
    for (uint32_t m = 0; m < count; m++) {
      const uint32_t k0 = 16u * (m & 3u);
      tc::mma_bf16(tbase, tc::sdesc(a0 + tc::core_off(0, k0, 64), 128u, sbo),
                   tc::sdesc(b0 + tc::core_off(0, k0, 64), 128u, sbo), id, m > 0);
    }
    const long long t1 = clock64();
    tc::mma_commit(&bar);
    const bool ok = tc::mbar_wait(&bar, 0);
    const long long t2 = clock64();
    clk[0] = (unsigned long long)(t1 - t0);
    clk[1] = (unsigned long long)(t2 - t0);
    if (!ok) *status = 1;
  }
  tc::tc_fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tbase, 256);
}

// =======================================================================================
// Network kernels
// =======================================================================================
using namespace guide;

// Tensor-memory placement of an M = 64 accumulator (cta_group::1): row r in lane
// 32 (r / 16) + r % 16 (lanes 0..15 of each 32-lane quarter) when set, else lane r.
#ifndef RX_M64_SPLIT
#define RX_M64_SPLIT 1
#endif
// Row of an M = 64 accumulator that tensor-memory lane `lane` (0..127) holds, or -1.
__device__ __forceinline__ int m64_row(int lane) {
#if RX_M64_SPLIT
  return (lane & 31) < 16 ? (lane >> 5) * 16 + (lane & 15) : -1;
#else
  return lane < 64 ? lane : -1;
#endif
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // a in the low half (lower address)
  return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xFFFF0000u); }

__device__ __forceinline__ void store_chunk(unsigned char* base, uint32_t off, const float (&f)[8]) {
  uint4 u;
  u.x = pack_bf16(f[0], f[1]);
  u.y = pack_bf16(f[2], f[3]);
  u.z = pack_bf16(f[4], f[5]);
  u.w = pack_bf16(f[6], f[7]);
  *reinterpret_cast<uint4*>(base + off) = u;
}

// Encodes one query (position, normal, outgoing direction) into row s of the 128 x 80
// input tile. Feature j < 72: coordinate c = j / 24, frequency f = (j % 24) / 2,
// sin (j even) or cos (j odd) of pi 2^f p_c with p_c = (x_c - min_c) / extent_c;
// 72..74 normal, 75..77 outgoing direction, 78 = 1, 79 = 0. Frequency 0 comes from
// sincospif, each next one from the double-angle identities (sin 2a = 2 sin a cos a,
// cos 2a = (cos a - sin a)(cos a + sin a)): the angle error doubles per step, about
// 1e-4 at f = 11, far below the BF16 rounding of the features (4e-3).
__device__ void encode_row(const float (&q)[9], bool valid, const Box& box, unsigned char* A0, int s) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float p = valid ? __fdiv_rn(__fsub_rn(q[c], box.mn[c]), box.ext[c]) : 0.0f;
    float sn = 0.0f, cs = 0.0f;
    if (valid) sincospif(p, &sn, &cs);
#pragma unroll
    for (int part = 0; part < 3; part++) {  // 4 frequencies = 8 features = one 16-byte row chunk
      float f[8];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        f[2 * t] = sn;
        f[2 * t + 1] = cs;
        float s2 = 2.0f * sn * cs, c2 = (cs - sn) * (cs + sn);
        sn = s2;
        cs = c2;
      }
      store_chunk(A0, tc::core_off(s, c * 24 + part * 8, kIn), f);
    }
  }
  float f[8] = {q[3], q[4], q[5], q[6], q[7], q[8], 1.0f, 0.0f};
  if (!valid)
#pragma unroll
    for (int t = 0; t < 8; t++) f[t] = 0.0f;
  store_chunk(A0, tc::core_off(s, 72, kIn), f);
}

// Hidden-layer epilogue: the thread's accumulator row (64 columns) -> ReLU -> BF16 row s.
__device__ __forceinline__ void epi_relu(uint32_t tacc, unsigned char* out, int s) {
#pragma unroll
  for (int c0 = 0; c0 < kHid; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tacc + c0, v);
    float a[8], b[8];
#pragma unroll
    for (int i = 0; i < 8; i++) {
      a[i] = fmaxf(v[i], 0.0f);
      b[i] = fmaxf(v[8 + i], 0.0f);
    }
    store_chunk(out, tc::core_off(s, c0, kHid), a);
    store_chunk(out, tc::core_off(s, c0 + 8, kHid), b);
  }
}

__device__ __forceinline__ void load_raw(uint32_t tacc, float (&raw)[48]) {
#pragma unroll
  for (int c0 = 0; c0 < 48; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tacc + c0, v);
#pragma unroll
    for (int i = 0; i < 16; i++) raw[c0 + i] = v[i];
  }
}

constexpr float kLogKMin = -4.0f, kLogKMax = 8.0f;

// Lobe j of the raw outputs: log weight (log-softmax), concentration, mean, and the log
// of the vMF normaliser kappa / (2 pi (1 - e^{-2 kappa})).
struct Lobe {
  float logpi, kappa, mu[3], len, lognorm;
  bool kin;  // log-concentration inside its clamp range (gradient flows)
};
__device__ __forceinline__ void decode(const float (&raw)[48], Lobe (&L)[kLobes]) {
  float amax = raw[0];
#pragma unroll
  for (int j = 1; j < kLobes; j++) amax = fmaxf(amax, raw[5 * j]);
  float z = 0.0f;
#pragma unroll
  for (int j = 0; j < kLobes; j++) z += expf(raw[5 * j] - amax);
  float logz = amax + logf(z);
#pragma unroll
  for (int j = 0; j < kLobes; j++) {
    Lobe& l = L[j];
    l.logpi = raw[5 * j] - logz;
    float b = raw[5 * j + 1];
    l.kin = b > kLogKMin && b < kLogKMax;
    l.kappa = expf(fminf(fmaxf(b, kLogKMin), kLogKMax));
    float m0 = raw[5 * j + 2], m1 = raw[5 * j + 3], m2 = raw[5 * j + 4];
    l.len = fmaxf(sqrtf(m0 * m0 + m1 * m1 + m2 * m2), 1e-6f);
    l.mu[0] = m0 / l.len;
    l.mu[1] = m1 / l.len;
    l.mu[2] = m2 / l.len;
    l.lognorm = logf(l.kappa) - logf(2.0f * RX_PI) - logf(-expm1f(-2.0f * l.kappa));
  }
}

// -scale * log q(wi) and its gradient with respect to the 40 raw outputs (returns the former).
__device__ float mix_loss_grad(const float (&raw)[48], const float (&wi)[3], float scale, float (&dz)[48]) {
  Lobe L[kLobes];
  decode(raw, L);
  float lv[kLobes], t[kLobes];
  float mx = -INFINITY;
#pragma unroll
  for (int j = 0; j < kLobes; j++) {
    t[j] = L[j].mu[0] * wi[0] + L[j].mu[1] * wi[1] + L[j].mu[2] * wi[2];
    lv[j] = L[j].logpi + L[j].lognorm + L[j].kappa * (t[j] - 1.0f);
    mx = fmaxf(mx, lv[j]);
  }
  float sum = 0.0f;
#pragma unroll
  for (int j = 0; j < kLobes; j++) sum += expf(lv[j] - mx);
  float lq = mx + logf(sum);
#pragma unroll
  for (int j = 0; j < kLobes; j++) {
    float g = expf(lv[j] - lq);  // responsibility
    float pi = expf(L[j].logpi);
    float k = L[j].kappa;
    dz[5 * j] = scale * (pi - g);
    float dk = 1.0f - 2.0f * k / expm1f(2.0f * k) + k * (t[j] - 1.0f);  // kappa * d log v / d kappa
    dz[5 * j + 1] = L[j].kin ? -scale * g * dk : 0.0f;
    float c = -scale * g * k / L[j].len;
#pragma unroll
    for (int a = 0; a < 3; a++) dz[5 * j + 2 + a] = c * (wi[a] - t[j] * L[j].mu[a]);
  }
#pragma unroll
  for (int i = kOutUsed; i < 48; i++) dz[i] = 0.0f;
  return -scale * lq;
}

// Mixture for sampling / evaluation: per lobe weight, kappa, mean, weight x normaliser
// (kLobes x kLobeFloats floats, written as 16-byte stores; `out` 16-byte aligned).
__device__ void mix_store(const float (&raw)[48], float* out) {
  Lobe L[kLobes];
  decode(raw, L);
  float o[kLobes * kLobeFloats];
#pragma unroll
  for (int j = 0; j < kLobes; j++) {
    o[j * kLobeFloats + 0] = expf(L[j].logpi);
    o[j * kLobeFloats + 1] = L[j].kappa;
    o[j * kLobeFloats + 2] = L[j].mu[0];
    o[j * kLobeFloats + 3] = L[j].mu[1];
    o[j * kLobeFloats + 4] = L[j].mu[2];
    o[j * kLobeFloats + 5] = expf(L[j].logpi + L[j].lognorm);
  }
  float4* o4 = reinterpret_cast<float4*>(out);
#pragma unroll
  for (int k = 0; k < kLobes * kLobeFloats / 4; k++) o4[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
}

__device__ float mix_pdf_raw(const float (&raw)[48], const float (&wi)[3]) {
  Lobe L[kLobes];
  decode(raw, L);
  float q = 0.0f;
#pragma unroll
  for (int j = 0; j < kLobes; j++) {
    float t = L[j].mu[0] * wi[0] + L[j].mu[1] * wi[1] + L[j].mu[2] * wi[2];
    q += expf(L[j].logpi + L[j].lognorm + L[j].kappa * (t - 1.0f));
  }
  return q;
}

// Issues the forward MMAs of layer l (A: 128 x K K-major, W: 64 x K K-major) into `tacc`.
__device__ __forceinline__ void issue_fwd(uint32_t tacc, const unsigned char* A, const unsigned char* W, int K) {
  const uint32_t id = tc::idesc_bf16(128, 64, false, false);
  const uint32_t a0 = tc::smem_u32(A), w0 = tc::smem_u32(W);
  const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint64_t ad = tc::sdesc(a0 + tc::core_off(0, k0, K), 128u, sbo);
    uint64_t wd = tc::sdesc(w0 + tc::core_off(0, k0, K), 128u, sbo);
    tc::mma_bf16(tacc, ad, wd, id, k0 > 0);
  }
}

// Block-wide barrier that also orders tensor-core work and generic shared-memory writes.
__device__ __forceinline__ void tc_sync() {
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
}

// Shared-memory plan of the network kernels (bytes from the dynamic base).
constexpr uint32_t kSmW = 0;                         // weight image, then the per-tile buffers
constexpr uint32_t kActBytes = 128 * kHid * 2;       // one 128 x 64 BF16 activation tile
constexpr int kInferTiles = 4;  // inference tiles in flight per CTA, one warpgroup each
// per tile: the 128 x 80 input (its first 16 KB also hold the odd layers' outputs) and one
// 128 x 64 activation buffer
constexpr uint32_t kInferTileBytes = 128 * kIn * 2 + kActBytes;
constexpr uint32_t kSmInfer = kImgBytes + kInferTiles * kInferTileBytes;

// Loads the weight image into shared memory with bulk copies (one per layer).
__device__ __forceinline__ void load_weights(unsigned char* sm, const unsigned char* img, uint64_t* bar) {
  tc::mbar_expect_tx(bar, kImgBytes);
#pragma unroll
  for (int l = 0; l < 5; l++) {
    uint32_t bytes = (l == 4 ? kImgBytes : layer_img(l + 1)) - layer_img(l);
    tc::bulk_g2s(sm + kSmW + layer_img(l), img + layer_img(l), bytes, bar);
  }
}

// ---- inference -------------------------------------------------------------------------
// Each IO splits its input into prefetch (the first, independent loads, issued one tile
// ahead) and finish (the rest), and stores a query's result with 16-byte stores.

// Queries from records (x, n, wo, wi, ...): raw outputs and the mixture pdf at wi.
struct RecordIO {
  const float* recs;
  float* raw_out;  // n x 40 (optional)
  float* pdf_out;  // n (optional)
  struct Pre {
    float4 a, b, c;
  };
  __device__ Pre prefetch(uint32_t i, bool valid) const {
    Pre p{};
    if (valid) {
      const float4* r = reinterpret_cast<const float4*>(recs + (size_t)i * kRec);
      p.a = r[0];
      p.b = r[1];
      p.c = r[2];
    }
    return p;
  }
  __device__ bool finish(const Pre& p, uint32_t, bool valid, float (&q)[9], float (&wi)[3]) const {
    q[0] = p.a.x; q[1] = p.a.y; q[2] = p.a.z; q[3] = p.a.w; q[4] = p.b.x; q[5] = p.b.y; q[6] = p.b.z; q[7] = p.b.w;
    q[8] = p.c.x;
    wi[0] = p.c.y; wi[1] = p.c.z; wi[2] = p.c.w;
    return valid;
  }
  __device__ void store(uint32_t i, const float (&raw)[48], const float (&wi)[3]) const {
    if (raw_out) {
      float4* o = reinterpret_cast<float4*>(raw_out + (size_t)i * kOutUsed);
#pragma unroll
      for (int k = 0; k < kOutUsed / 4; k++) o[k] = make_float4(raw[4 * k], raw[4 * k + 1], raw[4 * k + 2], raw[4 * k + 3]);
    }
    if (pdf_out) pdf_out[i] = mix_pdf_raw(raw, wi);
  }
};

// Queries from the wavefront: the hit point of each live path, if its surface is guided
// (diffuse, glossy or Phong, seen from the front, the path not inside an object). The
// path's scene is scenes[info.w >> 16].
struct PathIO {
  const DevScene* scenes;
  PathSoA P;
  const int2* hit;
  float* lobes;
  struct Pre {
    int2 h;
    int4 inf;
    float4 o, d;
  };
  __device__ Pre prefetch(uint32_t i, bool valid) const {
    Pre p;
    p.h = make_int2(-1, 0);
    if (valid) {
      p.h = hit[i];
      p.inf = P.info[i];
      p.o = P.o[i];
      p.d = P.d[i];
    }
    return p;
  }
  __device__ bool finish(const Pre& p, uint32_t i, bool valid, float (&q)[9], float (&wi)[3]) const {
    wi[0] = wi[1] = wi[2] = 0.0f;
    if (!valid) return false;
    const DevScene& S = scenes[(uint32_t)p.inf.w >> 16];
    bool ok = p.h.x >= 0 && p.inf.z < 0;
    int obj = ok ? (int)__ldg(&S.tri_obj[p.h.x]) : -1;
    if (ok) {
      uint32_t m = S.objects[obj].material;
      ok = m == kDiffuse || m == kGlossy || m == kPhong;
    }
    if (!ok) {
      lobes[(size_t)i * kLobeStride] = -1.0f;  // not guided
      return false;
    }
    float t = __int_as_float(p.h.y);
    F3 x = F3{p.o.x, p.o.y, p.o.z} + F3{p.d.x, p.d.y, p.d.z} * t;
    TriGeom g = tri_geom(S, p.h.x);
    F3 nn = world_normal(g, S.objects[obj].has_normals, x);
    if (nn.x * p.d.x + nn.y * p.d.y + nn.z * p.d.z > 0.0f) {
      lobes[(size_t)i * kLobeStride] = -1.0f;
      return false;
    }
    q[0] = x.x; q[1] = x.y; q[2] = x.z; q[3] = nn.x; q[4] = nn.y; q[5] = nn.z;
    q[6] = -p.d.x; q[7] = -p.d.y; q[8] = -p.d.z;
    return true;
  }
  __device__ void store(uint32_t i, const float (&raw)[48], const float (&)[3]) const {
    mix_store(raw, lobes + (size_t)i * kLobeStride);
  }
};

// Barrier of warpgroup g (its 128 threads, named barrier g + 1) that also orders
// tensor-core work and generic shared-memory writes; and its AND-reduction.
__device__ __forceinline__ void wg_sync(int g) {
  tc::fence_async_smem();
  tc::tc_fence_before();
  asm volatile("bar.sync %0, 128;" ::"r"(g + 1) : "memory");
  tc::tc_fence_after();
}
__device__ __forceinline__ bool wg_and(int g, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(g + 1)
      : "memory");
  return r != 0;
}

// Network k of a grouped launch: the segment of seg[0..nnet] holding row r.
__device__ __forceinline__ int seg_of(const uint32_t* seg, int nnet, uint32_t r) {
  int lo = 0, hi = nnet - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&seg[mid]) <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Persistent inference: kInferTiles warpgroups per CTA share the weight image and each
// runs its own 128-sample tiles through the five layers (its own input / activation
// buffers, TMEM columns 64 g .. 64 g + 63, mbarrier, and MMA-issuing thread), so several
// tiles' MMA -> epilogue chains interleave on the SM. The next tile's inputs are loaded
// while the current one runs. A CTA's step covers kInferTiles consecutive tiles (tile
// 4 st + g for warpgroup g).
//
// GROUPED: rows[r] (or -1 for padding) name the queries, and network k owns rows
// [seg[k], seg[k + 1]) (multiples of kGroupRows, so a step's four tiles share one
// network). When a step's network differs from the staged one, the CTA waits until every
// warpgroup is done with the old weights and stages the new ones (bulk copy, 43 KB).
// Steps run in increasing row order per CTA, so a CTA stages each network at most once.
// Every warpgroup runs the same number of steps; a failed wait skips the remaining work
// instead of leaving the loop, so the CTA-wide barriers stay matched.
template <class IO, bool GROUPED>
__global__ void __launch_bounds__(128 * kInferTiles, 1)
    k_guide_infer(IO io, const unsigned* count, uint32_t n_host, const NetDev* nets, int nnet, const int* rows,
                  const uint32_t* seg, const uint32_t* pass) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar_mma[kInferTiles], bar_w;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, s = tid & 127;
  uint32_t n = 0, nsteps;
  if constexpr (GROUPED) {
    nsteps = __ldg(&seg[nnet]) / kGroupRows;
  } else {
    if (pass && *pass < nets[0].warmup) return;
    n = count ? *count : n_host;
    nsteps = (n + kGroupRows - 1) / kGroupRows;
  }
  if (blockIdx.x >= nsteps) return;
  if (tid == 0) {
    for (int k = 0; k < kInferTiles; k++) tc::mbar_init(&bar_mma[k], 1);
    tc::mbar_init(&bar_w, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  int net = GROUPED ? seg_of(seg, nnet, blockIdx.x * kGroupRows) : 0;
  if (tid == 0) load_weights(sm, nets[net].img, &bar_w);
  if (warp == 0) tc::tmem_alloc(&tmem_base, 64 * kInferTiles);
  tc_sync();
  const uint32_t tcol = tmem_base + 64u * (uint32_t)g;
  const uint32_t tacc = tcol + ((uint32_t)((warp & 3) * 32) << 16);
  bool ok = __syncthreads_and(tc::mbar_wait(&bar_w, 0));
  uint32_t wph = 1;
  Box box = nets[net].box;
  uint32_t ph = 0;
  unsigned char* A0 = sm + kImgBytes + (uint32_t)g * kInferTileBytes;
  unsigned char* A1 = A0 + 128 * kIn * 2;
  // the query of row r: its index and whether it exists
  auto query = [&](uint32_t r, uint32_t& i) -> bool {
    if constexpr (GROUPED) {
      if (r >= nsteps * kGroupRows) return false;
      int q = __ldg(&rows[r]);
      i = (uint32_t)q;
      return q >= 0;
    } else {
      i = r;
      return r < n;
    }
  };
  uint32_t st = blockIdx.x;
  uint32_t qi = 0;
  bool qv = query((st * kInferTiles + (uint32_t)g) * kTile + (uint32_t)s, qi);
  typename IO::Pre pre = io.prefetch(qi, qv);
  for (; st < nsteps; st += gridDim.x) {
    if constexpr (GROUPED) {
      const int j = seg_of(seg, nnet, st * kGroupRows);  // the same for the whole CTA
      if (j != net) {
        tc::tc_fence_before();
        ok = __syncthreads_and(ok);  // every warpgroup's MMAs on the old weights are complete
        tc::tc_fence_after();
        if (ok && tid == 0) load_weights(sm, nets[j].img, &bar_w);
        if (ok) ok = __syncthreads_and(tc::mbar_wait(&bar_w, wph));
        wph ^= 1;
        net = j;
        box = nets[j].box;
      }
    } else {
      if (!ok) break;
    }
    const uint32_t tile = st * kInferTiles + (uint32_t)g;
    const uint32_t i = qi;
    float q[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, wi[3] = {0, 0, 0};
    const bool valid = io.finish(pre, i, qv, q, wi);
    qv = query(((st + gridDim.x) * kInferTiles + (uint32_t)g) * kTile + (uint32_t)s, qi);
    pre = io.prefetch(qi, qv);
    if (!GROUPED && tile * kTile >= n) continue;  // this warpgroup's tile is past the end
    if (!ok) continue;
    encode_row(q, valid, box, A0, s);
    wg_sync(g);
    float raw[48];
    for (int l = 0; l < 5; l++) {
      // layer l reads A0 (l = 0, 2, 4) or A1 (l = 1, 3) and writes the other
      const unsigned char* A = (l & 1) ? A1 : A0;
      if (s == 0) {
        issue_fwd(tcol, A, sm + kSmW + layer_img(l), layer_k(l));
        tc::mma_commit(&bar_mma[g]);
      }
      ok = wg_and(g, tc::mbar_wait(&bar_mma[g], ph));
      ph ^= 1;
      tc::tc_fence_after();
      if (!ok) break;
      if (l < 4) epi_relu(tacc, (l & 1) ? A0 : A1, s);
      else load_raw(tacc, raw);
      wg_sync(g);
    }
    if (ok && valid) io.store(i, raw, wi);
  }
  if (!ok && s == 0) atomicExch(nets[net].status, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem_base, 64 * kInferTiles);
}

// ---- training ----------------------------------------------------------------------
// The records a training step reads: with step >= 0, the step-th window of `len` records
// of the live count (device count clipped to cap, wrapping); else the first `len`
// records (clipped to cap).
__device__ __forceinline__ void train_window(const RecSeg& R, int step, uint32_t& lo, uint32_t& hi) {
  uint32_t n = R.count ? min(*R.count, R.cap) : R.cap;
  if (step >= 0) {
    uint32_t L = min(R.len, n);
    lo = n > R.len ? (uint32_t)(((uint64_t)step * R.len) % (n - R.len + 1)) : 0u;
    hi = lo + L;
  } else {
    lo = 0;
    hi = min(R.len, n);
  }
}

// Whether a network takes training step `step` of the render pass *pass (pass null:
// outside a render, always): inside its training passes and its steps per pass.
__device__ __forceinline__ bool net_trains(const NetDev& N, const uint32_t* pass, int step) {
  return !pass || (*pass < N.train && (uint32_t)step < N.steps_per_pass);
}

// Clears each training network's step scratch (weight sum, count, loss).
__global__ void k_net_clear(const NetDev* nets, int nnet, const uint32_t* pass, int step) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nnet && net_trains(nets[j], pass, step)) {
    nets[j].scratch[0] = 0.0f;
    nets[j].scratch[1] = 0.0f;
    nets[j].scratch[2] = 0.0f;
  }
}

// Sum of record weights and number of records per network (the loss normalisation);
// blocks [j * per, (j + 1) * per) serve network j.
__global__ void k_weight_sum(const NetDev* nets, const RecSeg* segs, int per, int step, const uint32_t* pass) {
  const int j = blockIdx.x / per;
  if (!net_trains(nets[j], pass, step)) return;
  const RecSeg R = segs[j];
  uint32_t lo, end;
  train_window(R, step, lo, end);
  float acc = 0.0f;
  unsigned c = 0;
  for (uint32_t i = lo + (blockIdx.x % per) * blockDim.x + threadIdx.x; i < end; i += per * blockDim.x) {
    acc += R.recs[(size_t)i * kRec + 12];
    c++;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0 && c) {
    atomicAdd(nets[j].scratch, acc);
    atomicAdd(nets[j].scratch + 1, (float)c);
  }
}

// Gradient of the batch loss over the records a window selects (train_window): forward
// and backward per tile, weight gradients accumulated in tensor memory across all tiles
// a CTA processes, flushed once per CTA into the network's FP32 gradient. The network's
// scratch holds {sum w, count}; weights are clipped at 32 x their batch mean before
// normalisation by the sum. CTAs [j * per, (j + 1) * per) train network j.
//
// A CTA carries kTrainTiles tiles of 128 samples at once, one warpgroup per tile (thread
// s of warpgroup g owns sample s of tile g, TMEM lane s of that tile's accumulator). The
// warpgroups run independently (own MMA-issuing thread, mbarrier and named barrier), so
// one tile's epilogues overlap the other's MMAs; both add into the shared
// weight-gradient accumulators, zeroed once, which the tensor core updates one MMA at a
// time. The 128 x 80 input tile is not kept: it lives in the region of activations 3-4
// during the forward pass and is encoded again from the records for the last weight
// gradient.
constexpr int kTrainTiles = 2;
constexpr uint32_t kTrainTileBytes = 5 * kActBytes;  // A1, A2, A3|A4 (A0 alias), dZ
constexpr uint32_t kSmTrain2 = kImgBytes + kTrainTiles * kTrainTileBytes;
constexpr uint32_t kDwCols = 336;  // TMEM columns of the five weight-gradient accumulators

__device__ __forceinline__ void load_record(const float* recs, uint32_t i, float (&q)[9], float (&wi)[3], float& w) {
  const float4* r = reinterpret_cast<const float4*>(recs + (size_t)i * kRec);
  float4 a = r[0], b = r[1], c = r[2], e = r[3];
  q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w; q[4] = b.x; q[5] = b.y; q[6] = b.z; q[7] = b.w; q[8] = c.x;
  wi[0] = c.y; wi[1] = c.z; wi[2] = c.w;
  w = e.x;
}

__global__ void __launch_bounds__(128 * kTrainTiles, 1)
    k_guide_train(const NetDev* nets, const RecSeg* segs, int per, int step, const uint32_t* pass) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar_mma[kTrainTiles], bar_w;
  __shared__ uint32_t tmem_base;
  __shared__ float red[4 * kTrainTiles];
  const int tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, s = tid & 127;
  const int j = blockIdx.x / per, part = blockIdx.x % per;
  const NetDev& N = nets[j];
  if (!net_trains(N, pass, step)) return;
  const RecSeg R = segs[j];
  const float* recs = R.recs;
  const Box box = N.box;
  float* grad = N.grad;
  uint32_t first, end;
  train_window(R, step, first, end);
  const uint32_t n = end - first;
  const uint32_t ntiles = (n + kTile - 1) / kTile;
  if ((uint32_t)part * kTrainTiles >= ntiles) return;
  if (tid == 0) {
    for (int k = 0; k < kTrainTiles; k++) tc::mbar_init(&bar_mma[k], 1);
    tc::mbar_init(&bar_w, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) load_weights(sm, N.img, &bar_w);
  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  tc_sync();
  const uint32_t T0 = tmem_base;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  // TMEM columns: per tile one 64-column accumulator (forward, then dA); the shared dW
  const uint32_t t_dw[5] = {T0 + 128, T0 + 208, T0 + 272, T0 + 336, T0 + 400};
  if (g == 0) {  // zero the weight-gradient accumulators (every MMA into them accumulates)
    const float z[16] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t c0 = 0; c0 < kDwCols; c0 += 16) tc::tmem_st16(T0 + 128 + lane_off + c0, z);
  }
  unsigned char* A1 = sm + kImgBytes + (uint32_t)g * kTrainTileBytes;  // this warpgroup's buffers
  unsigned char* A2 = A1 + kActBytes;
  unsigned char* A34 = A1 + 2 * kActBytes;  // A3, A4; A0 (20 KB) aliases it
  unsigned char* dZ = A1 + 4 * kActBytes;
  unsigned char* Al[5] = {A34, A1, A2, A34, A34 + kActBytes};
  const uint32_t tacc_col = T0 + 64u * (uint32_t)g;
  const uint32_t t_acc = tacc_col + lane_off;
  const float total = N.scratch[0], cnt = fmaxf(N.scratch[1], 1.0f);
  const float wclip = 32.0f * total / cnt;
  const float inv_total = total > 0.0f ? 1.0f / total : 0.0f;
  tc::tc_fence_before();
  bool ok = __syncthreads_and(tc::mbar_wait(&bar_w, 0));
  tc::tc_fence_after();
  uint32_t ph = 0;
  float loss = 0.0f;
  for (uint32_t tile = (uint32_t)part * kTrainTiles + (uint32_t)g; ok && tile < ntiles;
       tile += (uint32_t)per * kTrainTiles) {
    const uint32_t i = first + tile * kTile + s;
    const bool valid = i < end;
    float q[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, wi[3] = {0, 0, 0}, w = 0.0f;
    if (valid) {
      load_record(recs, i, q, wi, w);
      w = fminf(w, wclip) * inv_total;
    }
    encode_row(q, valid, box, Al[0], s);
    wg_sync(g);
    // forward
    for (int l = 0; l < 5 && ok; l++) {
      if (s == 0) {
        issue_fwd(tacc_col, Al[l], sm + kSmW + layer_img(l), layer_k(l));
        tc::mma_commit(&bar_mma[g]);
      }
      ok = wg_and(g, tc::mbar_wait(&bar_mma[g], ph));
      ph ^= 1;
      tc::tc_fence_after();
      if (!ok) break;
      if (l < 4) {
        epi_relu(t_acc, Al[l + 1], s);
      } else {
        float raw[48], dz[48];
        load_raw(t_acc, raw);
        if (valid && w > 0.0f) {
          loss += mix_loss_grad(raw, wi, w, dz);
        } else {
#pragma unroll
          for (int k = 0; k < 48; k++) dz[k] = 0.0f;
        }
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 8) {
          float f[8];
#pragma unroll
          for (int k = 0; k < 8; k++) f[k] = c0 + k < 48 ? dz[c0 + k] : 0.0f;
          store_chunk(dZ, tc::core_off(s, c0, kOut), f);
        }
      }
      wg_sync(g);
    }
    // backward: dZ holds dZ_{l+1}; dW_l += dZ^T A_l; dA_l = dZ W_l
    for (int l = 4; l >= 0 && ok; l--) {
      const int K = layer_k(l);
      if (l == 0) {  // the input tile again, into the (now free) activation 3-4 region
        encode_row(q, valid, box, Al[0], s);
        wg_sync(g);
      }
      if (s == 0) {
        const uint32_t w0 = tc::smem_u32(sm + kSmW + layer_img(l));
        const uint32_t id_w = tc::idesc_bf16(64, (uint32_t)K, true, true);
        const uint32_t id_a = tc::idesc_bf16(128, (uint32_t)K, false, true);
        const uint32_t dz0 = tc::smem_u32(dZ), a0 = tc::smem_u32(Al[l]);
        for (int s0 = 0; s0 < kTile; s0 += 16) {
          uint64_t ad = tc::sdesc(dz0 + tc::core_off(s0, 0, kOut), (kOut >> 3) * 128u, 128u);
          uint64_t bd = tc::sdesc(a0 + tc::core_off(s0, 0, K), (uint32_t)(K >> 3) * 128u, 128u);
          tc::mma_bf16(t_dw[l], ad, bd, id_w, 1u);
        }
        if (l > 0) {
          for (int n0 = 0; n0 < kOut; n0 += 16) {
            uint64_t ad = tc::sdesc(dz0 + tc::core_off(0, n0, kOut), 128u, (kOut >> 3) * 128u);
            uint64_t bd = tc::sdesc(w0 + tc::core_off(n0, 0, K), (uint32_t)(K >> 3) * 128u, 128u);
            tc::mma_bf16(tacc_col, ad, bd, id_a, n0 > 0);
          }
        }
        tc::mma_commit(&bar_mma[g]);
      }
      ok = wg_and(g, tc::mbar_wait(&bar_mma[g], ph));
      ph ^= 1;
      tc::tc_fence_after();
      if (!ok) break;
      if (l > 0) {
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
          float v[16];
          tc::tmem_ld16(t_acc + c0, v);
          uint4 m0 = *reinterpret_cast<const uint4*>(Al[l] + tc::core_off(s, c0, kHid));
          uint4 m1 = *reinterpret_cast<const uint4*>(Al[l] + tc::core_off(s, c0 + 8, kHid));
          uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
          float a[8], b[8];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            a[2 * k] = bf16_lo(mw[k]) > 0.0f ? v[2 * k] : 0.0f;
            a[2 * k + 1] = bf16_hi(mw[k]) > 0.0f ? v[2 * k + 1] : 0.0f;
            b[2 * k] = bf16_lo(mw[4 + k]) > 0.0f ? v[8 + 2 * k] : 0.0f;
            b[2 * k + 1] = bf16_hi(mw[4 + k]) > 0.0f ? v[8 + 2 * k + 1] : 0.0f;
          }
          store_chunk(dZ, tc::core_off(s, c0, kHid), a);
          store_chunk(dZ, tc::core_off(s, c0 + 8, kHid), b);
        }
      }
      wg_sync(g);
    }
  }
  tc::tc_fence_before();
  ok = __syncthreads_and(ok);
  tc::tc_fence_after();
  // flush the weight-gradient accumulators (warpgroup 0 reads them)
  if (ok && g == 0) {
    const int row = m64_row(s);
    for (int l = 0; l < 5; l++) {
      const int K = layer_k(l);
      for (int c0 = 0; c0 < K; c0 += 16) {
        float v[16];
        tc::tmem_ld16(t_dw[l] + lane_off + c0, v);
        if (row >= 0)
#pragma unroll
          for (int k = 0; k < 16; k++) atomicAdd(&grad[layer_w(l) + row * K + c0 + k], v[k]);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if ((tid & 31) == 0) red[warp] = loss;
  if (!ok && tid == 0) atomicExch(N.status, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 0) {
    float t = 0.0f;
    for (int k = 0; k < 4 * kTrainTiles; k++) t += red[k];
    atomicAdd(N.scratch + 2, t);
  }
  if (warp == 0) tc::tmem_dealloc(T0, 512);
}

// Writes the BF16 image of FP32 parameters (core-matrix layout per layer).
__device__ __forceinline__ void image_store(unsigned char* img, int i, float w) {
  int l = 4;
  while (l > 0 && i < layer_w(l)) l--;
  int K = layer_k(l), r = (i - layer_w(l)) / K, c = (i - layer_w(l)) % K;
  *reinterpret_cast<__nv_bfloat16*>(img + layer_img(l) + tc::core_off(r, c, K)) = __float2bfloat16_rn(w);
}

__global__ void k_make_image(const float* w, unsigned char* img) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) image_store(img, i, w[i]);
}

// Adam (bias-corrected with the network's step count), then the BF16 image; clears the
// gradient. blockIdx.y = network.
__global__ void k_adam(const NetDev* nets, const uint32_t* pass, int step, float b1, float b2, float eps) {
  const NetDev& N = nets[blockIdx.y];
  if (!net_trains(N, pass, step)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float t = (float)(*N.step + 1u);
  const float c1 = 1.0f / (1.0f - powf(b1, t)), c2 = 1.0f / (1.0f - powf(b2, t));
  float gi = N.grad[i];
  N.grad[i] = 0.0f;
  float mi = b1 * N.m[i] + (1.0f - b1) * gi;
  float vi = b2 * N.v[i] + (1.0f - b2) * gi * gi;
  N.m[i] = mi;
  N.v[i] = vi;
  float wi = N.params[i] - N.lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  N.params[i] = wi;
  image_store(const_cast<unsigned char*>(N.img), i, wi);
}

// Counts the Adam step of every training network (after k_adam read the old count).
__global__ void k_net_step(const NetDev* nets, int nnet, const uint32_t* pass, int step) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nnet && net_trains(nets[j], pass, step)) *nets[j].step += 1u;
}

}  // namespace rx

using rx::DevBuf;
using rx::DeviceGuard;

extern "C" rx_status rx_diag_umma_gemm(rx_context* c, uint32_t M, uint32_t N, uint32_t K, int32_t a_mn,
                                       int32_t b_mn, const uint16_t* a, const uint16_t* b, float* d_out) {
  if (!c) return RX_ERR_INVALID;
  if (!a || !b || !d_out) return c->fail(RX_ERR_INVALID, "null buffer");
  if ((M != 64 && M != 128) || N < 16 || N > 128 || N % 16 || K < 16 || K > 128 || K % 16)
    return c->fail(RX_ERR_INVALID, "M must be 64 or 128, N 16..128 and K 16..128 in steps of 16");
  DeviceGuard g(c->device);
  DevBuf da, db, dd, ds;
  rx_status s;
  if ((s = c->cuda(da.alloc((size_t)M * K * 2), "alloc")) != RX_OK) return s;
  if ((s = c->cuda(db.alloc((size_t)N * K * 2), "alloc")) != RX_OK) return s;
  if ((s = c->cuda(dd.alloc((size_t)128 * N * 4), "alloc")) != RX_OK) return s;
  if ((s = c->cuda(ds.alloc(4), "alloc")) != RX_OK) return s;
  cudaMemcpy(da.p, a, (size_t)M * K * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(db.p, b, (size_t)N * K * 2, cudaMemcpyHostToDevice);
  cudaMemset(ds.p, 0, 4);
  cudaFuncSetAttribute(rx::k_diag_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rx::kDiagSmem);
  rx::k_diag_umma<<<1, 128, rx::kDiagSmem, c->stream>>>(da.as<uint16_t>(), db.as<uint16_t>(), dd.as<float>(), M, N,
                                                         K, a_mn, b_mn, ds.as<int>());
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "umma self-test")) != RX_OK) return s;
  int st = 0;
  cudaMemcpy(&st, ds.p, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(d_out, dd.p, (size_t)128 * N * 4, cudaMemcpyDeviceToHost);
  if (st) return c->fail(RX_ERR_TIMEOUT, "tensor-core MMA did not complete");
  return RX_OK;
}

extern "C" rx_status rx_diag_umma_rate(rx_context* c, uint32_t N, uint32_t count, double* issue_clk,
                                       double* done_clk) {
  if (!c) return RX_ERR_INVALID;
  if (!issue_clk || !done_clk) return c->fail(RX_ERR_INVALID, "null output");
  if ((N != 64 && N != 128 && N != 256) || count == 0 || count > 4096)
    return c->fail(RX_ERR_INVALID, "N must be 64, 128 or 256 and count 1..4096");
  DeviceGuard g(c->device);
  DevBuf dc, ds;
  rx_status s;
  if ((s = c->cuda(dc.alloc(2 * sizeof(unsigned long long)), "alloc")) != RX_OK) return s;
  if ((s = c->cuda(ds.alloc(4), "alloc")) != RX_OK) return s;
  cudaMemset(ds.p, 0, 4);
  cudaFuncSetAttribute(rx::k_diag_umma_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rx::kRateSmem);
  for (int rep = 0; rep < 2; rep++)  // the first launch warms the instruction cache
    rx::k_diag_umma_rate<<<1, 128, rx::kRateSmem, c->stream>>>(N, count, dc.as<unsigned long long>(), ds.as<int>());
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "umma rate")) != RX_OK) return s;
  unsigned long long h[2] = {0, 0};
  int st = 0;
  cudaMemcpy(h, dc.p, sizeof h, cudaMemcpyDeviceToHost);
  cudaMemcpy(&st, ds.p, 4, cudaMemcpyDeviceToHost);
  if (st) return c->fail(RX_ERR_TIMEOUT, "tensor-core MMA did not complete");
  *issue_clk = (double)h[0] / count;
  *done_clk = (double)h[1] / count;
  return RX_OK;
}

// =======================================================================================
// Host state and entry points
// =======================================================================================
namespace rx {

struct GuideState {
  rx_guide_options opt{};
  guide::Box box{};
  // params, Adam moments, gradient, BF16 image; scratch {sum w, count, loss}; status;
  // step count; device copies of this network's NetDev and of the record segment the
  // single-network entry points train on
  DevBuf params, m, v, grad, img, scratch, status, step, dnet, dseg;
  RecSeg seg_uploaded{};  // what dseg holds (uploaded again only when it changes)
  int sms = 152;
  bool ready = false;
};

void guide_free(GuideState* g) { delete g; }
bool guide_ready(const GuideState* g) { return g && g->ready; }

NetDev guide_net(const GuideState* g) {
  NetDev N{};
  N.img = g->img.as<unsigned char>();
  N.params = g->params.as<float>();
  N.m = g->m.as<float>();
  N.v = g->v.as<float>();
  N.grad = g->grad.as<float>();
  N.scratch = g->scratch.as<float>();
  N.status = g->status.as<int>();
  N.step = g->step.as<uint32_t>();
  N.box = g->box;
  N.lr = g->opt.learning_rate;
  N.frac = g->opt.bsdf_fraction;
  N.batch = g->opt.batch;
  N.warmup = g->opt.warmup_passes;
  N.train = g->opt.train_passes;
  N.steps_per_pass = g->opt.steps_per_pass;
  return N;
}

// Opts the network kernels into their shared-memory sizes, once per device.
static void set_kernel_smem() {
  static uint64_t done_mask = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && (done_mask >> dev) & 1) return;
  cudaFuncSetAttribute(k_guide_infer<RecordIO, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmInfer);
  cudaFuncSetAttribute(k_guide_infer<PathIO, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmInfer);
  cudaFuncSetAttribute(k_guide_infer<PathIO, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmInfer);
  cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmTrain2);
  if (dev < 64) done_mask |= 1ull << dev;
}

void guide_prepare() { set_kernel_smem(); }

cudaError_t guide_infer_wave(const NetDev* nets, int nnet, const DevScene* scenes, const PathSoA& P,
                             const unsigned* count, const int2* hit, float* lobes, const int* rows,
                             const uint32_t* seg, const uint32_t* pass, int sms, cudaStream_t s) {
  set_kernel_smem();
  PathIO io{scenes, P, hit, lobes};
  if (rows)
    k_guide_infer<PathIO, true><<<sms, 128 * kInferTiles, kSmInfer, s>>>(io, nullptr, 0, nets, nnet, rows, seg, pass);
  else
    k_guide_infer<PathIO, false><<<sms, 128 * kInferTiles, kSmInfer, s>>>(io, count, 0, nets, 1, nullptr, nullptr,
                                                                           pass);
  return cudaGetLastError();
}

// CTAs per network of a training launch: enough for its batch, and together about one
// per SM.
static int train_ctas_per_net(uint32_t batch, int nnet, int sms) {
  int need = (int)((batch + kTile * kTrainTiles - 1) / (kTile * kTrainTiles));
  return std::max(1, std::min(need, (sms + nnet - 1) / nnet));
}

// One training step of every network (gradient, and with `update` Adam and the step
// count) on the window `step` of its records (step < 0: the first len records).
static cudaError_t train_nets_step(const NetDev* nets, const RecSeg* segs, int nnet, int per, int step,
                                   const uint32_t* pass, bool update, int sms, cudaStream_t s) {
  set_kernel_smem();
  k_net_clear<<<(nnet + 127) / 128, 128, 0, s>>>(nets, nnet, pass, step);
  const int wper = std::max(1, std::min(4 * sms / nnet, 64));
  k_weight_sum<<<nnet * wper, 256, 0, s>>>(nets, segs, wper, step, pass);
  k_guide_train<<<nnet * per, 128 * kTrainTiles, kSmTrain2, s>>>(nets, segs, per, step, pass);
  if (update) {
    k_adam<<<dim3((kParams + 255) / 256, nnet), 256, 0, s>>>(nets, pass, step, 0.9f, 0.999f, 1e-8f);
    k_net_step<<<(nnet + 127) / 128, 128, 0, s>>>(nets, nnet, pass, step);
  }
  return cudaGetLastError();
}

cudaError_t guide_train_nets(const NetDev* nets, const RecSeg* segs, int nnet, int steps, uint32_t batch_max,
                             const uint32_t* pass, int sms, cudaStream_t s) {
  const int per = train_ctas_per_net(batch_max, nnet, sms);
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < steps && e == cudaSuccess; k++) e = train_nets_step(nets, segs, nnet, per, k, pass, true, sms, s);
  return e;
}

// One step of this network alone on n device records (the single-network entry points).
static cudaError_t train_step(GuideState* g, const float* recs, uint32_t n, cudaStream_t s, bool update) {
  const RecSeg R{recs, nullptr, n, n};
  if (std::memcmp(&R, &g->seg_uploaded, sizeof R) != 0) {
    cudaError_t e = cudaMemcpyAsync(g->dseg.p, &R, sizeof R, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    g->seg_uploaded = R;
  }
  const int per = train_ctas_per_net(n, 1, g->sms);
  return train_nets_step(g->dnet.as<NetDev>(), g->dseg.as<RecSeg>(), 1, per, -1, nullptr, update, g->sms, s);
}

}  // namespace rx

namespace {
// Seeded uniform in [-1, 1) from (seed, index): splitmix64.
float init_uniform(uint64_t seed, uint64_t i) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)((z >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
}

rx_status need_guide(rx_context* c) {
  if (!c) return RX_ERR_INVALID;
  if (!rx::guide_ready(c->guide)) return c->fail(RX_ERR_STATE, "guiding network not initialised (rx_guide_init)");
  return RX_OK;
}
}  // namespace

extern "C" rx_status rx_guide_init(rx_context* c, const rx_guide_options* opt, const float* box6) {
  if (!c || !opt) return RX_ERR_INVALID;
  if (!(opt->learning_rate > 0.0f) || !(opt->bsdf_fraction > 0.0f) || opt->bsdf_fraction > 1.0f || opt->batch == 0)
    return c->fail(RX_ERR_INVALID, "learning_rate > 0, 0 < bsdf_fraction <= 1 and batch > 0 required");
  float bmin[3], bmax[3];
  if (box6) {
    for (int k = 0; k < 3; k++) bmin[k] = box6[k], bmax[k] = box6[3 + k];
  } else {
    if (c->verts.empty()) return c->fail(RX_ERR_STATE, "no geometry for the encoding box (pass box6)");
    for (int k = 0; k < 3; k++) bmin[k] = INFINITY, bmax[k] = -INFINITY;
    for (size_t i = 0; i < c->verts.size(); i += 3)
      for (int k = 0; k < 3; k++) bmin[k] = std::min(bmin[k], c->verts[i + k]), bmax[k] = std::max(bmax[k], c->verts[i + k]);
  }
  for (int k = 0; k < 3; k++)
    if (!(bmax[k] > bmin[k])) return c->fail(RX_ERR_INVALID, "degenerate encoding box");
  DeviceGuard dg(c->device);
  auto* g = new rx::GuideState();
  g->opt = *opt;
  cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, c->device);
  for (int k = 0; k < 3; k++) g->box.mn[k] = bmin[k], g->box.ext[k] = bmax[k] - bmin[k];
  const size_t pb = rx::guide::kParams * sizeof(float);
  rx_status s = RX_OK;
  for (DevBuf* b : {&g->params, &g->m, &g->v, &g->grad})
    if (s == RX_OK) s = c->cuda(b->alloc(pb), "allocate guide parameters");
  if (s == RX_OK) s = c->cuda(g->img.alloc(rx::guide::kImgBytes), "allocate guide image");
  if (s == RX_OK) s = c->cuda(g->scratch.alloc(64), "allocate guide scratch");
  if (s == RX_OK) s = c->cuda(g->status.alloc(16), "allocate guide status");
  if (s == RX_OK) s = c->cuda(g->step.alloc(16), "allocate guide step count");
  if (s == RX_OK) s = c->cuda(g->dnet.alloc(sizeof(rx::guide::NetDev)), "allocate guide view");
  if (s == RX_OK) s = c->cuda(g->dseg.alloc(sizeof(rx::guide::RecSeg)), "allocate guide records view");
  if (s != RX_OK) {
    delete g;
    return s;
  }
  // He-uniform hidden layers; the output layer scaled by 0.1 (near-uniform start); the
  // unused output rows 40..63 are zero.
  std::vector<float> w(rx::guide::kParams, 0.0f);
  for (int l = 0; l < 5; l++) {
    int K = rx::guide::layer_k(l);
    float a = std::sqrt(6.0f / (float)K) * (l == 4 ? 0.1f : 1.0f);
    int rows = l == 4 ? rx::guide::kOutUsed : 64;
    for (int r = 0; r < rows; r++)
      for (int k = 0; k < K; k++) {
        size_t i = (size_t)rx::guide::layer_w(l) + (size_t)r * K + k;
        w[i] = a * init_uniform(opt->seed, i);
      }
  }
  cudaMemcpy(g->params.p, w.data(), pb, cudaMemcpyHostToDevice);
  for (DevBuf* b : {&g->m, &g->v, &g->grad}) cudaMemset(b->p, 0, pb);
  cudaMemset(g->img.p, 0, rx::guide::kImgBytes);
  cudaMemset(g->status.p, 0, 16);
  cudaMemset(g->step.p, 0, 16);
  const rx::guide::NetDev view = rx::guide_net(g);
  cudaMemcpy(g->dnet.p, &view, sizeof view, cudaMemcpyHostToDevice);
  rx::k_make_image<<<(rx::guide::kParams + 255) / 256, 256, 0, c->stream>>>(g->params.as<float>(),
                                                                             g->img.as<unsigned char>());
  s = c->cuda(cudaStreamSynchronize(c->stream), "guide init");
  if (s != RX_OK) {
    delete g;
    return s;
  }
  g->ready = true;
  rx::guide_free(c->guide);
  c->guide = g;
  return RX_OK;
}

extern "C" rx_status rx_guide_get_params(rx_context* c, float* params) {
  rx_status s = need_guide(c);
  if (s != RX_OK) return s;
  if (!params) return c->fail(RX_ERR_INVALID, "null buffer");
  DeviceGuard dg(c->device);
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "guide sync")) != RX_OK) return s;
  return c->cuda(cudaMemcpy(params, c->guide->params.p, rx::guide::kParams * sizeof(float), cudaMemcpyDeviceToHost),
                 "read guide parameters");
}

extern "C" rx_status rx_guide_set_params(rx_context* c, const float* params) {
  rx_status s = need_guide(c);
  if (s != RX_OK) return s;
  if (!params) return c->fail(RX_ERR_INVALID, "null buffer");
  DeviceGuard dg(c->device);
  rx::GuideState* g = c->guide;
  const size_t pb = rx::guide::kParams * sizeof(float);
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "guide sync")) != RX_OK) return s;
  cudaMemcpy(g->params.p, params, pb, cudaMemcpyHostToDevice);
  for (DevBuf* b : {&g->m, &g->v, &g->grad}) cudaMemset(b->p, 0, pb);
  cudaMemset(g->step.p, 0, 16);
  rx::k_make_image<<<(rx::guide::kParams + 255) / 256, 256, 0, c->stream>>>(g->params.as<float>(),
                                                                             g->img.as<unsigned char>());
  return c->cuda(cudaStreamSynchronize(c->stream), "set guide parameters");
}

static rx_status guide_status(rx_context* c) {
  int st = 0;
  cudaMemcpy(&st, c->guide->status.p, sizeof st, cudaMemcpyDeviceToHost);
  if (st) {
    cudaMemset(c->guide->status.p, 0, sizeof st);
    return c->fail(RX_ERR_TIMEOUT, "tensor-core work did not complete in the network kernel");
  }
  return RX_OK;
}

extern "C" rx_status rx_guide_eval(rx_context* c, const float* recs, uint32_t n, float* raw40, float* pdf) {
  rx_status s = need_guide(c);
  if (s != RX_OK) return s;
  if (n == 0) return RX_OK;
  if (!recs || (!raw40 && !pdf)) return c->fail(RX_ERR_INVALID, "null buffer");
  DeviceGuard dg(c->device);
  rx::GuideState* g = c->guide;
  DevBuf dr, draw, dp;
  if ((s = c->cuda(dr.alloc((size_t)n * rx::guide::kRec * 4), "alloc")) != RX_OK) return s;
  if ((s = c->cuda(draw.alloc((size_t)n * rx::guide::kOutUsed * 4), "alloc")) != RX_OK) return s;
  if ((s = c->cuda(dp.alloc((size_t)n * 4), "alloc")) != RX_OK) return s;
  cudaMemcpy(dr.p, recs, (size_t)n * rx::guide::kRec * 4, cudaMemcpyHostToDevice);
  rx::set_kernel_smem();
  rx::RecordIO io{dr.as<float>(), draw.as<float>(), dp.as<float>()};
  uint32_t grid = std::min<uint32_t>((n + rx::guide::kGroupRows - 1) / rx::guide::kGroupRows, (uint32_t)g->sms);
  rx::k_guide_infer<rx::RecordIO, false><<<grid, 128 * rx::kInferTiles, rx::kSmInfer, c->stream>>>(
      io, nullptr, n, g->dnet.as<rx::guide::NetDev>(), 1, nullptr, nullptr, nullptr);
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "guide eval")) != RX_OK) return s;
  if ((s = guide_status(c)) != RX_OK) return s;
  if (raw40) cudaMemcpy(raw40, draw.p, (size_t)n * rx::guide::kOutUsed * 4, cudaMemcpyDeviceToHost);
  if (pdf) cudaMemcpy(pdf, dp.p, (size_t)n * 4, cudaMemcpyDeviceToHost);
  return RX_OK;
}

extern "C" rx_status rx_guide_eval_device(rx_context* c, const float* d_recs, uint32_t n, float* d_raw40, float* d_pdf,
                                          void* stream) {
  rx_status s = need_guide(c);
  if (s != RX_OK) return s;
  if (n == 0) return RX_OK;
  if (!d_recs || (!d_raw40 && !d_pdf)) return c->fail(RX_ERR_INVALID, "null buffer");
  if (reinterpret_cast<uintptr_t>(d_recs) % 16) return c->fail(RX_ERR_INVALID, "records must be 16-byte aligned");
  DeviceGuard dg(c->device);
  rx::GuideState* g = c->guide;
  rx::set_kernel_smem();
  rx::RecordIO io{d_recs, d_raw40, d_pdf};
  uint32_t grid = std::min<uint32_t>((n + rx::guide::kGroupRows - 1) / rx::guide::kGroupRows, (uint32_t)g->sms);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  rx::k_guide_infer<rx::RecordIO, false><<<grid, 128 * rx::kInferTiles, rx::kSmInfer, st>>>(
      io, nullptr, n, g->dnet.as<rx::guide::NetDev>(), 1, nullptr, nullptr, nullptr);
  return c->cuda(cudaGetLastError(), "guide eval");
}

extern "C" rx_status rx_guide_gradient(rx_context* c, const float* recs, uint32_t n, float* grad, float* loss) {
  rx_status s = need_guide(c);
  if (s != RX_OK) return s;
  if (!recs || !grad || n == 0) return c->fail(RX_ERR_INVALID, "null buffer or empty batch");
  DeviceGuard dg(c->device);
  rx::GuideState* g = c->guide;
  DevBuf dr;
  if ((s = c->cuda(dr.alloc((size_t)n * rx::guide::kRec * 4), "alloc")) != RX_OK) return s;
  cudaMemcpy(dr.p, recs, (size_t)n * rx::guide::kRec * 4, cudaMemcpyHostToDevice);
  cudaMemsetAsync(g->grad.p, 0, rx::guide::kParams * 4, c->stream);
  cudaError_t e = rx::train_step(g, dr.as<float>(), n, c->stream, false);
  if ((s = c->cuda(e, "guide gradient")) != RX_OK) return s;
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "guide gradient")) != RX_OK) return s;
  if ((s = guide_status(c)) != RX_OK) return s;
  cudaMemcpy(grad, g->grad.p, rx::guide::kParams * 4, cudaMemcpyDeviceToHost);
  cudaMemset(g->grad.p, 0, rx::guide::kParams * 4);
  if (loss) cudaMemcpy(loss, g->scratch.as<float>() + 2, 4, cudaMemcpyDeviceToHost);
  return RX_OK;
}

extern "C" rx_status rx_guide_train_step(rx_context* c, const float* d_recs, uint32_t n, float* loss, void* stream) {
  rx_status s = need_guide(c);
  if (s != RX_OK) return s;
  if (!d_recs || n == 0) return c->fail(RX_ERR_INVALID, "null buffer or empty batch");
  if (reinterpret_cast<uintptr_t>(d_recs) % 16) return c->fail(RX_ERR_INVALID, "records must be 16-byte aligned");
  DeviceGuard dg(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  cudaError_t e = rx::train_step(c->guide, d_recs, n, st, true);
  if ((s = c->cuda(e, "guide train step")) != RX_OK) return s;
  if (loss) {
    if ((s = c->cuda(cudaStreamSynchronize(st), "guide train step")) != RX_OK) return s;
    if ((s = guide_status(c)) != RX_OK) return s;
    cudaMemcpy(loss, c->guide->scratch.as<float>() + 2, 4, cudaMemcpyDeviceToHost);
  }
  return RX_OK;
}
