// device.cuh - device-side core of the GB300 rendering path: FP32 vector
// math, the counter-based sampler, primitive intersection, 4-wide BVH
// traversal, materials, lights and the camera.  Each routine restates the
// reference function cited beside it (paths relative to the reference
// project root) in FP32.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "layout.h"

namespace gprt {

// ----------------------------------------------------------------- float3
__device__ __forceinline__ float3 f3(float a, float b, float c) { return make_float3(a, b, c); }
__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float s) { a = a * s; return a; }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
// core.Vec3.Normalize (pkg/core/vec3.go:97-103): zero stays zero
__device__ __forceinline__ float3 normalize(float3 a) {
  float l = length(a);
  return l == 0.f ? f3(0.f, 0.f, 0.f) : f3(a.x / l, a.y / l, a.z / l);
}
// core.Vec3.Luminance (pkg/core/vec3.go:134-136)
__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__device__ __forceinline__ bool is_zero(float3 c) { return c.x == 0.f && c.y == 0.f && c.z == 0.f; }

constexpr float kPi = 3.14159265358979323846f;
#define kInfF (__int_as_float(0x7f800000))

// ----------------------------------------------------------------- sampler
// Counter-based sampler: every value is a pure function of (job seed, pixel,
// sample index, dimension), so a sample renders identically alone, batched
// with other jobs, or split across chunks.  The hash is the "pcg4d" mix of
// Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 9(3), 2020.
// It replaces the per-tile math/rand stream of pkg/renderer/progressive.go:444.
__device__ __forceinline__ uint4 pcg4d(uint4 v) {
  v.x = v.x * 1664525u + 1013904223u;
  v.y = v.y * 1664525u + 1013904223u;
  v.z = v.z * 1664525u + 1013904223u;
  v.w = v.w * 1664525u + 1013904223u;
  v.x += v.y * v.w;
  v.y += v.z * v.x;
  v.z += v.x * v.y;
  v.w += v.y * v.z;
  v.x ^= v.x >> 16;
  v.y ^= v.y >> 16;
  v.z ^= v.z >> 16;
  v.w ^= v.w >> 16;
  v.x += v.y * v.w;
  v.y += v.z * v.x;
  v.z += v.x * v.y;
  v.w += v.y * v.z;
  return v;
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// 32-bit finalizer of MurmurHash3 (fmix32, Austin Appleby): every input bit
// affects every output bit.
__host__ __device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

// The fourth pcg4d coordinate of a 64-bit job seed.  The seed is a
// coordinate of its own, hashed first: keying it into the pixel (pixel ^
// seed) would give seed s the streams seed 0 gives pixel ^ s, so renders with
// nearby seeds would reuse each other's random numbers on shuffled pixels.
__host__ __device__ __forceinline__ uint32_t seed_word(uint64_t seed) {
  return fmix32((uint32_t)seed ^ fmix32((uint32_t)(seed >> 32) ^ 0x9e3779b9u));
}

// The uniform numbers of one pixel sample, consumed sequentially in the
// reference's draw order (RandomSampler, pkg/core/sampling.go:17-39): draw k
// is word k % 4 of pcg4d(pixel, sample, k / 4, seed_word(seed)).  `pos`
// (draws consumed) is all the state a wavefront path carries between
// kernels.
struct Rng {
  uint32_t k0, k1, k3, pos;
  bool valid;
  uint4 buf;
  __device__ __forceinline__ void init(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t start = 0) {
    k0 = pixel;
    k1 = sample;
    k3 = seed_word(seed);
    pos = start;
    valid = false;
  }
  __device__ __forceinline__ float next() {
    uint32_t lane = pos & 3u;
    if (lane == 0 || !valid) {
      buf = pcg4d(make_uint4(k0, k1, pos >> 2, k3));
      valid = true;
    }
    uint32_t r = lane == 0 ? buf.x : lane == 1 ? buf.y : lane == 2 ? buf.z : buf.w;
    pos++;
    return u01(r);
  }
  __device__ __forceinline__ float2 next2() {
    float a = next();
    float b = next();
    return make_float2(a, b);
  }
};

// ----------------------------------------------------------------- warps
// SampleCosineHemisphere (pkg/core/sampling.go:42-67)
__device__ __forceinline__ float3 sample_cosine_hemisphere(float3 n, float2 s) {
  float sa, ca;
  sincosf(2.0f * kPi * s.x, &sa, &ca);
  float r = sqrtf(s.y);
  float x = r * ca, y = r * sa, z = sqrtf(1.0f - s.y);
  float3 nt = fabsf(n.x) > 0.1f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
  float3 t = normalize(cross(nt, n));
  float3 b = cross(n, t);
  return t * x + b * y + n * z;
}
// SampleCone (sampling.go:70-94): uniform direction within the cone of
// cosine cos_total about the unit direction w
__device__ __forceinline__ float3 sample_cone(float3 w, float cos_total, float2 s) {
  float3 u = fabsf(w.x) > 0.1f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
  u = normalize(cross(u, w));
  float3 v = cross(w, u);
  float ct = 1.0f - s.x * (1.0f - cos_total);
  float st = sqrtf(fmaxf(0.f, 1.0f - ct * ct));
  float sp, cp;
  sincosf(2.0f * kPi * s.y, &sp, &cp);
  return u * (st * cp) + v * (st * sp) + w * ct;
}
// SampleOnUnitSphere (sampling.go:97-104)
__device__ __forceinline__ float3 sample_on_unit_sphere(float2 s) {
  float z = 1.0f - 2.0f * s.x;
  float r = sqrtf(fmaxf(0.f, 1.0f - z * z));
  float sp, cp;
  sincosf(2.0f * kPi * s.y, &sp, &cp);
  return f3(r * cp, r * sp, z);
}
// SamplePointInUnitDisk, concentric (sampling.go:108-126)
__device__ __forceinline__ float2 sample_unit_disk(float2 s) {
  float ux = 2.f * s.x - 1.f, uy = 2.f * s.y - 1.f;
  if (ux == 0.f && uy == 0.f) return make_float2(0.f, 0.f);
  float theta, r;
  if (fabsf(ux) > fabsf(uy)) {
    r = ux;
    theta = kPi / 4.f * (uy / ux);
  } else {
    r = uy;
    theta = kPi / 2.f - kPi / 4.f * (ux / uy);
  }
  float st, ct;
  sincosf(theta, &st, &ct);
  return make_float2(r * ct, r * st);
}
// SamplePointInUnitSphere (sampling.go:130-147); pow(x, 1/3) == cbrt(x)
__device__ __forceinline__ float3 sample_in_unit_sphere(float3 s) {
  float r = cbrtf(s.x);
  float sp, cp;
  sincosf(2.f * kPi * s.y, &sp, &cp);
  float ct = 2.f * s.z - 1.f;
  float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
  return f3(r * st * cp, r * st * sp, r * ct);
}

// ----------------------------------------------------------------- hit record
struct Hit {
  float t;
  uint32_t prim;  // global primitive id or kNoHit
  float u, v;
};

// The primitive tests below spell out every rounding (explicit fma / mul /
// add / div intrinsics): kernels that inline them in different contexts -- the
// traversal variants, the single-job and the batched wavefronts -- then
// return bit-identical hits.
__device__ __forceinline__ float dot_rn(float3 a, float3 b) {
  return __fmaf_rn(a.x, b.x, __fmaf_rn(a.y, b.y, __fmul_rn(a.z, b.z)));
}
__device__ __forceinline__ float3 cross_rn(float3 a, float3 b) {
  return make_float3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
                     __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float3 sub_rn(float3 a, float3 b) {
  return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}

// ----------------------------------------------------------------- primitives
// Triangle.Hit, Moller-Trumbore, epsilon 1e-8 (pkg/geometry/triangle.go:107-175)
// Triangles are stored as (v0, e1 = v1 - v0, e2 = v2 - v0).
__device__ __forceinline__ bool hit_triangle(float3 o, float3 d, float4 a, float4 b, float4 c, float tmin,
                                             float tmax, float& t, float& uu, float& vv) {
  float3 v0 = f3(a), e1 = f3(b), e2 = f3(c);
  float3 h = cross_rn(d, e2);
  float det = dot_rn(e1, h);
  if (det > -1e-8f && det < 1e-8f) return false;
  float f = __frcp_rn(det);
  float3 s = sub_rn(o, v0);
  float u = __fmul_rn(f, dot_rn(s, h));
  if (u < 0.f || u > 1.f) return false;
  float3 q = cross_rn(s, e1);
  float v = __fmul_rn(f, dot_rn(d, q));
  if (v < 0.f || __fadd_rn(u, v) > 1.f) return false;
  float tt = __fmul_rn(f, dot_rn(e2, q));
  if (tt < tmin || tt > tmax) return false;
  t = tt;
  uu = u;
  vv = v;
  return true;
}

// Quad.Hit (pkg/geometry/quad.go:133-180).  Stored as 5 float4:
// (corner, D) (u, mat) (v, id) (normal, -) (W, -).
__device__ __forceinline__ bool hit_quad(float3 o, float3 d, const float4* q, float tmin, float tmax, float& t,
                                         float& alpha, float& beta) {
  float4 c = q[0];
  float3 n = f3(q[3]);
  float den = dot_rn(d, n);
  if (fabsf(den) < 1e-8f) return false;
  float tt = __fdiv_rn(__fsub_rn(c.w, dot_rn(o, n)), den);
  if (tt < tmin || tt > tmax) return false;
  float3 p = make_float3(__fmaf_rn(d.x, tt, o.x), __fmaf_rn(d.y, tt, o.y), __fmaf_rn(d.z, tt, o.z));
  float3 hv = sub_rn(p, f3(c));
  float3 U = f3(q[1]), V = f3(q[2]), W = f3(q[4]);
  float a = dot_rn(W, cross_rn(hv, V));
  float b = dot_rn(W, cross_rn(U, hv));
  if (a < 0.f || a > 1.f || b < 0.f || b > 1.f) return false;
  t = tt;
  alpha = a;
  beta = b;
  return true;
}

// Sphere.Hit (pkg/geometry/sphere.go:27-81): nearer root first, then the
// farther.  The discriminant uses the formulation of Haines, Guenther &
// Akenine-Moller, "Precision Improvements for Ray/Sphere Intersection"
// (Ray Tracing Gems, 2019, ch. 7) to keep FP32 usable for radius-1000
// spheres; the roots are the same quantities as (-halfB -/+ sqrt(D)) / a.
__device__ __forceinline__ bool hit_sphere(float3 o, float3 d, float4 s, float tmin, float tmax, float& t) {
  float3 f = sub_rn(o, f3(s));
  float a = dot_rn(d, d);
  float halfB = dot_rn(f, d);
  float k = __fdiv_rn(halfB, a);
  float3 l = make_float3(__fmaf_rn(-d.x, k, f.x), __fmaf_rn(-d.y, k, f.y), __fmaf_rn(-d.z, k, f.z));
  float r2 = __fmul_rn(s.w, s.w);
  float disc = __fmul_rn(a, __fsub_rn(r2, dot_rn(l, l)));
  if (disc < 0.f) return false;
  float sq = __fsqrt_rn(disc);
  float qq = __fsub_rn(-halfB, copysignf(sq, halfB));
  float c = __fsub_rn(dot_rn(f, f), r2);
  float t0, t1;
  if (qq == 0.f) {
    t0 = t1 = __fdiv_rn(-halfB, a);
  } else {
    float ra = __fdiv_rn(c, qq), rb = __fdiv_rn(qq, a);
    t0 = fminf(ra, rb);
    t1 = fmaxf(ra, rb);
  }
  float root = t0;
  if (root < tmin || root > tmax) {
    root = t1;
    if (root < tmin || root > tmax) return false;
  }
  t = root;
  return true;
}

// Disc (disc.go:49-92) and the circular caps of cylinders and cones
// (cylinder.go:224-266, cone.go:306-350): plane hit, |n.d| < eps rejected,
// inside when |p - c|^2 <= r^2.
__device__ __forceinline__ bool hit_cap_plane(float3 o, float3 d, float3 c, float3 n, float r, float eps, float tmin,
                                              float tmax, float& t) {
  float den = dot_rn(d, n);
  if (fabsf(den) < eps) return false;
  float tt = __fdiv_rn(dot_rn(sub_rn(c, o), n), den);
  if (tt < tmin || tt > tmax) return false;
  float3 p = make_float3(__fmaf_rn(d.x, tt, o.x), __fmaf_rn(d.y, tt, o.y), __fmaf_rn(d.z, tt, o.z));
  float3 cp = sub_rn(p, c);
  if (dot_rn(cp, cp) > __fmul_rn(r, r)) return false;
  t = tt;
  return true;
}

__device__ __forceinline__ float axial_height(float3 o, float3 d, float t, float3 base, float3 axis) {
  float3 p = make_float3(__fmaf_rn(d.x, t, o.x), __fmaf_rn(d.y, t, o.y), __fmaf_rn(d.z, t, o.z));
  return dot_rn(sub_rn(p, base), axis);
}

// Cylinder, cone and disc (cylinder.go:97-221, cone.go:128-303, disc.go:49).
// The quadratics are solved in the plane normal to the axis (cylinder) or
// with the half-b form and q = -(b' + sign(b') sqrt(D)) (cone), which keep
// FP32 roots accurate when the ray starts far away; the candidate order and
// the height / nappe checks are the reference's.  `part` tells the surface
// code which piece was hit: 0 body (or disc), 1 base cap, 2 top cap.
__device__ __forceinline__ bool hit_quadric(float3 o, float3 d, const float4* Q, float tmin, float tmax, float& t,
                                            float& part) {
  float4 g0 = __ldg(Q), g1 = __ldg(Q + 1), g4 = __ldg(Q + 4);
  int kind = __float_as_int(g4.x);
  float3 p0 = f3(g0), axis = f3(g1);
  if (kind == kQuadricDisc) {
    if (!hit_cap_plane(o, d, p0, axis, g0.w, 1e-6f, tmin, tmax, t)) return false;
    part = 0.f;
    return true;
  }
  float4 g2 = __ldg(Q + 2);
  float height = g1.w, best = tmax;
  bool any = false;
  if (kind == kQuadricCylinder) {
    float3 delta = sub_rn(o, p0);
    float DV = dot_rn(d, axis), dV = dot_rn(delta, axis);
    float3 dp = make_float3(__fmaf_rn(-axis.x, DV, d.x), __fmaf_rn(-axis.y, DV, d.y), __fmaf_rn(-axis.z, DV, d.z));
    float3 Dp = make_float3(__fmaf_rn(-axis.x, dV, delta.x), __fmaf_rn(-axis.y, dV, delta.y),
                            __fmaf_rn(-axis.z, dV, delta.z));
    float A = dot_rn(dp, dp);
    if (A >= 1e-8f) {
      float hb = dot_rn(Dp, dp);
      float k = __fdiv_rn(hb, A);
      float3 l = make_float3(__fmaf_rn(-dp.x, k, Dp.x), __fmaf_rn(-dp.y, k, Dp.y), __fmaf_rn(-dp.z, k, Dp.z));
      float r2 = __fmul_rn(g0.w, g0.w);
      float disc = __fmul_rn(A, __fsub_rn(r2, dot_rn(l, l)));
      if (disc >= 0.f) {
        float sq = __fsqrt_rn(disc);
        float q = __fsub_rn(-hb, copysignf(sq, hb));
        float C = __fsub_rn(dot_rn(Dp, Dp), r2);
        float t1, t2;
        if (q == 0.f) {
          t1 = t2 = __fdiv_rn(-hb, A);
        } else {
          float ra = __fdiv_rn(C, q), rb = __fdiv_rn(q, A);
          t1 = fminf(ra, rb);
          t2 = fmaxf(ra, rb);
        }
        float tc = t1;
        bool ok = true;
        if (tc < tmin || tc > best) {
          tc = t2;
          if (tc < tmin || tc > best) ok = false;
        }
        if (ok) {
          float h = axial_height(o, d, tc, p0, axis);
          if (h < 0.f || h > height) {
            ok = false;
            if (tc == t1) {
              tc = t2;
              if (!(tc < tmin || tc > best)) {
                h = axial_height(o, d, tc, p0, axis);
                ok = !(h < 0.f || h > height);
              }
            }
          }
        }
        if (ok) {
          best = tc;
          part = 0.f;
          any = true;
        }
      }
    }
  } else {
    float4 g3 = __ldg(Q + 3);
    float3 apex = f3(g3);
    float kk = __fadd_rn(1.f, g3.w);  // 1 + tan^2
    float3 CO = sub_rn(o, apex);
    float DV = dot_rn(d, axis), COV = dot_rn(CO, axis);
    float A = __fsub_rn(dot_rn(d, d), __fmul_rn(kk, __fmul_rn(DV, DV)));
    if (fabsf(A) >= 1e-8f) {
      float hb = __fsub_rn(dot_rn(d, CO), __fmul_rn(kk, __fmul_rn(DV, COV)));
      float C = __fsub_rn(dot_rn(CO, CO), __fmul_rn(kk, __fmul_rn(COV, COV)));
      float disc = __fmaf_rn(hb, hb, -__fmul_rn(A, C));
      if (disc >= 0.f) {
        float sq = __fsqrt_rn(disc);
        float q = __fsub_rn(-hb, copysignf(sq, hb));
        float ra, rb;
        if (q == 0.f) {
          ra = rb = __fdiv_rn(-hb, A);
        } else {
          ra = __fdiv_rn(C, q);
          rb = __fdiv_rn(q, A);
        }
        // the reference tries (-b - sqrt D) / 2a first: the smaller root when
        // a > 0, the larger when a < 0
        float first = A > 0.f ? fminf(ra, rb) : fmaxf(ra, rb);
        float second = A > 0.f ? fmaxf(ra, rb) : fminf(ra, rb);
        for (int pass = 0; pass < 2 && !any; pass++) {
          float tc = pass == 0 ? first : second;
          if (tc < tmin || tc > best) continue;
          float3 p = make_float3(__fmaf_rn(d.x, tc, o.x), __fmaf_rn(d.y, tc, o.y), __fmaf_rn(d.z, tc, o.z));
          float h = dot_rn(sub_rn(p, p0), axis);
          if (h < -1e-8f || h > height + 1e-8f) continue;
          if (dot_rn(sub_rn(p, apex), axis) > 1e-8f) continue;
          best = tc;
          part = 0.f;
          any = true;
        }
      }
    }
  }
  if (g4.z != 0.f) {  // caps: base (-axis), top (+axis) when it has a radius
    float tc;
    float3 na = make_float3(-axis.x, -axis.y, -axis.z);
    if (hit_cap_plane(o, d, p0, na, g0.w, 1e-8f, tmin, best, tc)) {
      best = tc;
      part = 1.f;
      any = true;
    }
    if (g2.w > 0.f && hit_cap_plane(o, d, f3(g2), axis, g2.w, 1e-8f, tmin, best, tc)) {
      best = tc;
      part = 2.f;
      any = true;
    }
  }
  if (any) t = best;
  return any;
}

// ----------------------------------------------------------------- BVH traversal
// Replaces geometry.BVH.Hit / hitNode (pkg/geometry/bvh.go:183-239).  The
// tree is this library's own 4-wide SAH BVH (layout.h) instead of the
// reference's binary midpoint BVH; the closest hit is the same, except that
// among candidates at exactly equal t the reference keeps the later one in
// its depth-first order while this traversal keeps the first one it meets.
struct TraceStats {
  uint32_t nodes, boxes, prims;
};

// State of one ray's traversal; `skip` is the primitive the ray leaves from:
// a ray cannot re-enter the plane of the triangle or quad it starts on, and
// for the sphere it starts on hits closer than 2e-4 x radius are rounding
// noise of the FP32 origin.
struct Trav {
  float3 o, d, inv, ood;
  float tmin, best;
  uint32_t skip;
  int node, sp;
  Hit hit;
};

// `root` is the BVH node the ray starts at (-1: nothing to intersect).  A
// root carrying kRootStackCap starts the ray with only kTestStackCap free
// stack entries (the stack is entered near its top, below a -1 sentinel that
// ends the traversal when popped), so that tests can drive the stack-overflow
// path of one job on an ordinary scene.
__device__ __forceinline__ void trav_init(Trav& s, float3 o, float3 d, float tmin, float tmax, uint32_t skip,
                                          int root, int* stack) {
  s.o = o;
  s.d = d;
  s.inv.x = 1.0f / (fabsf(d.x) > 1e-20f ? d.x : copysignf(1e-20f, d.x));
  s.inv.y = 1.0f / (fabsf(d.y) > 1e-20f ? d.y : copysignf(1e-20f, d.y));
  s.inv.z = 1.0f / (fabsf(d.z) > 1e-20f ? d.z : copysignf(1e-20f, d.z));
  s.ood = o * s.inv;
  s.tmin = tmin;
  s.best = tmax;
  s.skip = skip;
  s.node = root;
  s.sp = 0;
  if (root >= 0 && (root & kRootStackCap)) {
    s.node = root & ~kRootStackCap;
    s.sp = kTraceStack - kTestStackCap;
    stack[s.sp - 1] = -1;
  }
  s.hit.prim = kNoHit;
  s.hit.t = -1.f;
  s.hit.u = s.hit.v = 0.f;
}

// Visits node s.node: tests its children near-first, intersects the leaves
// it hits, pushes the farther internal children and moves s.node to the
// nearest one or to the top of the stack (-1 when the ray is finished).
// Returns true when an any-hit query found a hit.  When the farther children
// do not fit on the stack the ray ends at once with the marker hit
// (prim = kOverflowHit): its result is not the closest hit, and the caller
// reports the bound against the ray's job.
template <bool kAnyHit, bool kCount>
__device__ __forceinline__ bool trav_visit(const DevScene& sc, Trav& s, int* stack, TraceStats* st) {
  const float4* N = sc.nodes + (size_t)s.node * 8;
  if (kCount) st->nodes++;
  int nint = 0;
  int ich[4];
  float itn[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    float4 a = __ldg(N + 2 * i);
    int ref = __float_as_int(a.w);
    if (ref == kEmptyChild) break;
    float4 b = __ldg(N + 2 * i + 1);
    int meta = __float_as_int(b.w);
    if (kCount) st->boxes++;
    float x0 = fmaf(s.inv.x < 0.f ? b.x : a.x, s.inv.x, -s.ood.x);
    float x1 = fmaf(s.inv.x < 0.f ? a.x : b.x, s.inv.x, -s.ood.x);
    float y0 = fmaf(s.inv.y < 0.f ? b.y : a.y, s.inv.y, -s.ood.y);
    float y1 = fmaf(s.inv.y < 0.f ? a.y : b.y, s.inv.y, -s.ood.y);
    float z0 = fmaf(s.inv.z < 0.f ? b.z : a.z, s.inv.z, -s.ood.z);
    float z1 = fmaf(s.inv.z < 0.f ? a.z : b.z, s.inv.z, -s.ood.z);
    float tn = fmaxf(fmaxf(x0, y0), fmaxf(z0, s.tmin));
    float tf = fminf(fminf(x1, y1), fminf(z1, s.best));
    if (tn > tf) continue;
    if (meta == 0) {
      int k = nint++;
      while (k > 0 && itn[k - 1] > tn) {
        itn[k] = itn[k - 1];
        ich[k] = ich[k - 1];
        k--;
      }
      itn[k] = tn;
      ich[k] = ref;
      continue;
    }
    int cnt = meta & kLeafCountMask;
    int type = (meta >> kLeafTypeShift) & 3;
    for (int k = 0; k < cnt; k++) {
      int p = ref + k;
      uint32_t gid = (type == kPrimTriangle ? 0u
                      : type == kPrimQuad   ? sc.quad_base
                      : type == kPrimSphere ? sc.sphere_base
                                            : sc.quadric_base) +
                     (uint32_t)p;
      float t, u = 0.f, v = 0.f;
      bool h;
      if (kCount) st->prims++;
      if (type == kPrimTriangle) {
        if (gid == s.skip) continue;
        const float4* T = sc.tris + (size_t)p * 3;
        h = hit_triangle(s.o, s.d, __ldg(T), __ldg(T + 1), __ldg(T + 2), s.tmin, s.best, t, u, v);
      } else if (type == kPrimQuad) {
        if (gid == s.skip) continue;
        const float4* Q = sc.quads + (size_t)p * 5;
        float4 qq[5] = {__ldg(Q), __ldg(Q + 1), __ldg(Q + 2), __ldg(Q + 3), __ldg(Q + 4)};
        h = hit_quad(s.o, s.d, qq, s.tmin, s.best, t, u, v);
      } else if (type == kPrimSphere) {
        float4 S = __ldg(sc.spheres + (size_t)p * 2);
        float lo = gid == s.skip ? fmaxf(s.tmin, 2e-4f * fabsf(S.w)) : s.tmin;
        h = hit_sphere(s.o, s.d, S, lo, s.best, t);
      } else {
        // a ray leaving a quadric may hit it again (the other side of a
        // cylinder); hits closer than 2e-4 x radius are its own surface
        const float4* Q = sc.quadrics + (size_t)p * 5;
        float lo = s.tmin;
        if (gid == s.skip) {
          float4 g0 = __ldg(Q);
          if (__float_as_int(__ldg(Q + 4).x) == kQuadricDisc) continue;  // planar
          lo = fmaxf(s.tmin, 2e-4f * g0.w);
        }
        h = hit_quadric(s.o, s.d, Q, lo, s.best, t, u);
      }
      if (h) {
        s.best = t;
        s.hit.t = t;
        s.hit.u = u;
        s.hit.v = v;
        s.hit.prim = gid;
        if (kAnyHit) {
          s.node = -1;
          return true;
        }
      }
    }
  }
  // internal children still nearer than the (possibly shrunk) best distance
  int keep = 0;
  for (int k = 0; k < nint; k++)
    if (itn[k] <= s.best) {
      itn[keep] = itn[k];
      ich[keep] = ich[k];
      keep++;
    }
  if (keep > 0) {
    if (s.sp + keep - 1 > kTraceStack) {
      s.node = -1;
      s.hit.prim = kOverflowHit;
      return false;
    }
    for (int k = keep - 1; k >= 1; k--) stack[s.sp++] = ich[k];
    s.node = ich[0];
  } else {
    s.node = s.sp > 0 ? stack[--s.sp] : -1;
  }
  return false;
}

// Whole traversal of one ray from BVH node `root`.  A stack overflow returns
// no hit and, when `err` is given, sets kErrStackOverflow there.
template <bool kAnyHit, bool kCount>
__device__ __forceinline__ bool trace_from(const DevScene& sc, int root, float3 o, float3 d, float tmin, float tmax,
                                           uint32_t skip, Hit& hit, int* err, TraceStats* st = nullptr) {
  Trav s;
  int stack[kTraceStack];
  trav_init(s, o, d, tmin, tmax, skip, root, stack);
  while (s.node >= 0) {
    if (trav_visit<kAnyHit, kCount>(sc, s, stack, st)) break;
  }
  if (s.hit.prim == kOverflowHit) {
    if (err) atomicOr(err, kErrStackOverflow);
    s.hit.prim = kNoHit;
    s.hit.t = -1.f;
  }
  hit = s.hit;
  return s.hit.prim != kNoHit;
}

// Whole traversal of one ray of the scene (used inside the BDPT kernel).
template <bool kAnyHit, bool kCount>
__device__ __forceinline__ bool trace(const DevScene& sc, float3 o, float3 d, float tmin, float tmax, uint32_t skip,
                                      Hit& hit, int* err, TraceStats* st = nullptr) {
  return trace_from<kAnyHit, kCount>(sc, sc.root, o, d, tmin, tmax, skip, hit, err, st);
}

// Persistent traversal of a batch of rays: every warp loops until its work
// is exhausted, one node visit per iteration, and lanes whose ray finished
// take new rays once at least 16 lanes are idle (half the warp: fewer,
// larger refills; on the sphere-scene batch extend + shadow ran 665 ms per
// batch at 8, 632 at 16, 640 at 24), so warps stay full instead of waiting
// for their slowest ray.  A warp draws rays from a chunk: with
// `work` != null, chunks of 64 rays come from that counter (zeroed by the
// previous kernel on the same stream); otherwise each warp owns a static
// contiguous range of the batch.  Source provides count(),
// load(i, o, d, tmin, tmax, skip, root) and store(i, hit); store() sees the
// marker hit of a ray that overflowed its stack and reports it.
constexpr uint32_t kFetchChunk = 64;

template <bool kAnyHit, bool kCount, class Source>
__device__ __forceinline__ void trace_persistent(const DevScene& sc, Source& src, uint32_t* work, TraceStats* st,
                                                 uint32_t* traced) {
  const uint32_t n = src.count();
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  uint32_t cur, end;  // the warp's current chunk [cur, end), warp-uniform
  if (work) {
    cur = end = 0;
  } else {
    uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    cur = (uint32_t)(n * w / nw);
    end = (uint32_t)(n * (w + 1) / nw);
  }
  bool more = true;  // the warp may still draw rays
  Trav s;
  int stack[kTraceStack];
  int ray = -1;
  for (;;) {
    bool idle = ray < 0;
    unsigned idle_mask = __ballot_sync(0xffffffffu, idle);
    if (more && idle_mask && (__popc(idle_mask) >= 16 || idle_mask == 0xffffffffu)) {
      if (cur == end && work) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, kFetchChunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        cur = min(base, n);
        end = min(base + kFetchChunk, n);
      }
      if (cur == end) {
        more = false;
      } else {
        uint32_t take = min((uint32_t)__popc(idle_mask), end - cur);
        uint32_t rank = (uint32_t)__popc(idle_mask & lt);
        if (idle && rank < take) {
          float3 o, d;
          float tmin, tmax;
          uint32_t skip;
          int root;
          uint32_t mine = cur + rank;
          src.load(mine, o, d, tmin, tmax, skip, root);
          trav_init(s, o, d, tmin, tmax, skip, root, stack);
          ray = (int)mine;
          if (kCount) (*traced)++;
        }
        cur += take;
      }
    }
    if (__ballot_sync(0xffffffffu, ray >= 0) == 0 && !more) break;
    if (ray >= 0) {
      if (s.node >= 0) trav_visit<kAnyHit, kCount>(sc, s, stack, st);
      if (s.node < 0) {
        src.store((uint32_t)ray, s.hit);
        ray = -1;
      }
    }
  }
}

// Warp-aggregated append: one atomic per warp, lanes get consecutive slots.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
  unsigned mask = __ballot_sync(__activemask(), want);
  if (!want) return 0;
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// Largest k < n with start[k] <= x (start[0] = 0, start ascending).
__device__ __forceinline__ uint32_t find_range(const uint32_t* start, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(start + mid) <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Where a wavefront reports a device bound of one path: the job's error
// word, or, in a multi-job wavefront, the error word of the work item whose
// path range [start[k], start[k+1]) holds the path's origin index, so that
// only that job fails.
struct ErrSink {
  uint32_t* word;           // single job: its error word
  uint32_t* items;          // multi-job: one error word per item (else null)
  const uint32_t* start;    // multi-job: first origin index of each item
  const uint32_t* n_items;  // multi-job: items of the step
  __device__ void report(uint32_t origin, uint32_t bits) const {
    if (items) atomicOr(items + find_range(start, *n_items, origin), bits);
    else atomicOr(word, bits);
  }
};

// ----------------------------------------------------------------- surface data
// Resolves a hit into the SurfaceInteraction of the reference: point,
// front-face shading normal (SetFaceNormal, pkg/material/interfaces.go:58-65)
// and material.
struct Surface {
  float3 p, n;
  bool front;
  int mat;
  float2 uv;  // SurfaceInteraction.UV, set when the scene has textures
};

// UV of a point on a cylinder / cone body (cylinder.go:187-205, cone.go:234-253)
__device__ __forceinline__ float2 axial_uv(float3 axis, float3 radial, float h, float height) {
  float3 ref = fabsf(axis.y) < 0.9f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
  float3 tangent = normalize(cross(axis, ref));
  float3 bitangent = cross(axis, tangent);
  float a = atan2f(dot(radial, bitangent), dot(radial, tangent));
  return make_float2((a + kPi) / (2.f * kPi), h / height);
}
// UV of a point on a cap of outward normal n (cylinder.go:241-255, cone.go:322-339)
__device__ __forceinline__ float2 cap_uv(float3 n, float3 c, float r, float3 p) {
  float3 ref = fabsf(n.y) < 0.9f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
  float3 tangent = normalize(cross(n, ref));
  float3 bitangent = cross(n, tangent);
  float3 l = p - c;
  return make_float2((dot(l, tangent) / r + 1.f) * 0.5f, (dot(l, bitangent) / r + 1.f) * 0.5f);
}

__device__ __forceinline__ void surface_at(const DevScene& sc, float3 o, float3 d, const Hit& h, Surface& s) {
  s.p = o + d * h.t;  // Ray.At (pkg/core/vec3.go:216-218)
  float3 outward;
  uint32_t p = h.prim;
  const bool uv = sc.has_textures;
  if (p < sc.quad_base) {
    const float4* T = sc.tris + (size_t)p * 3;
    float4 a = __ldg(T);
    float4 nn = __ldg(sc.tri_normals + p);
    outward = f3(nn);  // precomputed normalize(e1 x e2) (triangle.go:92-99)
    s.mat = __float_as_int(a.w);
    if (uv) {  // per-vertex UVs interpolated with the barycentrics, else the barycentrics (triangle.go:151-161)
      s.uv = make_float2(h.u, h.v);
      if (sc.tri_uvs) {
        float4 A = __ldg(sc.tri_uvs + 2 * (size_t)p), Bq = __ldg(sc.tri_uvs + 2 * (size_t)p + 1);
        if (Bq.z != 0.f) {
          float w = 1.f - h.u - h.v;
          s.uv = make_float2(A.x * w + A.z * h.u + Bq.x * h.v, A.y * w + A.w * h.u + Bq.y * h.v);
        }
      }
    }
  } else if (p < sc.sphere_base) {
    const float4* Q = sc.quads + (size_t)(p - sc.quad_base) * 5;
    outward = f3(__ldg(Q + 3));
    s.mat = __float_as_int(__ldg(Q + 1).w);
    if (uv) s.uv = make_float2(h.u, h.v);  // (alpha, beta) (quad.go:165-166)
  } else if (p < sc.quadric_base) {
    const float4* S = sc.spheres + (size_t)(p - sc.sphere_base) * 2;
    float4 c = __ldg(S);
    outward = (s.p - f3(c)) * (1.0f / c.w);  // (p - c) / r (sphere.go:62)
    s.mat = __float_as_int(__ldg(S + 1).x);
    if (uv) {  // spherical angles (sphere.go:64-68)
      float theta = acosf(fminf(1.f, fmaxf(-1.f, -outward.y)));
      float phi = atan2f(-outward.z, outward.x) + kPi;
      s.uv = make_float2(phi / (2.f * kPi), theta / kPi);
    }
  } else {
    const float4* Q = sc.quadrics + (size_t)(p - sc.quadric_base) * 5;
    float4 g0 = __ldg(Q), g1 = __ldg(Q + 1), g4 = __ldg(Q + 4);
    float3 axis = f3(g1);
    int kind = __float_as_int(g4.x);
    s.mat = __float_as_int(g4.y);
    if (kind == kQuadricDisc) {
      outward = axis;
      if (uv) {  // disc.go:68-73
        float3 l = s.p - f3(g0);
        s.uv = make_float2((dot(l, f3(__ldg(Q + 2))) / g0.w + 1.f) * 0.5f,
                           (dot(l, f3(__ldg(Q + 3))) / g0.w + 1.f) * 0.5f);
      }
    } else if (h.u == 2.f) {
      outward = axis;  // top cap
      if (uv) {
        float4 g2 = __ldg(Q + 2);
        s.uv = cap_uv(axis, f3(g2), g2.w, s.p);
      }
    } else if (h.u == 1.f) {
      outward = -axis;  // base cap
      if (uv) s.uv = cap_uv(-axis, f3(g0), g0.w, s.p);
    } else {
      // body: radial from the axis (cylinder.go:188-191), tilted by the
      // cone's slope (cone.go:240-248)
      float3 base = f3(g0);
      float hh = dot(s.p - base, axis);
      float3 radial = s.p - (base + axis * hh);
      if (uv) s.uv = axial_uv(axis, radial, hh, g1.w);
      if (kind == kQuadricCone) radial = radial + axis * ((g0.w - __ldg(Q + 2).w) / g1.w);
      outward = normalize(radial);
    }
  }
  s.front = dot(d, outward) < 0.f;
  s.n = s.front ? outward : -outward;
}

// ----------------------------------------------------------------- materials
__device__ __forceinline__ DevMaterial load_material(const DevScene& sc, int m) { return sc.materials[m]; }

// ImageTexture.Evaluate (image_texture.go:25-52): u, v wrapped into [0,1)
// (Go's int() truncates toward zero), nearest texel, v = 0 at the last row
__device__ __forceinline__ float3 tex_eval(const DevScene& sc, int t, float2 uv) {
  uint4 ti = __ldg(sc.tex_info + t);
  float u = uv.x - truncf(uv.x), v = uv.y - truncf(uv.y);
  if (u < 0.f) u += 1.f;
  if (v < 0.f) v += 1.f;
  int x = (int)(u * (float)ti.y), y = (int)((1.f - v) * (float)ti.z);
  x = min(max(x, 0), (int)ti.y - 1);
  y = min(max(y, 0), (int)ti.z - 1);
  return f3(__ldg(sc.texels + ti.x + (size_t)y * ti.y + (uint32_t)x));
}
// ColorSource.Evaluate of a Lambertian / Metal albedo (color_source.go)
__device__ __forceinline__ float3 albedo_at(const DevScene& sc, const DevMaterial& m, const Surface& s) {
  return m.tex >= 0 ? tex_eval(sc, m.tex, s.uv) : m.albedo;
}

__device__ __forceinline__ float3 reflect(float3 v, float3 n) { return v - n * (2.f * dot(v, n)); }
// refractVector (pkg/material/dielectric.go:158-163)
__device__ __forceinline__ float3 refract(float3 uv, float3 n, float eta) {
  float ct = fminf(-dot(uv, n), 1.0f);
  float3 perp = (uv + n * ct) * eta;
  float3 par = n * (-sqrtf(fabsf(1.0f - dot(perp, perp))));
  return perp + par;
}
// Reflectance, Schlick (dielectric.go:166-172); pow(x,5) as a product
__device__ __forceinline__ float schlick(float c, float ratio) {
  float r0 = (1.f - ratio) / (1.f + ratio);
  r0 = r0 * r0;
  float x = 1.f - c;
  float x2 = x * x;
  return r0 + (1.f - r0) * (x2 * x2 * x);
}

struct Scatter {
  float3 dir;  // scattered direction (not normalised for metal, like the reference)
  float3 att;
  float pdf;   // <= 0: specular (ScatterResult.IsSpecular, interfaces.go:42-45)
};

// Material.Scatter for Lambertian / Metal / Dielectric / Emissive / Layered
// (lambertian.go:25-49, metal.go:38-62, dielectric.go:20-59,
// emissive.go:17-21, layered.go:24-79).  Returns didScatter.
__device__ __forceinline__ bool scatter_basic(const DevScene& sc, const DevMaterial& m, float3 din, const Surface& s,
                                              Rng& rng, Scatter& out) {
  switch (m.kind) {
    case kMatLambertian: {
      float2 u = rng.next2();
      float3 dir = sample_cosine_hemisphere(s.n, u);
      float c = fmaxf(0.f, dot(normalize(dir), s.n));
      out.dir = dir;
      out.att = albedo_at(sc, m, s) * (1.0f / kPi);
      out.pdf = c / kPi;
      return true;
    }
    case kMatMetal: {
      float3 r = reflect(normalize(din), s.n);
      if (m.fuzz > 0.f) {
        float a = rng.next(), b = rng.next(), c = rng.next();
        r = r + sample_in_unit_sphere(f3(a, b, c)) * m.fuzz;
      }
      out.dir = r;
      out.att = albedo_at(sc, m, s);
      out.pdf = 0.f;
      return dot(r, s.n) > 0.f;
    }
    case kMatDielectric: {
      float ratio = s.front ? 1.0f / m.ior : m.ior;
      float3 ud = normalize(din);
      float ct = fminf(-dot(ud, s.n), 1.0f);
      float st = sqrtf(1.0f - ct * ct);
      bool cannot = ratio * st > 1.0f;
      // no sample is drawn under total internal reflection (Go's || short-circuit)
      if (cannot || schlick(ct, ratio) > rng.next())
        out.dir = reflect(ud, s.n);
      else
        out.dir = refract(ud, s.n, ratio);
      out.att = f3(1.f, 1.f, 1.f);
      out.pdf = 0.f;
      return true;
    }
    default:
      return false;  // Emissive absorbs
  }
}

__device__ __forceinline__ bool scatter(const DevScene& sc, const DevMaterial& m, float3 din, const Surface& s,
                                        Rng& rng, Scatter& out) {
  if (m.kind == kMatMix)  // Mix.Scatter (mix.go:30-37): material 2 below the ratio
    return scatter_basic(sc, load_material(sc, rng.next() < m.fuzz ? m.inner : m.outer), din, s, rng, out);
  if (m.kind != kMatLayered) return scatter_basic(sc, m, din, s, rng, out);
  DevMaterial mo = load_material(sc, m.outer);
  Scatter o;
  if (!scatter_basic(sc, mo, din, s, rng, o)) return false;
  float3 sd = normalize(o.dir);
  if (!(dot(sd, s.n) < 0.f)) {
    out = o;
    return true;
  }
  DevMaterial mi = load_material(sc, m.inner);
  Scatter in;
  if (!scatter_basic(sc, mi, sd, s, rng, in)) {
    out = o;
    return true;
  }
  out.dir = in.dir;
  out.att = o.att * in.att;
  out.pdf = in.pdf;
  return true;
}

// EvaluateBRDF (lambertian.go:52-62, metal.go:65-77, dielectric.go:62-142,
// emissive.go:35-38, layered.go:81-95)
__device__ __forceinline__ float3 brdf_basic(const DevScene& sc, const DevMaterial& m, float3 in, float3 out,
                                             const Surface& s, bool radiance) {
  switch (m.kind) {
    case kMatLambertian:
      if (dot(out, s.n) <= 0.f) return f3(0.f, 0.f, 0.f);
      return albedo_at(sc, m, s) * (1.0f / kPi);
    case kMatMetal: {
      float3 r = reflect(-in, s.n);
      if (length(out - r) < 0.001f) return albedo_at(sc, m, s);
      return f3(0.f, 0.f, 0.f);
    }
    case kMatDielectric: {
      float3 wi = normalize(in), wo = normalize(out), n = normalize(s.n);
      float wiN = dot(wi, n), woN = dot(wo, n);
      bool same = (wiN > 0.f) == (woN > 0.f);
      float ratio = s.front ? 1.0f / m.ior : m.ior;
      if (!same) {
        float3 r = reflect(wi, n);
        if (length(wo - r) < 0.001f) {
          float f = schlick(fabsf(wiN), ratio);
          return f3(f, f, f);
        }
      } else {
        float3 rf = refract(wi, n, ratio);
        if (length(wo - rf) < 0.001f) {
          float tr = 1.f - schlick(fabsf(wiN), ratio);
          if (radiance) {
            float etap = s.front ? m.ior : 1.0f / m.ior;
            tr /= etap * etap;
          }
          return f3(tr, tr, tr);
        }
      }
      return f3(0.f, 0.f, 0.f);
    }
    default:
      return f3(0.f, 0.f, 0.f);
  }
}

// isReflectionPath (layered.go:110-119)
__device__ __forceinline__ bool is_reflection_path(float3 in, float3 out, float3 n) {
  float3 inc = -in;
  float3 r = inc - n * (2.f * dot(inc, n));
  return length(out - r) < 0.1f;
}

__device__ __forceinline__ float3 brdf(const DevScene& sc, const DevMaterial& m, float3 in, float3 out,
                                       const Surface& s, bool radiance) {
  if (m.kind == kMatMix)  // Mix.EvaluateBRDF (mix.go:40-46)
    return brdf_basic(sc, load_material(sc, m.outer), in, out, s, radiance) * (1.f - m.fuzz) +
           brdf_basic(sc, load_material(sc, m.inner), in, out, s, radiance) * m.fuzz;
  if (m.kind != kMatLayered) return brdf_basic(sc, m, in, out, s, radiance);
  int sub = is_reflection_path(in, out, s.n) ? m.outer : m.inner;
  return brdf_basic(sc, load_material(sc, sub), in, out, s, radiance);
}

// Material.PDF (lambertian.go:65-72, metal.go:80-84, dielectric.go:145-149,
// emissive.go:41-44, layered.go:98-107).  Returns pdf; sets delta.
__device__ __forceinline__ float pdf_basic(const DevMaterial& m, float3 out, float3 n, bool& delta) {
  switch (m.kind) {
    case kMatLambertian: {
      delta = false;
      float c = dot(out, n);
      return c <= 0.f ? 0.f : c / kPi;
    }
    case kMatMetal:
    case kMatDielectric:
      delta = true;
      return 0.f;
    default:
      delta = false;
      return 0.f;
  }
}
__device__ __forceinline__ float mat_pdf(const DevScene& sc, const DevMaterial& m, float3 in, float3 out, float3 n,
                                         bool& delta) {
  if (m.kind == kMatMix) {  // Mix.PDF (mix.go:49-59): never delta
    bool d;
    float p1 = pdf_basic(load_material(sc, m.outer), out, n, d);
    float p2 = pdf_basic(load_material(sc, m.inner), out, n, d);
    delta = false;
    return p1 * (1.f - m.fuzz) + p2 * m.fuzz;
  }
  if (m.kind != kMatLayered) return pdf_basic(m, out, n, delta);
  int sub = is_reflection_path(in, out, n) ? m.outer : m.inner;
  bool d;
  float p = pdf_basic(load_material(sc, sub), out, n, d);
  delta = false;
  return p;
}

// Material Emit with a hit record, for a ray of direction d: Emissive
// (emissive.go:24-32) emits from the front face; the disc spot light's
// emitter (disc_spot_light.go:26-48) also needs d against its spot direction
// (cosine at most -0.3, d as given).
__device__ __forceinline__ float3 emitted(const DevMaterial& m, bool front, float3 d) {
  if (!front) return f3(0.f, 0.f, 0.f);
  if (m.kind == kMatEmissive) return m.emission;
  if (m.kind == kMatSpotEmissive && dot(d, m.albedo) <= -0.3f) return m.emission;
  return f3(0.f, 0.f, 0.f);
}

// ----------------------------------------------------------------- lights
struct LightSample {
  float3 point, normal, dir;
  float dist;
  float3 emission;
  float pdf;
};

__device__ __forceinline__ float3 gradient_emission(const DevLight& L, float3 dnorm) {
  float t = 0.5f * (dnorm.y + 1.0f);
  return L.b * (1.0f - t) + L.a * t;
}

// Spot falloff (point_spot_light.go:140-158, disc_spot_light.go:150-168)
__device__ __forceinline__ float spot_falloff(const DevLight& L, float c) {
  if (c < L.cos_total) return 0.f;
  if (c >= L.cos_falloff) return 1.f;
  float x = (c - L.cos_total) / (L.cos_falloff - L.cos_total);
  x = x * x;
  return x * x;
}

// Disc.SampleUniform (disc.go:120-134) on a disc record (centre + radius,
// normal, right, up)
__device__ __forceinline__ float3 disc_point(const float4* Q, float2 u) {
  float4 g0 = __ldg(Q);
  float r = sqrtf(u.x) * g0.w;
  float s_, c_;
  sincosf(2.f * kPi * u.y, &s_, &c_);
  return f3(g0) + f3(__ldg(Q + 2)) * (r * c_) + f3(__ldg(Q + 3)) * (r * s_);
}

// Light.Sample (quad_light.go:36-86, sphere_light.go:29-141,
// uniform_infinite_light.go:66-80, gradient_infinite_light.go:77-91,
// disc_light.go, disc_spot_light.go, point_spot_light.go)
__device__ __forceinline__ LightSample light_sample(const DevScene& sc, const DevLight& L, float3 p, float3 n,
                                                    float2 u) {
  LightSample ls;
  if (L.kind == kLightQuad) {
    const float4* Q = sc.quads + (size_t)L.prim * 5;
    float3 c = f3(__ldg(Q)), U = f3(__ldg(Q + 1)), V = f3(__ldg(Q + 2)), N = f3(__ldg(Q + 3));
    float3 sp = c + U * u.x + V * u.y;
    float3 to = sp - p;
    float dist = length(to);
    float3 dir = to * (1.0f / dist);
    float ct = fabsf(dot(N, -dir));
    ls.point = sp;
    ls.normal = N;
    ls.dir = dir;
    ls.dist = dist;
    if (ct < 1e-8f) {
      ls.emission = f3(0.f, 0.f, 0.f);
      ls.pdf = 0.f;
      return ls;
    }
    ls.pdf = (1.0f / L.area) * dist * dist / ct;
    ls.emission = dot(dir, N) < 0.f ? L.a : f3(0.f, 0.f, 0.f);
    return ls;
  }
  if (L.kind == kLightSphere) {
    float4 S = make_float4(L.pos.x, L.pos.y, L.pos.z, L.radius);
    float3 c = f3(S);
    float r = S.w;
    float3 tc = c - p;
    float dc = length(tc);
    bool uniform = dc <= r;
    if (!uniform) {
      // sampleVisible (sphere_light.go:81-141)
      float3 w = normalize(tc);
      float3 uu = fabsf(w.x) > 0.1f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
      uu = normalize(cross(uu, w));
      float3 vv = cross(w, uu);
      float sinMax = r / dc;
      float cosMax = sqrtf(fmaxf(0.f, 1.f - sinMax * sinMax));
      float ct = 1.f - u.x * (1.f - cosMax);
      float st = sqrtf(fmaxf(0.f, 1.f - ct * ct));
      float sp2, cp2;
      sincosf(2.f * kPi * u.y, &sp2, &cp2);
      float3 dir = uu * (st * cp2) + vv * (st * sp2) + w * ct;
      float t;
      if (hit_sphere(p, dir, S, 0.001f, kInfF, t)) {
        float3 hp = p + dir * t;
        float3 on = (hp - c) * (1.0f / r);
        ls.point = hp;
        ls.normal = dot(dir, on) < 0.f ? on : -on;
        ls.dir = dir;
        ls.dist = t;
        ls.emission = L.a;
        ls.pdf = 1.0f / (2.f * kPi * (1.f - cosMax));
        return ls;
      }
      uniform = true;  // the reference falls back to uniform sampling
    }
    // sampleUniform (sphere_light.go:44-78)
    float z = 1.f - 2.f * u.x;
    float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp3, cp3;
    sincosf(2.f * kPi * u.y, &sp3, &cp3);
    float3 ld = f3(rr * cp3, rr * sp3, z);
    float3 sp = c + ld * r;
    float3 dd = sp - p;
    ls.point = sp;
    ls.normal = ld;
    ls.dir = normalize(dd);
    ls.dist = length(dd);
    ls.emission = L.a;
    ls.pdf = 1.0f / (4.f * kPi * r * r);
    return ls;
  }
  if (L.kind == kLightDisc || L.kind == kLightDiscSpot) {
    // DiscLight.Sample (disc_light.go:28-75); the spot variant scales the
    // emission by the falloff seen from the sampled point (disc_spot_light.go:115-130)
    const float4* Q = sc.quadrics + (size_t)L.prim * 5;
    float3 N = f3(__ldg(Q + 1));
    float3 sp = disc_point(Q, u);
    float3 to = sp - p;
    float dist = length(to);
    ls.point = sp;
    ls.normal = N;
    if (dist == 0.f) {
      ls.dir = f3(0.f, 1.f, 0.f);
      ls.dist = 0.f;
      ls.emission = f3(0.f, 0.f, 0.f);
      ls.pdf = 1.f;
      return ls;
    }
    float3 dir = to * (1.0f / dist);
    float ct = fabsf(dot(N, -dir));
    ls.pdf = ct < 1e-6f ? 0.f : (1.0f / L.area) * dist * dist / ct;
    ls.dir = dir;
    ls.dist = dist;
    ls.emission = L.a;  // Emit(ray, nil) of the emissive material
    if (L.kind == kLightDiscSpot) {
      if (dot(dir, L.b) > -0.3f) ls.emission = f3(0.f, 0.f, 0.f);
      ls.emission = ls.emission * spot_falloff(L, dot(L.b, normalize(p - sp)));
    }
    return ls;
  }
  if (L.kind == kLightPointSpot) {
    // PointSpotLight.Sample (point_spot_light.go:46-97)
    float3 to = L.pos - p;
    float dist = length(to);
    ls.point = L.pos;
    ls.pdf = 1.f;
    if (dist == 0.f) {
      ls.normal = ls.dir = f3(0.f, 1.f, 0.f);
      ls.dist = 0.f;
      ls.emission = f3(0.f, 0.f, 0.f);
      return ls;
    }
    float3 tl = to * (1.0f / dist);
    ls.emission = L.a * (spot_falloff(L, dot(L.b, -tl)) / (dist * dist));
    ls.normal = -tl;
    ls.dir = tl;
    ls.dist = dist;
    return ls;
  }
  // infinite lights: cosine-weighted hemisphere about the shading normal
  float3 dir = sample_cosine_hemisphere(n, u);
  ls.point = p + dir * 1e10f;
  ls.normal = -dir;
  ls.dir = dir;
  ls.dist = kInfF;
  ls.emission = L.kind == kLightUniformInfinite ? L.a : gradient_emission(L, dir);
  ls.pdf = dot(dir, n) / kPi;
  return ls;
}

// Light.PDF (quad_light.go:90-109, sphere_light.go:144-166,
// uniform_infinite_light.go:83-91, gradient_infinite_light.go:94-102,
// disc_light.go:78-100 (also the disc spot light), point_spot_light.go:101-118)
__device__ __forceinline__ float light_pdf(const DevScene& sc, const DevLight& L, float3 p, float3 n, float3 dir) {
  if (L.kind == kLightQuad) {
    const float4* Q = sc.quads + (size_t)L.prim * 5;
    float4 qq[5] = {__ldg(Q), __ldg(Q + 1), __ldg(Q + 2), __ldg(Q + 3), __ldg(Q + 4)};
    float t, a, b;
    if (!hit_quad(p, dir, qq, 0.001f, kInfF, t, a, b)) return 0.f;
    float ct = fabsf(dot(f3(qq[3]), -dir));
    if (ct < 1e-8f) return 0.f;
    return (1.0f / L.area) * t * t / ct;
  }
  if (L.kind == kLightSphere) {
    float4 S = make_float4(L.pos.x, L.pos.y, L.pos.z, L.radius);
    float t;
    if (!hit_sphere(p, dir, S, 0.001f, kInfF, t)) return 0.f;
    float dc = length(f3(S) - p);
    if (dc <= S.w) return 1.0f / (4.f * kPi * S.w * S.w);
    float sinMax = S.w / dc;
    float cosMax = sqrtf(fmaxf(0.f, 1.f - sinMax * sinMax));
    return 1.0f / (2.f * kPi * (1.f - cosMax));
  }
  if (L.kind == kLightDisc || L.kind == kLightDiscSpot) {  // disc_light.go:78-100
    const float4* Q = sc.quadrics + (size_t)L.prim * 5;
    float t, part;
    if (!hit_quadric(p, dir, Q, 0.001f, kInfF, t, part)) return 0.f;
    float ct = fabsf(dot(f3(__ldg(Q + 1)), -dir));
    if (ct < 1e-6f) return 0.f;
    return (1.0f / L.area) * t * t / ct;
  }
  if (L.kind == kLightPointSpot) {  // point_spot_light.go:101-118
    float3 to = L.pos - p;
    float len = length(to);
    if (len == 0.f) return 0.f;
    return dot(dir, to * (1.0f / len)) > 0.999f ? 1.f : 0.f;
  }
  float c = dot(dir, n);
  return c <= 0.f ? 0.f : c / kPi;
}

// CalculateLightPDF (pkg/lights/light_sampling.go:11-26): sum over ALL lights
__device__ __forceinline__ float total_light_pdf(const DevScene& sc, float3 p, float3 n, float3 dir) {
  float total = 0.f;
  for (int i = 0; i < sc.n_lights; i++) {
    DevLight L = sc.lights[i];
    total += light_pdf(sc, L, p, n, dir) * L.prob;
  }
  return total;
}

// WeightedLightSampler.SampleLight (weighted_light_sampler.go:82-100)
__device__ __forceinline__ int pick_light(const DevScene& sc, float u) {
  float cum = 0.f;
  for (int i = 0; i < sc.n_lights; i++) {
    cum += sc.lights[i].prob;
    if (u <= cum) return i;
  }
  return sc.n_lights - 1;
}

// Sum of Light.Emit over the infinite lights for a missed ray
// (path_tracing.go:51-59, bdpt.go:214-229)
__device__ __forceinline__ float3 background(const DevScene& sc, float3 d) {
  float3 e = f3(0.f, 0.f, 0.f);
  if (!sc.has_infinite) return e;
  float3 dn = normalize(d);
  for (int i = 0; i < sc.n_lights; i++) {
    DevLight L = sc.lights[i];
    if (L.kind == kLightUniformInfinite) e += L.a;
    else if (L.kind == kLightGradientInfinite) e += gradient_emission(L, dn);
  }
  return e;
}

// powerHeuristic (path_tracing.go:225-235)
__device__ __forceinline__ float power_heuristic(float f, float g) {
  if (f == 0.f) return 0.f;
  return (f * f) / (f * f + g * g);
}

// ----------------------------------------------------------------- camera
// Camera.GetRay (pkg/geometry/camera.go:173-190)
__device__ __forceinline__ void camera_ray(const DevCamera& c, int i, int j, float2 lens, float2 jit, float3& o,
                                           float3& d) {
  float3 ps = c.pixel00 + c.du * ((float)i + (jit.x - 0.5f)) + c.dv * ((float)j + (jit.y - 0.5f));
  o = c.center;
  if (c.has_lens) {
    float2 p = sample_unit_disk(lens);
    o = c.center + c.disk_u * p.x + c.disk_v * p.y;
  }
  d = normalize(ps - o);
}

}  // namespace gprt
