// kernels_bdpt.cu - bidirectional path tracing.
//
// Restates BDPTIntegrator.RayColor (pkg/integrator/bdpt.go:73-102): a camera
// subpath and a light subpath are generated (generateCameraPath :106-135,
// generateLightPath :139-202, extendPath :206-291), every (s,t) strategy is
// evaluated (:294-561) and weighted by calculateMISWeight
// (pkg/integrator/bdpt_mis.go:13-335).  t=1 light-tracing contributions are
// splatted into the film's splat buffer with atomic adds and applied after
// the pass (processSplats, pkg/renderer/progressive.go:371-391).
//
// Every helper is inlined: an out-of-line call takes its vertex and scene
// arguments by reference, which puts them in each thread's local stack
// (3 KB per thread for the strategy kernel, 245 MB at full occupancy, more
// than L2), and that stack traffic went to DRAM.
//
// Per chunk of samples:
//   k_bdpt_camgen      the camera vertex and ray of every sample;
//   k_bdpt_trace       (per bounce) closest hits of the subpath queue;
//   k_bdpt_extend      (per bounce) each subpath's next vertex into a global
//                      vertex store (fields indexed [vertex][sample]) and the
//                      continuing subpaths compacted into the other queue; a
//                      camera subpath that ends starts its light subpath;
//   k_bdpt_list        lists, per strategy (s,t) and window of 16,384
//                      samples, the samples that have it;
//   k_bdpt_prefix      each strategy class's prefix sums of the list counts
//                      in (window, strategy) order;
//   k_bdpt_strategies  one thread per listed (strategy, sample) item, in
//                      (window, strategy) order, so every strategy of a
//                      window runs while its vertices are in L2; the
//                      items of a strategy in consecutive threads: each warp
//                      runs a single (s,t) for 32 samples that have it, so
//                      control flow is uniform and neighbouring warps share
//                      code; its sampler position is the sample's position
//                      after the subpaths plus the draws of the strategies
//                      before it (draws_before);
//   k_bdpt_sum         adds each sample's strategy contributions in the
//                      reference's s-major order.
#include <algorithm>

#include "device.cuh"
#include "kernels.h"

namespace gprt {

namespace {


constexpr int kFlagLight = 1, kFlagCamera = 2, kFlagSpecular = 4, kFlagInfinite = 8, kFlagFront = 16;

struct BVert {  // bdpt.go:14-36
  float3 p, n, beta, Le, wi;
  float2 uv;  // surface UV (textured scenes)
  float fwd, rev;
  int mat;    // material index, -1 for none
  int light;  // index in the light table, -1 for none
  uint32_t prim;
  int flags;
  __device__ bool is(int f) const { return (flags & f) != 0; }
};

__device__ __forceinline__ bool light_is_area(const DevScene& sc, int li) {
  int k = sc.lights[li].kind;
  return k == kLightQuad || k == kLightSphere || k == kLightDisc || k == kLightDiscSpot;
}

// Vertex.IsOnSurface (bdpt.go:42-49)
__device__ __forceinline__ bool on_surface(const DevScene& sc, const BVert& v) {
  if (v.is(kFlagLight) && v.light >= 0) return light_is_area(sc, v.light);
  return v.mat >= 0;
}

// convertSolidAngleToAreaPdf (bdpt_mis.go:341-363)
__device__ __forceinline__ float to_area(const DevScene& sc, const BVert& from, const BVert& next, float pdf) {
  if (next.is(kFlagInfinite)) return pdf;
  float3 d = next.p - from.p;
  float d2 = dot(d, d);
  if (d2 == 0.f) return 0.f;
  float inv = 1.0f / d2;
  if (on_surface(sc, next)) pdf *= fabsf(dot(d * sqrtf(inv), next.n));
  return pdf * inv;
}

// ---------------------------------------------------------------- camera
// MapRayToPixel (camera.go:280-316)
__device__ __forceinline__ bool map_ray_to_pixel(const DevCamera& c, float3 o, float3 d, int& px, int& py) {
  float3 ipc = c.center - c.w * c.focus_distance;
  float t = dot(ipc - o, c.w) / dot(d, c.w);
  if (t <= 0.f) return false;
  float3 rel = o + d * t - ipc;
  float nx = (dot(rel, c.u) + c.viewport_width / 2.f) / c.viewport_width;
  float ny = (dot(rel, c.v) + c.viewport_height / 2.f) / c.viewport_height;
  float fx = nx * (float)c.width, fy = ny * (float)c.height;
  if (!(fx > -1.f && fx < (float)c.width + 1.f && fy > -1.f && fy < (float)c.height + 1.f)) return false;
  int x = (int)fx, y = (int)fy;  // Go int() truncates toward zero
  if (x >= 0 && x < c.width && y >= 0 && y < c.height) {
    px = x;
    py = y;
    return true;
  }
  return false;
}
// CalculateRayPDFs direction pdf (camera.go:194-216)
__device__ __forceinline__ float camera_dir_pdf(const DevCamera& c, float3 o, float3 d) {
  float ct = dot(d, c.forward);
  if (ct <= c.cos_total_width) return 0.f;
  int x, y;
  if (!map_ray_to_pixel(c, o, d, x, y)) return 0.f;
  return 1.0f / (c.image_plane_area * ct * ct * ct);
}
// EvaluateRayImportance (camera.go:263-277)
__device__ __forceinline__ float camera_importance(const DevCamera& c, float3 d) {
  float ct = dot(d, c.forward);
  if (ct < c.cos_total_width) return 0.f;
  float c2 = ct * ct;
  return 1.0f / (c.image_plane_area * c.lens_area * c2 * c2);
}

// ---------------------------------------------------------------- lights
// SampleEmission (quad_light.go:113-145, sphere_light.go:169-184,
// disc_light.go:103-110, disc_spot_light.go:210-240, point_spot_light.go:161-191,
// light_sampling.go:58-115 for the infinite lights)
__device__ __forceinline__ void sample_emission(const DevScene& sc, const DevLight& L, float2 sp, float2 sd, float3& p, float3& n,
                                float3& dir, float3& Le, float& area_pdf, float& dir_pdf) {
  if (L.kind == kLightQuad) {
    const float4* Q = sc.quads + (size_t)L.prim * 5;
    float3 c = f3(__ldg(Q)), U = f3(__ldg(Q + 1)), V = f3(__ldg(Q + 2)), N = f3(__ldg(Q + 3));
    p = c + U * sp.x + V * sp.y;
    dir = sample_cosine_hemisphere(N, sd);
    n = N;
    area_pdf = 1.0f / L.area;
    dir_pdf = dot(dir, N) / kPi;
    Le = L.a;
    return;
  }
  if (L.kind == kLightSphere) {
    float4 S = make_float4(L.pos.x, L.pos.y, L.pos.z, L.radius);
    float z = 1.f - 2.f * sp.x;
    float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float s_, c_;
    sincosf(2.f * kPi * sp.y, &s_, &c_);
    float3 ld = f3(r * c_, r * s_, z);
    p = f3(S) + ld * S.w;
    n = ld;
    dir = sample_cosine_hemisphere(n, sd);
    dir_pdf = dot(dir, n) / kPi;
    area_pdf = 1.0f / (4.f * kPi * S.w * S.w);
    Le = L.a;
    return;
  }
  if (L.kind == kLightDisc || L.kind == kLightDiscSpot || L.kind == kLightPointSpot) {
    if (L.kind == kLightPointSpot) {
      p = L.pos;
      area_pdf = 1.f;
    } else {
      const float4* Q = sc.quadrics + (size_t)L.prim * 5;
      p = disc_point(Q, sp);
      n = f3(__ldg(Q + 1));
      area_pdf = 1.0f / L.area;
    }
    if (L.kind == kLightDisc) {  // SampleEmissionDirection (light_sampling.go:58-80)
      dir = sample_cosine_hemisphere(n, sd);
      dir_pdf = dot(dir, n) / kPi;
      Le = L.a;
      return;
    }
    dir = sample_cone(L.b, L.cos_total, sd);
    Le = L.a * spot_falloff(L, dot(dir, L.b));
    dir_pdf = 1.0f / (2.f * kPi * (1.f - L.cos_total));  // UniformConePDF (light_sampling.go:83-85)
    if (L.kind == kLightPointSpot) n = dir;
    return;
  }
  // SampleInfiniteLight (light_sampling.go:89-115)
  float3 d = sample_on_unit_sphere(sd);
  float3 up = fabsf(d.x) > 0.9f ? f3(0.f, 1.f, 0.f) : f3(1.f, 0.f, 0.f);
  float3 right = normalize(cross(d, up));
  up = normalize(cross(right, d));
  float2 ds = sample_unit_disk(sp);
  float R = sc.world_radius;
  float3 dp = sc.world_center + right * (ds.x * R) + up * (ds.y * R);
  p = dp + d * (-R);
  n = -d;
  dir = d;
  area_pdf = 1.0f / (kPi * R * R);
  dir_pdf = 1.0f / (4.f * kPi);
  Le = L.kind == kLightUniformInfinite ? L.a : gradient_emission(L, d);
}

// PDF_Le direction pdf (quad_light.go:148-185, sphere_light.go:187-209,
// disc_light.go:113-136, disc_spot_light.go:243-264, point_spot_light.go:194-214,
// uniform_infinite_light.go:94-106); pos receives the position pdf
__device__ __forceinline__ float pdf_le(const DevScene& sc, const DevLight& L, float3 p, float3 dir, float& pos) {
  pos = 0.f;
  if (L.kind == kLightQuad) {
    const float4* Q = sc.quads + (size_t)L.prim * 5;
    float3 c = f3(__ldg(Q)), U = f3(__ldg(Q + 1)), V = f3(__ldg(Q + 2)), N = f3(__ldg(Q + 3));
    float3 tp = p - c;
    float uu = dot(U, U), vv = dot(V, V), uv = dot(U, V);
    if (uu == 0.f || vv == 0.f) return 0.f;
    float det = uu * vv - uv * uv;
    if (fabsf(det) < 1e-8f) return 0.f;
    float tu = dot(tp, U), tv = dot(tp, V);
    float al = (vv * tu - uv * tv) / det, be = (uu * tv - uv * tu) / det;
    if (al < 0.f || al > 1.f || be < 0.f || be > 1.f) return 0.f;
    float3 rec = c + U * al + V * be;
    if (length(rec - p) > 0.001f * fmaxf(1.f, length(p) * 1e-3f)) return 0.f;
    pos = 1.0f / L.area;
    float ct = dot(dir, N);
    return ct <= 0.f ? 0.f : ct / kPi;
  }
  if (L.kind == kLightSphere) {
    float4 S = make_float4(L.pos.x, L.pos.y, L.pos.z, L.radius);
    float dc = length(p - f3(S));
    if (!(fabsf(dc - S.w) <= 0.001f * fmaxf(1.f, fabsf(S.w) * 1e-3f))) return 0.f;
    float3 n = normalize(p - f3(S));
    if (dot(dir, n) <= 0.f) return 0.f;
    pos = 1.0f / (4.f * kPi * S.w * S.w);
    return dot(dir, n) / kPi;
  }
  if (L.kind == kLightDisc || L.kind == kLightDiscSpot) {
    const float4* Q = sc.quadrics + (size_t)L.prim * 5;
    float4 g0 = __ldg(Q);
    float3 N = f3(__ldg(Q + 1));
    // validatePointOnDisc (disc_light.go:153-165), tolerance 0.001
    float3 tp = p - f3(g0);
    float h = dot(tp, N);
    if (fabsf(h) > 0.001f || length(tp - N * h) > g0.w) return 0.f;
    float ct = dot(dir, N);
    if (ct <= 0.f) return 0.f;
    if (L.kind == kLightDiscSpot && dot(dir, L.b) < L.cos_total) {
      pos = 1.0f / L.area;
      return 0.f;
    }
    pos = 1.0f / L.area;
    return ct / kPi;
  }
  if (L.kind == kLightPointSpot) {
    if (length(p - L.pos) > 0.001f || dot(dir, L.b) < L.cos_total) return 0.f;
    pos = 1.f;
    return 1.0f / (2.f * kPi * (1.f - L.cos_total));
  }
  if (sc.world_radius <= 0.f) return 0.f;
  pos = 1.0f / (kPi * sc.world_radius * sc.world_radius);
  return 1.0f / (4.f * kPi);
}

// calculateInfiniteLightDensity (bdpt_mis.go:313-335)
__device__ float infinite_density(const DevScene& sc, float3 p, float3 n, float3 dir) {
  float t = 0.f;
  for (int i = 0; i < sc.n_lights; i++) {
    DevLight L = sc.lights[i];
    if (L.kind == kLightUniformInfinite || L.kind == kLightGradientInfinite) {
      float c = dot(dir, n);
      t += (c <= 0.f ? 0.f : c / kPi) * L.prob;
    }
  }
  return t;
}

// ---------------------------------------------------------------- BRDF at a vertex
// evaluateBRDF (bdpt.go:564-583)
__device__ __forceinline__ float3 vertex_brdf(const DevScene& sc, const BVert& v, float3 out, bool radiance) {
  if (v.is(kFlagInfinite)) return f3(0.f, 0.f, 0.f);
  if (v.is(kFlagLight) && v.mat < 0) return f3(1.f, 1.f, 1.f);
  if (v.mat < 0) return f3(0.f, 0.f, 0.f);
  Surface s;
  s.p = v.p;
  s.n = v.n;
  s.front = v.is(kFlagFront);
  s.mat = v.mat;
  s.uv = v.uv;
  return brdf(sc, load_material(sc, v.mat), v.wi, out, s, radiance);
}

// calculateLightPdf (bdpt_mis.go:239-272)
__device__ __forceinline__ float vertex_light_pdf(const DevScene& sc, const BVert& cur, const BVert& to) {
  float3 w = to.p - cur.p;
  float inv = 1.0f / dot(w, w);
  w = w * sqrtf(inv);
  float pdf = 0.f;
  if (cur.is(kFlagLight)) {
    if (cur.is(kFlagInfinite)) {
      float r = sc.world_radius == 0.f ? 1.f : sc.world_radius;
      pdf = 1.0f / (kPi * r * r);
    } else if (cur.light >= 0) {
      float pos;
      pdf = pdf_le(sc, sc.lights[cur.light], cur.p, w, pos) * inv;
    }
  }
  if (on_surface(sc, to)) pdf *= fabsf(dot(to.n, w));
  return pdf;
}

// calculateVertexPdf (bdpt_mis.go:186-236)
__device__ __forceinline__ float vertex_pdf(const DevScene& sc, const BVert& cur, const BVert* prev, const BVert& next) {
  if (cur.is(kFlagLight)) return vertex_light_pdf(sc, cur, next);
  float3 wn = next.p - cur.p;
  if (dot(wn, wn) == 0.f) return 0.f;
  wn = normalize(wn);
  float3 wp = f3(0.f, 0.f, 0.f);
  if (prev) {
    wp = prev->p - cur.p;
    if (dot(wp, wp) == 0.f) return 0.f;
    wp = normalize(wp);
  } else if (!cur.is(kFlagCamera)) {
    return 0.f;
  }
  float pdf;
  if (cur.is(kFlagCamera)) {
    pdf = camera_dir_pdf(sc.cam, cur.p, wn);
    if (pdf == 0.f) return 0.f;
  } else if (cur.mat >= 0) {
    bool delta;
    pdf = mat_pdf(sc, load_material(sc, cur.mat), wp, wn, cur.n, delta);
    if (delta) return 0.f;
  } else {
    return 0.f;
  }
  return to_area(sc, cur, next, pdf);
}

// calculateLightOriginPdf (bdpt_mis.go:275-308)
__device__ __forceinline__ float light_origin_pdf(const DevScene& sc, const BVert& lv, const BVert& to) {
  float3 w = to.p - lv.p;
  if (dot(w, w) == 0.f) return 0.f;
  w = normalize(w);
  if (lv.is(kFlagInfinite)) return infinite_density(sc, to.p, to.n, -w);
  if (!lv.is(kFlagLight) || lv.light < 0) return 0.f;
  if (sc.n_lights == 0) return 0.f;
  float pos;
  pdf_le(sc, sc.lights[lv.light], lv.p, w, pos);
  return pos * sc.lights[lv.light].prob;
}

// Any-hit test of a connection / shadow ray (one call site for all strategies).
__device__ __forceinline__ bool occluded(const DevScene& sc, float3 o, float3 d, float tmax, uint32_t skip, int* err) {
  Hit hh;
  return trace<true, false>(sc, o, d, 0.001f, tmax, skip, hh, err);
}

// ---------------------------------------------------------------- vertex store
// Subpath vertices live in global memory as 5 float4 fields indexed
// [vertex * ns + sample], so the 32 lanes of a warp (32 consecutive samples)
// read one field of one vertex in a single coalesced access.  The first two
// fields hold what a pdf request of the MIS weight reads of a vertex
// (position, normal, material, flags, light), so those requests load two
// fields; the forward and reverse pdfs live in the pdf record.
__device__ __forceinline__ void put_vert(const DevBdpt& B, int v, uint32_t i, const BVert& x, float pre = 0.f) {
  size_t k = (size_t)v * B.ns + i;
  B.v[0][k] = make_float4(x.p.x, x.p.y, x.p.z, __int_as_float((x.mat + 1) | (x.flags << 24)));
  B.v[1][k] = make_float4(x.n.x, x.n.y, x.n.z, __int_as_float(x.light));
  B.v[2][k] = make_float4(x.beta.x, x.beta.y, x.beta.z, x.wi.x);
  B.v[3][k] = make_float4(x.Le.x, x.Le.y, x.Le.z, x.wi.y);
  B.v[4][k] = make_float4(x.wi.z, __uint_as_float(x.prim), 0.f, 0.f);
  B.pdf[k] = make_float4(x.fwd, __int_as_float(x.flags | ((x.light + 1) << 8)), x.rev, pre);
  if (B.uv) B.uv[k] = x.mat >= 0 ? x.uv : make_float2(0.f, 0.f);
}

__device__ __forceinline__ BVert get_vert(const DevBdpt& B, int v, uint32_t i) {
  size_t k = (size_t)v * B.ns + i;
  float4 a = B.v[0][k], b = B.v[1][k], c = B.v[2][k], d = B.v[3][k], e = B.v[4][k], q = B.pdf[k];
  BVert x;
  x.p = f3(a);
  int mf = __float_as_int(a.w);
  x.mat = (mf & 0xFFFFFF) - 1;
  x.flags = (mf >> 24) & 0xFF;
  x.n = f3(b);
  x.light = __float_as_int(b.w);
  x.fwd = q.x;
  x.rev = q.z;  // patched after the next bounce
  x.beta = f3(c);
  x.Le = f3(d);
  x.wi = make_float3(c.w, d.w, e.x);
  x.prim = __float_as_uint(e.y);
  x.uv = B.uv ? B.uv[k] : make_float2(0.f, 0.f);
  return x;
}

// The pdfs and flags of a stored vertex and its subpath's MIS prefix (one
// 16-byte record): all the MIS weight reads away from the connection.
struct VPdf {
  float fwd, rev;
  int flags, light;
  float pre;
};
__device__ __forceinline__ VPdf get_vpdf(const DevBdpt& B, int v, uint32_t i) {
  float4 a = B.pdf[(size_t)v * B.ns + i];
  VPdf r;
  r.fwd = a.x;
  r.rev = a.z;
  int m = __float_as_int(a.y);
  r.flags = m & 0xFF;
  r.light = (m >> 8) - 1;
  r.pre = a.w;
  return r;
}
// a vertex on a point light (LightTypePoint, bdpt_mis.go:130-137)
__device__ __forceinline__ bool is_delta_light(const DevScene& sc, const VPdf& v) {
  return (v.flags & kFlagLight) && v.light >= 0 && sc.lights[v.light].kind == kLightPointSpot;
}

__device__ __forceinline__ float remap0(float f) { return f != 0.f ? f : 1.f; }

// The MIS prefix of a finished subpath, written into each vertex's pdf
// record.  calculateMISWeight (bdpt_mis.go:13-181) walks each subpath from
// the connection outwards, multiplying ratios r_i = remap0(rev_i) /
// remap0(fwd_i) and adding the running product at every connectible vertex;
// away from the two vertices next to the connection those ratios and flags
// do not depend on the strategy, so the sum over vertices 0..k is kept as
//   A_k = r_k * (A_{k-1} + c_k)
// (camera subpath: from vertex 1, c_k = neither vertex k nor k-1 specular;
// light subpath: from vertex 0, c_k also excludes delta lights), and each
// strategy evaluates only its two connection-side steps on top of it.
__device__ __forceinline__ void subpath_prefix(const DevScene& sc, const DevBdpt& B, int base, int len, uint32_t i,
                                               bool camera) {
  float acc = 0.f;
  bool prev_ok = true;  // the previous vertex is neither specular nor a delta light
  for (int k = 0; k < len; k++) {
    size_t at = (size_t)(base + k) * B.ns + i;
    float4 a = B.pdf[at];
    int m = __float_as_int(a.y);
    int flags = m & 0xFF, light = (m >> 8) - 1;
    bool ok = !(flags & kFlagSpecular);
    if (!camera) ok = ok && !((flags & kFlagLight) && light >= 0 && sc.lights[light].kind == kLightPointSpot);
    if (camera && k == 0) {
      acc = 0.f;  // the camera vertex takes no part in the walk
    } else {
      bool conn = ok && (k == 0 || prev_ok);
      acc = (remap0(a.z) / remap0(a.x)) * (acc + (conn ? 1.f : 0.f));
    }
    B.pdf[at].w = acc;
    prev_ok = ok;
  }
}

// The vertices of one sample's subpath (camera: base 0, light: base maxv).
struct SubpathRef {
  const DevBdpt* B;
  uint32_t i;
  int base;
  __device__ BVert operator[](int k) const { return get_vert(*B, base + k, i); }
  __device__ VPdf pdfs(int k) const { return get_vpdf(*B, base + k, i); }
};

// ---------------------------------------------------------------- subpath wavefront
// generateCameraPath / generateLightPath / extendPath (bdpt.go:106-291) one
// bounce per launch over a compacted queue of subpaths: a persistent
// closest-hit traversal of the queue, then one thread per slot extends its
// subpath by the vertex hit, compacting the continuing subpaths into the
// other queue.  A sample's light subpath starts, in the same sampler stream,
// in the step that ends its camera subpath, so both kinds share the queue.
// Each vertex is stored when it is created; its reverse pdf (set by the
// scatter at the next vertex, bdpt.go:273-285) and its MIS prefix
// (subpath_prefix) are patched one bounce later with one 8-byte store.

// State bits of a queue slot (BdQueue::st.x): length, bounces, kind, and
// properties of the last two vertices; st.y holds the camera subpath length.
constexpr uint32_t kStCamera = 1u << 16, kStOkBefore = 1u << 17, kStOkLast = 1u << 18, kStSurfLast = 1u << 19,
                   kStInfLast = 1u << 20;

// The subpath vertex is neither specular nor (light subpaths) a delta light:
// it can take part in a connection (bdpt_mis.go:61-178).
__device__ __forceinline__ bool vertex_ok(const DevScene& sc, const BVert& v, bool camera) {
  bool ok = !v.is(kFlagSpecular);
  if (!camera) ok = ok && !(v.is(kFlagLight) && v.light >= 0 && sc.lights[v.light].kind == kLightPointSpot);
  return ok;
}

// convertSolidAngleToAreaPdf (bdpt_mis.go:341-363) towards a vertex known by
// its position, normal and kind.
__device__ __forceinline__ float to_area_at(float3 from, float3 p, float3 n, bool surface, bool infinite, float pdf) {
  if (infinite) return pdf;
  float3 d = p - from;
  float d2 = dot(d, d);
  if (d2 == 0.f) return 0.f;
  float inv = 1.0f / d2;
  if (surface) pdf *= fabsf(dot(d * sqrtf(inv), n));
  return pdf * inv;
}

// The MIS prefix of vertex k of a subpath from the prefix `acc` through
// vertex k - 1 (subpath_prefix's recurrence; the camera vertex has none).
__device__ __forceinline__ float next_prefix(bool camera, int k, float rev, float fwd, bool ok, bool ok_before,
                                             float acc) {
  if (camera && k == 0) return 0.f;
  bool conn = ok && (k == 0 || ok_before);
  return (remap0(rev) / remap0(fwd)) * (acc + (conn ? 1.f : 0.f));
}

// The reverse pdf and MIS prefix of a stored vertex, once final.
__device__ __forceinline__ void patch_vert(const DevBdpt& B, int v, uint32_t i, float rev, float pre) {
  *reinterpret_cast<float2*>(&B.pdf[(size_t)v * B.ns + i].z) = make_float2(rev, pre);
}

// The strategies that draw uniform numbers (draws_before) and the sample's
// record for the strategy kernels, once both subpaths are stored.
template <int MAXV>
__device__ __forceinline__ void finish_sample(const DevScene& sc, const DevBdpt& B, uint32_t p, int nc, int nl,
                                              uint32_t pos, uint32_t pix, uint32_t sample) {
  uint32_t lm = 0, cm = 0;
  for (int s = 2; s <= nl; s++)
    if (!(get_vpdf(B, MAXV + s - 1, p).flags & kFlagSpecular)) lm |= 1u << s;
  if (sc.n_lights > 0)
    for (int t = 2; t <= nc; t++) {
      BVert v = get_vert(B, t - 1, p);
      if (!v.is(kFlagSpecular) && v.mat >= 0) cm |= 1u << t;
    }
  B.meta[p] = make_uint4((uint32_t)nc | ((uint32_t)nl << 8), pos, pix, sample);
  B.masks[p] = make_uint2(lm, cm);
}

// calculateMISWeight (bdpt_mis.go:13-181) over the stored subpaths
// A vertex named by a pdf request: camera subpath vertex k (k >= 0), light
// subpath vertex k (kLightV + k), the strategy's sampled vertex, or none.
constexpr int kNoV = -1, kSampledV = -2, kLightV = 1024;

__device__ __forceinline__ BVert fetch_vert(const SubpathRef& C, const SubpathRef& Lp, const BVert* sampled, int id) {
  if (id == kSampledV) return *sampled;
  return id >= kLightV ? Lp[id - kLightV] : C[id];
}

template <int CLS>
__device__ __forceinline__ float mis_weight(const DevScene& sc, const SubpathRef& C, const SubpathRef& Lp,
                                         const BVert* sampled, int s, int t) {
  if (s + t == 2) return 1.f;
  // The reverse pdfs the walk recomputes next to the connection
  // (bdpt_mis.go:61-105 camera side, :140-178 light side): at most two per
  // side, each calculateVertexPdf(cur, prev, next), or for s = 0 at t-1
  // calculateLightOriginPdf(cur, next).  They are named by vertex ids and
  // evaluated in one loop, so the pdf code is inlined once.
  int rq[4][3];
  int nq = 0;
  int cam1 = -1, cam2 = -1, lit1 = -1, lit2 = -1;  // request of rev at t-1, t-2, s-1, s-2
  const int c1 = t - 1, c2 = t - 2, l1 = kLightV + s - 1, l2 = kLightV + s - 2;
  auto add = [&](int cur, int prev, int next) {
    rq[nq][0] = cur;
    rq[nq][1] = prev;
    rq[nq][2] = next;
    return nq++;
  };
  if (CLS == 0) {
    if (t > 1) cam1 = add(c1, kNoV, c2);  // the light origin pdf
    if (t > 2) cam2 = add(c1, kNoV, c2);
  } else if (CLS == 1) {
    lit1 = add(kSampledV, kNoV, l1);
    lit2 = add(l1, kSampledV, l2);
  } else if (CLS == 2) {
    cam1 = add(kSampledV, kNoV, c1);
    cam2 = add(c1, kSampledV, c2);
    lit1 = add(c1, c2, kSampledV);
  } else {
    cam1 = add(l1, l2, c1);
    cam2 = add(c1, l1, c2);
    lit1 = add(c1, c2, l1);
    lit2 = add(l1, c1, l2);
  }
  float rv[4];
  for (int q = 0; q < nq; q++) {
    BVert cur = fetch_vert(C, Lp, sampled, rq[q][0]);
    BVert next = fetch_vert(C, Lp, sampled, rq[q][2]);
    if (CLS == 0 && q == cam1) {
      rv[q] = light_origin_pdf(sc, cur, next);
    } else {
      BVert prev;
      bool hp = rq[q][1] != kNoV;
      if (hp) prev = fetch_vert(C, Lp, sampled, rq[q][1]);
      rv[q] = vertex_pdf(sc, cur, hp ? &prev : nullptr, next);
    }
  }
  // the walk of bdpt_mis.go:61-178 in prefix form: the two steps next to
  // the connection on each side (with the recomputed reverse pdfs and the
  // connection's own connectibility), then the subpath's stored prefix
  float sum = 0.f;
  if (t >= 2) {  // camera vertices t-1 .. 1
    VPdf v1 = C.pdfs(t - 1), v2 = C.pdfs(t - 2);
    float r1 = remap0(cam1 >= 0 ? rv[cam1] : v1.rev) / remap0(v1.fwd);
    bool c1 = (cam1 >= 0 || !(v1.flags & kFlagSpecular)) && !(v2.flags & kFlagSpecular);
    float inner = 0.f;
    if (t >= 3) {
      VPdf v3 = C.pdfs(t - 3);
      float r2 = remap0(cam2 >= 0 ? rv[cam2] : v2.rev) / remap0(v2.fwd);
      bool c2 = !(v2.flags & kFlagSpecular) && !(v3.flags & kFlagSpecular);
      inner = r2 * (v3.pre + (c2 ? 1.f : 0.f));
    }
    sum += r1 * (inner + (c1 ? 1.f : 0.f));
  }
  if (s >= 1) {  // light vertices s-1 .. 0
    VPdf u1 = Lp.pdfs(s - 1);
    float fw1 = (CLS == 2 && lit1 >= 0) ? sampled->fwd : u1.fwd;
    float q1 = remap0(lit1 >= 0 ? rv[lit1] : u1.rev) / remap0(fw1);
    bool d1 = !(u1.flags & kFlagSpecular) && !is_delta_light(sc, u1);
    float inner = 0.f;
    if (s >= 2) {
      VPdf u2 = Lp.pdfs(s - 2);
      bool ok2 = !(u2.flags & kFlagSpecular) && !is_delta_light(sc, u2);
      d1 = d1 && ok2;
      float q2 = remap0(lit2 >= 0 ? rv[lit2] : u2.rev) / remap0(u2.fwd);
      bool d2 = ok2;
      float b3 = 0.f;
      if (s >= 3) {
        VPdf u3 = Lp.pdfs(s - 3);
        d2 = d2 && !(u3.flags & kFlagSpecular) && !is_delta_light(sc, u3);
        b3 = u3.pre;
      }
      inner = q2 * (b3 + (d2 ? 1.f : 0.f));
    }
    if (lit1 >= 0) d1 = true;
    sum += q1 * (inner + (d1 ? 1.f : 0.f));
  }
  return 1.f / (1.f + sum);
}

// Uniform numbers the strategies before (s, t) draw, in the reference's
// s-major order: light tracing (s >= 2, t = 1) draws 2 when its light vertex
// is not specular (mask bit s); direct lighting (s = 1, t >= 2) draws 3 when
// its camera vertex is a non-specular surface and the scene has lights (mask
// bit t); every other strategy draws nothing.
__device__ __forceinline__ uint32_t draws_before(int s, int t, uint2 m) {
  if (s == 0) return 0;
  uint32_t lo_t = ((1u << t) - 1u) & ~3u;  // bits 2 .. t-1
  if (s == 1) return 3u * __popc(m.y & lo_t);
  uint32_t lo_s = ((1u << s) - 1u) & ~3u;  // bits 2 .. s-1
  return 3u * __popc(m.y) + 2u * __popc(m.x & lo_s) + (t > 1 ? 2u * ((m.x >> s) & 1u) : 0u);
}

// evaluateBDPTStrategy (bdpt.go:294-561) for strategy (s, t) of sample i;
// returns the weighted contribution to the sample (t = 1 splats instead).
template <int CLS>
__device__ __forceinline__ float3 eval_strategy(const DevScene& sc, const DevFilm& film, const DevBdpt& B, uint32_t i,
                                             int s, int t, Rng& rs, int* err) {
  const float3 zero = f3(0.f, 0.f, 0.f);
  SubpathRef C{&B, i, 0}, Lp{&B, i, B.maxv};
  float3 Lc = zero;
  BVert sampled;
  bool has = false, splat = false;
  int spx = 0, spy = 0;
  bool test = false;
  float3 ro = zero, rd = f3(0.f, 0.f, 1.f);
  float rt = 0.f;
  uint32_t rskip = kNoHit;
  if (CLS == 0) {
    // evaluatePathTracingStrategy (bdpt.go:317-332): the caller passes t == nc only
    BVert last = C[t - 1];
    Lc = last.Le * last.beta;
  } else if (CLS == 1) {
    // evaluateLightTracingStrategy (bdpt.go:398-486)
    BVert lv = Lp[s - 1];
    if (s <= 1 || lv.is(kFlagSpecular)) return zero;
    float2 cs = rs.next2();
    float2 lens2 = sample_unit_disk(cs);
    float3 lp = sc.cam.center + sc.cam.u * (lens2.x * sc.cam.lens_radius) + sc.cam.v * (lens2.y * sc.cam.lens_radius);
    float3 toRef = lv.p - lp;
    float dist = length(toRef);
    float3 dir = normalize(toRef);
    float cpdf = (dist * dist) / (fabsf(dot(sc.cam.forward, dir)) * sc.cam.lens_area);
    float imp = camera_importance(sc.cam, dir);
    if (imp == 0.f) return zero;  // SampleCameraFromPoint returns nil
    float3 toCam = -dir;
    float3 f = vertex_brdf(sc, lv, toCam, false);
    float cb = imp / cpdf;
    float cosine = dot(toCam, lv.n);
    if (cosine <= 0.f) return zero;
    float3 c = f * cb * lv.beta;
    if (on_surface(sc, lv)) c = c * cosine;
    if (is_zero(c)) return zero;
    test = true;
    ro = lv.p;
    rd = toCam;
    rt = dist - 0.001f;
    rskip = lv.prim;
    sampled.p = lp;
    sampled.n = toCam;
    sampled.wi = dir;  // (scratch: the lens-to-vertex direction)
    sampled.beta = f3(cb, cb, cb);
    sampled.Le = zero;
    sampled.fwd = cpdf;
    sampled.rev = 0.f;
    sampled.mat = -1;
    sampled.light = -1;
    sampled.prim = kNoHit;
    sampled.flags = kFlagCamera;
    has = true;
    splat = true;
    Lc = c;
  } else if (CLS == 2) {
    // evaluateDirectLightingStrategy (bdpt.go:334-394)
    BVert cv = C[t - 1];
    if (cv.is(kFlagSpecular) || cv.mat < 0) return zero;
    if (sc.n_lights == 0) return zero;
    int li = pick_light(sc, rs.next());
    DevLight L = sc.lights[li];
    LightSample ls = light_sample(sc, L, cv.p, cv.n, rs.next2());
    ls.pdf *= L.prob;
    if (is_zero(ls.emission) || ls.pdf <= 0.f) return zero;
    float ct = fabsf(dot(ls.dir, cv.n));
    if (ct <= 0.f) return zero;
    float3 f = vertex_brdf(sc, cv, ls.dir, true);
    float3 lb = ls.emission * (1.f / ls.pdf);
    float3 c = f * cv.beta * lb * ct;
    if (is_zero(c)) return zero;
    test = true;
    ro = cv.p;
    rd = ls.dir;
    rt = ls.dist - 0.001f;
    rskip = cv.prim;
    sampled.p = ls.point;
    sampled.n = ls.normal;
    sampled.wi = zero;
    sampled.light = li;
    sampled.mat = -1;
    sampled.prim = kNoHit;
    sampled.fwd = ls.pdf;
    sampled.rev = 0.f;
    bool inf = L.kind == kLightUniformInfinite || L.kind == kLightGradientInfinite;
    sampled.flags = kFlagLight | (inf ? kFlagInfinite : 0);
    sampled.beta = lb;
    sampled.Le = ls.emission;
    has = true;
    Lc = c;
  } else {
    // evaluateConnectionStrategy (bdpt.go:502-561)
    BVert lv = Lp[s - 1];
    BVert cv = C[t - 1];
    if (lv.is(kFlagSpecular) || cv.is(kFlagSpecular)) return zero;
    float3 dd = lv.p - cv.p;
    float dist = length(dd);
    if (dist < 0.001f) return zero;
    dd = dd * (1.f / dist);
    float cc = dot(dd, cv.n), cl = dot(-dd, lv.n);
    if (cc <= 0.f || cl <= 0.f) return zero;
    float g = (cc * cl) / (dist * dist);
    float3 cb = vertex_brdf(sc, cv, dd, true);
    float3 lb = vertex_brdf(sc, lv, -dd, false);
    float3 c = lv.beta * lb * cb * cv.beta * g;
    if (is_zero(c)) return zero;
    test = true;
    ro = cv.p;
    rd = dd;
    rt = dist - 0.001f;
    rskip = cv.prim;
    Lc = c;
  }
  if (test && occluded(sc, ro, rd, rt, rskip, err)) return zero;
  if (splat) {
    // MapRayToPixel, then the light pdf of the camera vertex (bdpt.go:440-470)
    float3 dir = sampled.wi;
    sampled.wi = zero;
    if (!map_ray_to_pixel(sc.cam, sampled.p, dir, spx, spy)) return zero;
    sampled.rev = total_light_pdf(sc, sampled.p, sampled.n, normalize(Lp[s - 1].p - sampled.p));
  }
  if (is_zero(Lc) && !splat) return zero;
  float w = mis_weight<CLS>(sc, C, Lp, has ? &sampled : nullptr, s, t);
  if (splat) {
    float3 c = Lc * w;
    float4* dst = film.splat + (size_t)spy * film.width + spx;
    atomicAdd(&dst->x, c.x);
    atomicAdd(&dst->y, c.y);
    atomicAdd(&dst->z, c.z);
    return zero;
  }
  return Lc * w;
}

// generateCameraPath (bdpt.go:106-135): the camera vertex and ray of every
// sample of the chunk, queue 0 slot p = sample p.
template <int MAXV>
__global__ void k_bdpt_camgen(DevScene sc, DevFilm film, DevPaths PS, ChunkDesc ch) {
  const DevBdpt& B = PS.bd;
  const uint32_t n = ch.npix * ch.layers;
  const BdQueue& Q = B.q[0];
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    uint32_t layer = p / ch.npix, i = p - layer * ch.npix;
    uint32_t pix = ch.pix_list ? ch.pix_list[ch.pix0 + i] : ch.pix0 + i;
    uint32_t sample = film.count[pix] + layer;
    int x = (int)(pix % (uint32_t)film.width), y = (int)(pix / (uint32_t)film.width);
    Rng rng;
    rng.init(ch.seed, pix, sample);
    float2 lens = rng.next2();
    float2 jit = rng.next2();
    float3 o, d;
    camera_ray(sc.cam, x, y, lens, jit, o, d);
    BVert c;
    c.p = o;
    c.n = -d;
    c.wi = f3(0.f, 0.f, 0.f);
    c.beta = f3(1.f, 1.f, 1.f);
    c.Le = f3(0.f, 0.f, 0.f);
    c.uv = make_float2(0.f, 0.f);
    c.fwd = 0.f;
    c.rev = 0.f;
    c.mat = -1;
    c.light = -1;
    c.prim = kNoHit;
    c.flags = kFlagCamera;
    put_vert(B, 0, p, c, 0.f);
    Q.o[p] = make_float4(o.x, o.y, o.z, __uint_as_float(kNoHit));
    Q.d[p] = make_float4(d.x, d.y, d.z, camera_dir_pdf(sc.cam, o, d));
    Q.beta[p] = make_float4(1.f, 1.f, 1.f, 0.f);
    Q.last[p] = make_float4(c.n.x, c.n.y, c.n.z, 0.f);
    Q.ids[p] = make_uint4(p, rng.pos, pix, sample);
    Q.st[p] = make_uint2(1u | kStCamera | kStOkBefore | kStOkLast, 0u);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    PS.counters[0] = n;
    PS.counters[1] = 0;
    PS.counters[4] = 0;
  }
}

// The rays of the subpath queue; the marker hit of a stack overflow sets the
// job's error bits and is stored as a miss.
struct BdptSource {
  const float4* o;
  const float4* d;
  float4* hit;
  const uint32_t* n;
  int root;
  int* err;
  __device__ uint32_t count() const { return *n; }
  __device__ void load(uint32_t i, float3& ro, float3& rd, float& tmin, float& tmax, uint32_t& skip, int& rt) const {
    float4 a = o[i], b = d[i];
    ro = f3(a);
    rd = f3(b);
    tmin = 0.001f;
    tmax = kInfF;
    skip = __float_as_uint(a.w);
    rt = root;
  }
  __device__ void store(uint32_t i, const Hit& h) const {
    bool any = h.prim != kNoHit;
    if (h.prim == kOverflowHit) {
      atomicOr(err, kErrStackOverflow);
      any = false;
    }
    hit[i] = make_float4(any ? h.t : -1.f, __uint_as_float(any ? h.prim : kNoHit), h.u, h.v);
  }
};

__global__ void __launch_bounds__(128, 8) k_bdpt_trace(DevScene sc, BdptSource src, uint32_t* counters, int cur) {
  if (blockIdx.x == 0 && threadIdx.x == 0) counters[cur ^ 1] = 0;  // the next queue starts empty
  trace_persistent<false, false>(sc, src, counters + 4, nullptr, nullptr);
}

// One bounce of extendPath (bdpt.go:206-291) for every subpath of queue
// `cur`: the vertex hit (or the camera subpath's background vertex,
// createBackgroundVertex bdpt.go:585-601), its scatter, the reverse pdf of
// the vertex before it; continuing subpaths move to queue cur ^ 1.  A camera
// subpath that ends starts the sample's light subpath (generateLightPath,
// bdpt.go:139-202); a light subpath that ends gets the infinite-light pdf
// fix-ups and completes its sample.
template <int MAXV>
__global__ void __launch_bounds__(128, 4) k_bdpt_extend(DevScene sc, DevPaths PS, ChunkDesc ch, int cur) {
  const DevBdpt& B = PS.bd;
  const BdQueue& Q = B.q[cur];
  const BdQueue& N = B.q[cur ^ 1];
  const uint32_t n = PS.counters[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) PS.counters[4] = 0;  // the next traversal's ray fetch counter
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    uint32_t i = base + threadIdx.x;
    bool live = i < n;
    bool cont = false;
    float4 no = make_float4(0.f, 0.f, 0.f, 0.f), nd = no, nb = no, nl4 = no;
    uint4 nids = make_uint4(0, 0, 0, 0);
    uint2 nst = make_uint2(0, 0);
    if (live) {
      float4 o4 = Q.o[i], d4 = Q.d[i], b4 = Q.beta[i], l4 = Q.last[i], h4 = B.hit[i];
      uint4 ids = Q.ids[i];
      uint2 st2 = Q.st[i];
      const uint32_t p = ids.x;
      Rng rng;
      rng.init(ch.seed, ids.z, ids.w, ids.y);
      const uint32_t bits = st2.x;
      bool camera = bits & kStCamera;
      int len = (int)(bits & 0xFF), b = (int)((bits >> 8) & 0xFF);
      int nc = (int)st2.y;
      const int vb = camera ? 0 : MAXV;  // vertex base of the subpath
      const int max_bounces = camera ? sc.max_depth : sc.max_depth - 1;
      float3 o = f3(o4), d = f3(d4), beta = f3(b4);
      float pdf_fwd = d4.w, acc = b4.w;
      bool ok_before = bits & kStOkBefore, ok_last = bits & kStOkLast;
      bool surf_last = bits & kStSurfLast, inf_last = bits & kStInfLast;
      float3 last_n = f3(l4);
      float last_fwd = l4.w;
      bool ended = true;
      uint32_t prim = __float_as_uint(h4.y);
      float rev_last = 0.f;  // the reverse pdf of the last vertex (0 unless the new vertex scatters)
      BVert v;
      bool has_v = false, v_ok = false;
      if (prim == kNoHit) {
        if (camera) {  // createBackgroundVertex (bdpt.go:585-601)
          float3 bg = background(sc, d);
          v.p = o + d * 1000.f;
          v.n = -d;
          v.wi = -d;
          v.fwd = pdf_fwd;
          v.rev = 0.f;
          v.beta = beta;
          v.Le = bg;
          v.uv = make_float2(0.f, 0.f);
          v.mat = -1;
          v.light = -1;
          v.prim = kNoHit;
          v.flags = kFlagInfinite | (is_zero(bg) ? 0 : kFlagLight);
          has_v = true;
        }
      } else {
        Hit h{h4.x, prim, h4.z, h4.w};
        Surface s;
        surface_at(sc, o, d, h, s);
        DevMaterial m = load_material(sc, s.mat);
        v.p = s.p;
        v.n = s.n;
        v.wi = -d;
        v.beta = beta;
        v.Le = emitted(m, s.front, d);
        v.mat = s.mat;
        v.uv = s.uv;
        v.light = -1;
        v.prim = prim;
        v.flags = (s.front ? kFlagFront : 0) | (is_zero(v.Le) ? 0 : kFlagLight);
        v.rev = 0.f;
        v.fwd = to_area_at(o, v.p, v.n, v.mat >= 0, false, pdf_fwd);
        has_v = true;
        Scatter scn;
        if (scatter(sc, m, d, s, rng, scn)) {
          float npdf = scn.pdf;
          if (scn.pdf <= 0.f) v.flags |= kFlagSpecular;
          float ct = fabsf(dot(scn.dir, s.n));
          float3 nbeta = scn.pdf <= 0.f ? beta * scn.att : beta * scn.att * (ct / scn.pdf);
          bool rdelta;
          float pdf_rev = mat_pdf(sc, m, scn.dir, -d, s.n, rdelta);
          if (rdelta) {
            v.flags |= kFlagSpecular;
            pdf_rev = 0.f;
            npdf = 0.f;
          }
          rev_last = to_area_at(v.p, o, last_n, surf_last, inf_last, pdf_rev);
          if (b + 1 < max_bounces && len + 1 < MAXV) {
            ended = false;
            no = make_float4(s.p.x, s.p.y, s.p.z, __uint_as_float(prim));
            nd = make_float4(scn.dir.x, scn.dir.y, scn.dir.z, npdf);
            beta = nbeta;
          }
        }
      }
      // the last vertex is final now: its reverse pdf and MIS prefix
      float pre_last = next_prefix(camera, len - 1, rev_last, last_fwd, ok_last, ok_before, acc);
      patch_vert(B, vb + len - 1, p, rev_last, pre_last);
      if (has_v) {
        v_ok = vertex_ok(sc, v, camera);
        // a vertex that ends its subpath is stored with its final prefix
        float pre_v = ended ? next_prefix(camera, len, 0.f, v.fwd, v_ok, ok_last, pre_last) : 0.f;
        put_vert(B, vb + len, p, v, pre_v);
        len++;
      }
      if (!ended) {
        nb = make_float4(beta.x, beta.y, beta.z, pre_last);
        nl4 = make_float4(v.n.x, v.n.y, v.n.z, v.fwd);
        nids = make_uint4(p, rng.pos, ids.z, ids.w);
        nst = make_uint2((uint32_t)len | ((uint32_t)(b + 1) << 8) | (camera ? kStCamera : 0u) |
                             (ok_last ? kStOkBefore : 0u) | (v_ok ? kStOkLast : 0u) | (v.mat >= 0 ? kStSurfLast : 0u),
                         (uint32_t)nc);
        cont = true;
      } else if (camera) {
        nc = len;
        if (sc.n_lights > 0) {
          // generateLightPath (bdpt.go:139-202), in the same sampler stream
          int li = pick_light(sc, rng.next());
          DevLight L = sc.lights[li];
          float2 sp = rng.next2();
          float2 sd = rng.next2();
          float3 ep, en, ed, Le;
          float apdf, dpdf;
          sample_emission(sc, L, sp, sd, ep, en, ed, Le, apdf, dpdf);
          float ct = fabsf(dot(ed, en));
          BVert lv;
          lv.p = ep;
          lv.n = en;
          lv.wi = f3(0.f, 0.f, 0.f);
          lv.uv = make_float2(0.f, 0.f);
          lv.light = li;
          lv.mat = -1;
          lv.prim = L.kind == kLightQuad     ? sc.quad_base + (uint32_t)L.prim
                    : L.kind == kLightSphere ? (L.prim >= 0 ? sc.sphere_base + (uint32_t)L.prim : kNoHit)
                    : (L.kind == kLightDisc || L.kind == kLightDiscSpot) ? sc.quadric_base + (uint32_t)L.prim
                                                                         : kNoHit;
          lv.fwd = apdf * L.prob;
          lv.rev = 0.f;
          bool inf = L.kind == kLightUniformInfinite || L.kind == kLightGradientInfinite;
          lv.flags = kFlagLight | (inf ? kFlagInfinite : 0);
          lv.beta = Le;
          lv.Le = Le;
          bool lok = vertex_ok(sc, lv, false);
          bool lsurf = light_is_area(sc, li);
          if (inf) {
            B.lorig[3 * (size_t)p] = make_float4(ep.x, ep.y, ep.z, apdf);
            B.lorig[3 * (size_t)p + 1] = make_float4(en.x, en.y, en.z, L.prob);
            B.lorig[3 * (size_t)p + 2] = make_float4(ed.x, ed.y, ed.z, 0.f);
          }
          if (0 < sc.max_depth - 1 && 1 < MAXV) {
            put_vert(B, MAXV, p, lv, 0.f);
            float3 lb = Le * (ct / (L.prob * apdf * dpdf));
            no = make_float4(ep.x, ep.y, ep.z, __uint_as_float(lv.prim));
            nd = make_float4(ed.x, ed.y, ed.z, dpdf);
            nb = make_float4(lb.x, lb.y, lb.z, 0.f);
            nl4 = make_float4(en.x, en.y, en.z, lv.fwd);
            nids = make_uint4(p, rng.pos, ids.z, ids.w);
            nst = make_uint2(1u | kStOkBefore | (lok ? kStOkLast : 0u) | (lsurf ? kStSurfLast : 0u) |
                                 (inf ? kStInfLast : 0u),
                             (uint32_t)nc);
            cont = true;
          } else {  // a light subpath of the light vertex alone
            put_vert(B, MAXV, p, lv, next_prefix(false, 0, 0.f, lv.fwd, lok, true, 0.f));
            if (inf) {  // the fix-up of the light vertex (bdpt.go:188-199)
              BVert l0 = get_vert(B, MAXV, p);
              l0.fwd = infinite_density(sc, ep, en, ed);
              put_vert(B, MAXV, p, l0);
              subpath_prefix(sc, B, MAXV, 1, p, false);
            }
            finish_sample<MAXV>(sc, B, p, nc, 1, rng.pos, ids.z, ids.w);
          }
        } else {
          finish_sample<MAXV>(sc, B, p, nc, 0, rng.pos, ids.z, ids.w);
        }
      } else {
        int nl = len;
        if (get_vpdf(B, MAXV, p).flags & kFlagInfinite) {
          // the infinite-light fix-ups of generateLightPath (bdpt.go:188-199)
          float4 e0 = B.lorig[3 * (size_t)p], e1 = B.lorig[3 * (size_t)p + 1], e2 = B.lorig[3 * (size_t)p + 2];
          float3 ep = f3(e0), en = f3(e1), ed = f3(e2);
          float apdf = e0.w, lprob = e1.w;
          if (nl > 1) {
            BVert fb = get_vert(B, MAXV + 1, p);
            fb.fwd = apdf * lprob;
            if (fb.mat >= 0) fb.fwd *= fabsf(dot(ed, fb.n));
            put_vert(B, MAXV + 1, p, fb);
          }
          BVert l0 = get_vert(B, MAXV, p);
          l0.fwd = infinite_density(sc, ep, en, ed);
          put_vert(B, MAXV, p, l0);
          subpath_prefix(sc, B, MAXV, nl, p, false);  // the corrected pdfs change every prefix
        }
        finish_sample<MAXV>(sc, B, p, nc, nl, rng.pos, ids.z, ids.w);
      }
    }
    // continuing subpaths to consecutive slots of the next queue (one atomic per warp)
    uint32_t slot = warp_append(&PS.counters[cur ^ 1], live && cont);
    if (live && cont) {
      N.o[slot] = no;
      N.d[slot] = nd;
      N.beta[slot] = nb;
      N.last[slot] = nl4;
      N.ids[slot] = nids;
      N.st[slot] = nst;
    }
  }
}

// Strategy k = s * MAXV + (t - 1) of a sample is evaluated when s <= nl and
// t <= nc, except (1,1) (bdpt.go:300-301) and s = 0 with t != nc (the
// path-tracing strategy contributes only at the full camera path).
__device__ __forceinline__ bool has_strategy(int s, int t, int nc, int nl) {
  return s <= nl && t <= nc && !(s == 1 && t == 1) && !(s == 0 && t != nc);
}

// A strategy the sample has whose contribution can be non-zero: listed for
// the strategy kernels and summed.  The others return zero before drawing
// any number, so leaving them out changes neither a sampler position
// (draws_before) nor a sum: light tracing with a specular light vertex
// (mask bit s clear), direct lighting at a specular or material-less camera
// vertex or without lights (bit t clear), and a connection with either
// (bdpt.go:398-561).
__device__ __forceinline__ bool listed_strategy(int s, int t, int nc, int nl, uint2 m) {
  if (!has_strategy(s, t, nc, nl)) return false;
  if (s == 0) return true;
  bool ls = (m.x >> s) & 1u, ct = (m.y >> t) & 1u;
  return t == 1 ? ls : s == 1 ? ct : ls && ct;
}

// Lists, per strategy, the samples that have it, so that the strategy kernel
// gives each warp 32 real (s, t, sample) items.  A block of 1,024 samples
// counts each strategy's items in shared memory (one shared atomic per warp
// and strategy), reserves its range of every list with one global atomic per
// strategy, then writes the items: per-warp global atomics on the
// (MAXV + 1) x MAXV list counters serialised in L2 (16.7 ms of a 200 ms
// Cornell-boxes frame).  The order within a list does not matter: every
// item writes its own contribution slot.
template <int MAXV>
__global__ void __launch_bounds__(1024) k_bdpt_list(DevPaths PS, ChunkDesc ch) {
  constexpr int K = (MAXV + 1) * MAXV;
  __shared__ uint32_t cnt[K], base[K];
  __shared__ uint16_t wofs[32][K];  // each warp's offset within the block's range (< 1,024)
  const DevBdpt& B = PS.bd;
  const uint32_t n = ch.npix * ch.layers;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  for (uint32_t start = blockIdx.x * 1024u; start < n; start += gridDim.x * 1024u) {
    const uint32_t w = start / kBdWindow;  // the block's samples lie in one window
    for (int k = threadIdx.x; k < K; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    uint32_t i = start + threadIdx.x;
    int nc = 0, nl = -1;
    uint2 mk = make_uint2(0u, 0u);
    if (i < n) {
      uint32_t m = B.meta[i].x;
      nc = (int)(m & 0xFF);
      nl = (int)(m >> 8);
      mk = B.masks[i];
    }
    // a warp visits only the strategies its longest subpaths reach (both
    // loops over the same range: wofs is written and read for those only)
    const int wnc = __reduce_max_sync(0xFFFFFFFFu, nc), wnl = __reduce_max_sync(0xFFFFFFFFu, nl);
    for (int s = 0; s <= wnl; s++)
      for (int t = 1; t <= wnc; t++) {
        const int k = s * MAXV + t - 1;
        unsigned mask = __ballot_sync(0xFFFFFFFFu, listed_strategy(s, t, nc, nl, mk));
        if (mask && lane == 0) wofs[wp][k] = (uint16_t)atomicAdd(&cnt[k], (uint32_t)__popc(mask));
      }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x)
      base[k] = cnt[k] ? w * kBdWindow + atomicAdd(B.scount + w * K + k, cnt[k]) : 0u;
    __syncthreads();
    for (int s = 0; s <= wnl; s++)
      for (int t = 1; t <= wnc; t++) {
        const int k = s * MAXV + t - 1;
        bool has = listed_strategy(s, t, nc, nl, mk);
        unsigned mask = __ballot_sync(0xFFFFFFFFu, has);
        if (has) B.slist[(size_t)k * B.ns + base[k] + wofs[wp][k] + __popc(mask & below)] = i;
      }
    __syncthreads();  // cnt, base and wofs are rewritten for the next range
  }
}

// The strategy classes, each evaluated by its own launch so that a launch
// holds only its class's code: 0 the path-tracing strategy (s = 0, t = nc),
// 1 light tracing (s >= 2, t = 1), 2 direct lighting (s = 1, t >= 2),
// 3 connections (s, t >= 2).
__host__ __device__ constexpr int strategy_class(int s, int t) {
  return s == 0 ? 0 : t == 1 ? 1 : s == 1 ? 2 : 3;
}

// The per-class prefix sums of the list counts in (window, strategy) order,
// which map a strategy kernel's class-wide item index g to the entry
// e = w * K + k with sprefix[e] <= g < sprefix[e + 1].  One block: each
// thread sums a contiguous run of entries for the four classes, and a
// block-wide scan of the runs gives their offsets.
template <int MAXV>
__global__ void __launch_bounds__(1024) k_bdpt_prefix(DevPaths PS) {
  constexpr int K = (MAXV + 1) * MAXV;
  __shared__ uint32_t part[4][1024];
  const DevBdpt& B = PS.bd;
  const uint32_t E = B.nw * K;
  const uint32_t per = (E + 1023u) / 1024u;
  const uint32_t t = threadIdx.x;
  const uint32_t lo = min(E, t * per), hi = min(E, lo + per);
  uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (uint32_t e = lo; e < hi; e++) {
    int k = (int)(e % K), c = strategy_class(k / MAXV, k % MAXV + 1);
    uint32_t v = B.scount[e];
    s0 += c == 0 ? v : 0u;
    s1 += c == 1 ? v : 0u;
    s2 += c == 2 ? v : 0u;
    s3 += c == 3 ? v : 0u;
  }
  part[0][t] = s0;
  part[1][t] = s1;
  part[2][t] = s2;
  part[3][t] = s3;
  __syncthreads();
  for (uint32_t d = 1; d < 1024u; d <<= 1) {  // inclusive scan (Hillis-Steele)
    uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    if (t >= d) {
      a0 = part[0][t - d];
      a1 = part[1][t - d];
      a2 = part[2][t - d];
      a3 = part[3][t - d];
    }
    __syncthreads();
    part[0][t] += a0;
    part[1][t] += a1;
    part[2][t] += a2;
    part[3][t] += a3;
    __syncthreads();
  }
  uint32_t r0 = part[0][t] - s0, r1 = part[1][t] - s1, r2 = part[2][t] - s2, r3 = part[3][t] - s3;
  uint32_t* P = B.sprefix;
  for (uint32_t e = lo; e < hi; e++) {
    P[e] = r0;
    P[(E + 1) + e] = r1;
    P[2 * (E + 1) + e] = r2;
    P[3 * (E + 1) + e] = r3;
    int k = (int)(e % K), c = strategy_class(k / MAXV, k % MAXV + 1);
    uint32_t v = B.scount[e];
    r0 += c == 0 ? v : 0u;
    r1 += c == 1 ? v : 0u;
    r2 += c == 2 ? v : 0u;
    r3 += c == 3 ? v : 0u;
  }
  if (t == 1023u) {
    P[E] = part[0][t];
    P[(E + 1) + E] = part[1][t];
    P[2 * (E + 1) + E] = part[2][t];
    P[3 * (E + 1) + E] = part[3][t];
  }
}

// One thread per listed (strategy, sample) item of class CLS, in (window,
// strategy) order: a warp evaluates one (s, t) for 32 samples of one window
// that have it (uniform control flow, neighbouring warps on the same code),
// and every strategy of a window of samples runs before the next window, so
// the vertex reads of the window's later strategies hit L2.  The work is
// latency-bound; 8 blocks per SM (at most 64 registers, a few spilled)
// measured fastest on the Cornell-boxes frame (558 ms vs 624 ms at 96
// registers and 5 blocks).
template <int MAXV, int CLS>
__global__ void __launch_bounds__(128, 8) k_bdpt_strategies(DevScene sc, DevFilm film, DevPaths PS, ChunkDesc ch) {
  constexpr int K = (MAXV + 1) * MAXV;
  const DevBdpt& B = PS.bd;
  const uint32_t n = ch.npix * ch.layers;
  const uint32_t E = B.nw * K;
  const uint32_t* P = B.sprefix + (size_t)CLS * (E + 1);
  const uint32_t total = __ldg(P + E);
  int* err = reinterpret_cast<int*>(PS.counters + 3);
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = E;  // P[lo] <= g < P[hi]
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (__ldg(P + mid) <= g) lo = mid;
      else hi = mid;
    }
    const uint32_t w = lo / K;
    const int k = (int)(lo - w * K);
    const uint32_t i = B.slist[(size_t)k * B.ns + w * kBdWindow + (g - __ldg(P + lo))];
    const int s = k / MAXV, t = k % MAXV + 1;
    uint4 m = B.meta[i];
    Rng rs;
    rs.init(ch.seed, m.z, m.w, m.y + draws_before(s, t, B.masks[i]));
    float3 c = eval_strategy<CLS>(sc, film, B, i, s, t, rs, err);
    B.contrib[(size_t)k * n + i] = make_float4(c.x, c.y, c.z, 0.f);
  }
}

template <int MAXV>
__global__ void k_bdpt_sum(DevPaths PS, ChunkDesc ch) {
  const DevBdpt& B = PS.bd;
  uint32_t n = ch.npix * ch.layers;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint4 m = B.meta[i];
    const uint2 mk = B.masks[i];
    int nc = (int)(m.x & 0xFF), nl = (int)(m.x >> 8);
    float3 total = f3(0.f, 0.f, 0.f);
    for (int s = 0; s <= nl; s++)
      for (int t = 1; t <= nc; t++) {
        if (!listed_strategy(s, t, nc, nl, mk)) continue;  // contributes nothing: not evaluated
        float4 c = B.contrib[(size_t)(s * MAXV + t - 1) * n + i];
        total += f3(c);
      }
    PS.Lout[i] = make_float4(total.x, total.y, total.z, 0.f);
  }
}

template <int MAXV>
void launch_bdpt_maxv(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int sms,
                      cudaStream_t st) {
  const uint32_t n = ch.npix * ch.layers;
  const int gs = launch_grid(n, 128, std::max(1, sms * 8));  // grid-stride kernels over the queue
  const int gt = std::max(1, sms * 8);                       // persistent traversal
  const int g2 = std::max(1, sms * 16);
  const int g3 = launch_grid(n, 256, 0);
  const int gl = std::min(launch_grid(n, 1024, 0), std::max(1, sms * 2));
  k_bdpt_camgen<MAXV><<<g3, 256, 0, st>>>(sc, film, P, ch);
  int cur = 0;
  // at most max_depth camera bounces, then max_depth - 1 light bounces
  for (int it = 0; it < 2 * sc.max_depth; it++) {
    BdptSource src{P.bd.q[cur].o, P.bd.q[cur].d, P.bd.hit, P.counters + cur, sc.root,
                   reinterpret_cast<int*>(P.counters + 3)};
    k_bdpt_trace<<<gt, 128, 0, st>>>(sc, src, P.counters, cur);
    k_bdpt_extend<MAXV><<<gs, 128, 0, st>>>(sc, P, ch, cur);
    cur ^= 1;
  }
  k_bdpt_list<MAXV><<<gl, 1024, 0, st>>>(P, ch);
  k_bdpt_prefix<MAXV><<<1, 1024, 0, st>>>(P);
  k_bdpt_strategies<MAXV, 0><<<g2, 128, 0, st>>>(sc, film, P, ch);
  k_bdpt_strategies<MAXV, 1><<<g2, 128, 0, st>>>(sc, film, P, ch);
  k_bdpt_strategies<MAXV, 2><<<g2, 128, 0, st>>>(sc, film, P, ch);
  k_bdpt_strategies<MAXV, 3><<<g2, 128, 0, st>>>(sc, film, P, ch);
  k_bdpt_sum<MAXV><<<g3, 256, 0, st>>>(P, ch);
}

}  // namespace

// Subpaths as a wavefront (camera rays, then per bounce: traversal and
// extension over the compacted queue), per-strategy lists, one launch per
// strategy class, the per-sample sums.
void launch_bdpt(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                 cudaStream_t st) {
  (void)block;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaMemsetAsync(P.bd.scount, 0, sizeof(uint32_t) * P.bd.nw * (P.bd.maxv + 1) * P.bd.maxv, st);
  if (P.bd.maxv == 10) launch_bdpt_maxv<10>(sc, film, P, ch, sms, st);
  else launch_bdpt_maxv<18>(sc, film, P, ch, sms, st);
}

}  // namespace gprt
