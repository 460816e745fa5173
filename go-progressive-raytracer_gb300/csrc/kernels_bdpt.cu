// kernels_bdpt.cu - bidirectional path tracing, one pixel sample per thread.
//
// Restates BDPTIntegrator.RayColor (pkg/integrator/bdpt.go:73-102): a camera
// subpath and a light subpath are generated (generateCameraPath :106-135,
// generateLightPath :139-202, extendPath :206-291), every (s,t) strategy is
// evaluated (:294-561) and weighted by calculateMISWeight
// (pkg/integrator/bdpt_mis.go:13-335).  t=1 light-tracing contributions are
// splatted into the film's splat buffer with atomic adds and applied after
// the pass (processSplats, pkg/renderer/progressive.go:371-391).
// The subpath vertices live in per-thread local arrays (the compiler
// interleaves local memory per thread, so the accesses are coalesced).
#include "device.cuh"
#include "kernels.h"

namespace gprt {

namespace {

constexpr int kFlagLight = 1, kFlagCamera = 2, kFlagSpecular = 4, kFlagInfinite = 8, kFlagFront = 16;

struct BVert {  // bdpt.go:14-36
  float3 p, n, beta, Le, wi;
  float fwd, rev;
  int mat;    // material index, -1 for none
  int light;  // index in the light table, -1 for none
  uint32_t prim;
  int flags;
  __device__ bool is(int f) const { return (flags & f) != 0; }
};

__device__ __forceinline__ bool light_is_area(const DevScene& sc, int li) {
  int k = sc.lights[li].kind;
  return k == kLightQuad || k == kLightSphere;
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
// light_sampling.go:58-115 for the infinite lights)
__device__ void sample_emission(const DevScene& sc, const DevLight& L, float2 sp, float2 sd, float3& p, float3& n,
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
    float4 S = __ldg(sc.spheres + (size_t)L.prim * 2);
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
// uniform_infinite_light.go:94-106); pos receives the position pdf
__device__ float pdf_le(const DevScene& sc, const DevLight& L, float3 p, float3 dir, float& pos) {
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
    float4 S = __ldg(sc.spheres + (size_t)L.prim * 2);
    float dc = length(p - f3(S));
    if (!(fabsf(dc - S.w) <= 0.001f * fmaxf(1.f, fabsf(S.w) * 1e-3f))) return 0.f;
    float3 n = normalize(p - f3(S));
    if (dot(dir, n) <= 0.f) return 0.f;
    pos = 1.0f / (4.f * kPi * S.w * S.w);
    return dot(dir, n) / kPi;
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
__device__ float3 vertex_brdf(const DevScene& sc, const BVert& v, float3 out, bool radiance) {
  if (v.is(kFlagInfinite)) return f3(0.f, 0.f, 0.f);
  if (v.is(kFlagLight) && v.mat < 0) return f3(1.f, 1.f, 1.f);
  if (v.mat < 0) return f3(0.f, 0.f, 0.f);
  Surface s;
  s.p = v.p;
  s.n = v.n;
  s.front = v.is(kFlagFront);
  s.mat = v.mat;
  return brdf(sc, load_material(sc, v.mat), v.wi, out, s, radiance);
}

template <int MAXV>
struct Paths {
  BVert cam[MAXV];
  BVert lgt[MAXV];
  int nc, nl;
};

// extendPath (bdpt.go:206-291)
template <int MAXV>
__device__ void extend_path(const DevScene& sc, BVert* path, int& len, float3 o, float3 d, float3 beta, float pdf_fwd,
                            int max_bounces, bool camera, Rng& rng, uint32_t skip, int* err) {
  for (int b = 0; b < max_bounces && len < MAXV; b++) {
    BVert& prev = path[len - 1];
    Hit h;
    if (!trace<false, false>(sc, o, d, 0.001f, kInfF, skip, h, err)) {
      if (camera) {
        // createBackgroundVertex (bdpt.go:585-601)
        float3 bg = background(sc, d);
        BVert& v = path[len++];
        v.p = o + d * 1000.f;
        v.n = -d;
        v.wi = -d;
        v.fwd = pdf_fwd;
        v.rev = 0.f;
        v.beta = beta;
        v.Le = bg;
        v.mat = -1;
        v.light = -1;
        v.prim = kNoHit;
        v.flags = kFlagInfinite | (is_zero(bg) ? 0 : kFlagLight);
      }
      break;
    }
    Surface s;
    surface_at(sc, o, d, h, s);
    DevMaterial m = load_material(sc, s.mat);
    BVert& v = path[len];
    v.p = s.p;
    v.n = s.n;
    v.wi = -d;
    v.beta = beta;
    v.Le = emitted(m, s.front);
    v.mat = s.mat;
    v.light = -1;
    v.prim = h.prim;
    v.flags = (s.front ? kFlagFront : 0) | (is_zero(v.Le) ? 0 : kFlagLight);
    v.rev = 0.f;
    v.fwd = to_area(sc, prev, v, pdf_fwd);
    Scatter scn;
    if (!scatter(sc, m, d, s, rng, scn)) {
      len++;
      break;
    }
    pdf_fwd = scn.pdf;
    if (scn.pdf <= 0.f) v.flags |= kFlagSpecular;
    float ct = fabsf(dot(scn.dir, s.n));
    if (scn.pdf <= 0.f) beta = beta * scn.att;
    else beta = beta * scn.att * (ct / scn.pdf);
    bool rdelta;
    float pdf_rev = mat_pdf(sc, m, scn.dir, -d, s.n, rdelta);
    if (rdelta) {
      v.flags |= kFlagSpecular;
      pdf_rev = 0.f;
      pdf_fwd = 0.f;
    }
    prev.rev = to_area(sc, v, prev, pdf_rev);
    len++;
    o = s.p;
    d = scn.dir;
    skip = h.prim;
  }
}

// calculateLightPdf (bdpt_mis.go:239-272)
__device__ float vertex_light_pdf(const DevScene& sc, const BVert& cur, const BVert& to) {
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
__device__ float vertex_pdf(const DevScene& sc, const BVert& cur, const BVert* prev, const BVert& next) {
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
__device__ float light_origin_pdf(const DevScene& sc, const BVert& lv, const BVert& to) {
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

__device__ __forceinline__ float remap0(float f) { return f != 0.f ? f : 1.f; }

// calculateMISWeight (bdpt_mis.go:13-181)
template <int MAXV>
__device__ float mis_weight(const DevScene& sc, const Paths<MAXV>& P, const BVert* sampled, int s, int t) {
  if (s + t == 2) return 1.f;
  const BVert* C = P.cam;
  const BVert* Lp = P.lgt;
  float sum = 0.f, ri = 1.f;
  for (int i = t - 1; i > 0; i--) {
    const BVert& v = C[i];
    float fwd = v.fwd, rev = v.rev;
    bool conn = !v.is(kFlagSpecular);
    if (s == 0) {
      if (i == t - 1 && t > 1) {
        rev = light_origin_pdf(sc, C[t - 1], C[t - 2]);
        conn = true;
      } else if (i == t - 2 && t > 2) {
        rev = vertex_pdf(sc, C[t - 1], nullptr, C[t - 2]);
      }
    } else if (t == 1) {
      if (i == 0) {
        fwd = sampled->fwd;
        rev = sampled->rev;
        conn = true;
      }
    } else if (s == 1) {
      if (i == t - 1 && t > 0) {
        rev = vertex_pdf(sc, *sampled, nullptr, C[t - 1]);
        conn = true;
      } else if (i == t - 2 && t > 1) {
        rev = vertex_pdf(sc, C[t - 1], sampled, C[t - 2]);
      }
    } else {
      if (i == t - 1) {
        rev = vertex_pdf(sc, Lp[s - 1], &Lp[s - 2], C[t - 1]);
        conn = true;
      } else if (i == t - 2 && t > 1) {
        rev = vertex_pdf(sc, C[t - 1], &Lp[s - 1], C[t - 2]);
      }
    }
    if (i > 0) conn = conn && !C[i - 1].is(kFlagSpecular);
    ri *= remap0(rev) / remap0(fwd);
    if (conn) sum += ri;
  }
  ri = 1.f;
  for (int i = s - 1; i >= 0; i--) {
    const BVert& v = Lp[i];
    float fwd = v.fwd, rev = v.rev;
    bool conn = !v.is(kFlagSpecular);  // no point lights on this path
    if (i > 0) conn = conn && !Lp[i - 1].is(kFlagSpecular);
    if (t == 1) {
      if (i == s - 1 && s > 1) {
        rev = vertex_pdf(sc, *sampled, nullptr, Lp[s - 1]);
        conn = true;
      } else if (i == s - 2 && s > 1) {
        rev = vertex_pdf(sc, Lp[s - 1], sampled, Lp[s - 2]);
      }
    } else if (s == 1) {
      if (i == s - 1 && sampled) {
        fwd = sampled->fwd;
        rev = vertex_pdf(sc, C[t - 1], &C[t - 2], *sampled);
        conn = true;
      }
    } else {
      if (i == s - 1) {
        rev = vertex_pdf(sc, C[t - 1], &C[t - 2], Lp[s - 1]);
        conn = true;
      } else if (i == s - 2 && s > 1) {
        rev = vertex_pdf(sc, Lp[s - 1], &C[t - 1], Lp[s - 2]);
      }
    }
    ri *= remap0(rev) / remap0(fwd);
    if (conn) sum += ri;
  }
  return 1.f / (1.f + sum);
}

template <int MAXV>
__global__ void __launch_bounds__(128) k_bdpt(DevScene sc, DevFilm film, DevPaths PS, ChunkDesc ch) {
  uint32_t n = ch.npix * ch.layers;
  int* err = reinterpret_cast<int*>(PS.counters + 3);
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    uint32_t layer = p / ch.npix, i = p - layer * ch.npix;
    uint32_t pix = ch.pix_list ? ch.pix_list[ch.pix0 + i] : ch.pix0 + i;
    uint32_t sample = film.count[pix] + layer;
    int x = (int)(pix % (uint32_t)film.width), y = (int)(pix / (uint32_t)film.width);
    // one sequential stream per sample, drawn in the reference's order:
    // GetRay, camera subpath, light subpath, then the strategies
    Rng rng;
    rng.init(ch.seed, pix, sample);
    float2 lens = rng.next2();
    float2 jit = rng.next2();
    float3 o, d;
    camera_ray(sc.cam, x, y, lens, jit, o, d);
    Paths<MAXV> P;
    // generateCameraPath (bdpt.go:106-135)
    {
      BVert& c = P.cam[0];
      c.p = o;
      c.n = -d;
      c.wi = f3(0.f, 0.f, 0.f);
      c.beta = f3(1.f, 1.f, 1.f);
      c.Le = f3(0.f, 0.f, 0.f);
      c.fwd = 0.f;
      c.rev = 0.f;
      c.mat = -1;
      c.light = -1;
      c.prim = kNoHit;
      c.flags = kFlagCamera;
      P.nc = 1;
      float dir_pdf = camera_dir_pdf(sc.cam, o, d);
      extend_path<MAXV>(sc, P.cam, P.nc, o, d, f3(1.f, 1.f, 1.f), dir_pdf, sc.max_depth, true, rng, kNoHit, err);
    }
    // generateLightPath (bdpt.go:139-202)
    P.nl = 0;
    if (sc.n_lights > 0) {
      Rng& rl = rng;
      float ul = rl.next();
      int li = pick_light(sc, ul);
      DevLight L = sc.lights[li];
      float2 sp = rl.next2();
      float2 sd = rl.next2();
      float3 ep, en, ed, Le;
      float apdf, dpdf;
      sample_emission(sc, L, sp, sd, ep, en, ed, Le, apdf, dpdf);
      float ct = fabsf(dot(ed, en));
      BVert& lv = P.lgt[0];
      lv.p = ep;
      lv.n = en;
      lv.wi = f3(0.f, 0.f, 0.f);
      lv.light = li;
      lv.mat = -1;
      lv.prim = L.kind == kLightQuad ? sc.quad_base + (uint32_t)L.prim
                                     : (L.kind == kLightSphere ? sc.sphere_base + (uint32_t)L.prim : kNoHit);
      lv.fwd = apdf * L.prob;
      lv.rev = 0.f;
      bool inf = L.kind == kLightUniformInfinite || L.kind == kLightGradientInfinite;
      lv.flags = kFlagLight | (inf ? kFlagInfinite : 0);
      lv.beta = Le;
      lv.Le = Le;
      P.nl = 1;
      float3 beta = Le * (ct / (L.prob * apdf * dpdf));
      extend_path<MAXV>(sc, P.lgt, P.nl, ep, ed, beta, dpdf, sc.max_depth - 1, false, rl, lv.prim, err);
      if (inf) {
        if (P.nl > 1) {
          BVert& fb = P.lgt[1];
          fb.fwd = apdf * L.prob;
          if (fb.mat >= 0) fb.fwd *= fabsf(dot(ed, fb.n));
        }
        P.lgt[0].fwd = infinite_density(sc, ep, en, ed);
      }
    }
    // all strategies (bdpt.go:83-99)
    float3 total = f3(0.f, 0.f, 0.f);
    Rng& rs = rng;
    for (int s = 0; s <= P.nl; s++) {
      for (int t = 1; t <= P.nc; t++) {
        if (s == 1 && t == 1) continue;
        float3 Lc = f3(0.f, 0.f, 0.f);
        BVert sampled;
        bool has = false;
        bool splat = false;
        int spx = 0, spy = 0;
        if (s == 0) {
          // evaluatePathTracingStrategy (bdpt.go:317-332)
          if (t == P.nc) {
            const BVert& last = P.cam[t - 1];
            Lc = last.Le * last.beta;
          }
        } else if (t == 1) {
          // evaluateLightTracingStrategy (bdpt.go:398-486)
          const BVert& lv = P.lgt[s - 1];
          if (s <= 1 || lv.is(kFlagSpecular)) continue;
          float2 cs = rs.next2();
          float2 lens2 = sample_unit_disk(cs);
          float3 lp = sc.cam.center + sc.cam.u * (lens2.x * sc.cam.lens_radius) + sc.cam.v * (lens2.y * sc.cam.lens_radius);
          float3 toRef = lv.p - lp;
          float dist = length(toRef);
          float3 dir = normalize(toRef);
          float cpdf = (dist * dist) / (fabsf(dot(sc.cam.forward, dir)) * sc.cam.lens_area);
          float imp = camera_importance(sc.cam, dir);
          if (imp == 0.f) continue;  // SampleCameraFromPoint returns nil
          float3 toCam = -dir;
          float3 f = vertex_brdf(sc, lv, toCam, false);
          float cb = imp / cpdf;
          float cosine = dot(toCam, lv.n);
          if (cosine <= 0.f) continue;
          float3 c = f * cb * lv.beta;
          if (on_surface(sc, lv)) c = c * cosine;
          if (is_zero(c)) continue;
          Hit hh;
          if (trace<true, false>(sc, lv.p, toCam, 0.001f, dist - 0.001f, lv.prim, hh, err)) continue;
          if (!map_ray_to_pixel(sc.cam, lp, dir, spx, spy)) continue;
          float lpdf = total_light_pdf(sc, lp, toCam, normalize(lv.p - lp));
          sampled.p = lp;
          sampled.n = toCam;
          sampled.wi = f3(0.f, 0.f, 0.f);
          sampled.beta = f3(cb, cb, cb);
          sampled.Le = f3(0.f, 0.f, 0.f);
          sampled.fwd = cpdf;
          sampled.rev = lpdf;
          sampled.mat = -1;
          sampled.light = -1;
          sampled.prim = kNoHit;
          sampled.flags = kFlagCamera;
          has = true;
          splat = true;
          Lc = c;
        } else if (s == 1) {
          // evaluateDirectLightingStrategy (bdpt.go:334-394)
          const BVert& cv = P.cam[t - 1];
          if (cv.is(kFlagSpecular) || cv.mat < 0) continue;
          if (sc.n_lights == 0) continue;
          int li = pick_light(sc, rs.next());
          DevLight L = sc.lights[li];
          LightSample ls = light_sample(sc, L, cv.p, cv.n, rs.next2());
          ls.pdf *= L.prob;
          if (is_zero(ls.emission) || ls.pdf <= 0.f) continue;
          float ct = fabsf(dot(ls.dir, cv.n));
          if (ct <= 0.f) continue;
          float3 f = vertex_brdf(sc, cv, ls.dir, true);
          float3 lb = ls.emission * (1.f / ls.pdf);
          float3 c = f * cv.beta * lb * ct;
          if (is_zero(c)) continue;
          Hit hh;
          if (trace<true, false>(sc, cv.p, ls.dir, 0.001f, ls.dist - 0.001f, cv.prim, hh, err)) continue;
          sampled.p = ls.point;
          sampled.n = ls.normal;
          sampled.wi = f3(0.f, 0.f, 0.f);
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
          const BVert& lv = P.lgt[s - 1];
          const BVert& cv = P.cam[t - 1];
          if (lv.is(kFlagSpecular) || cv.is(kFlagSpecular)) continue;
          float3 dd = lv.p - cv.p;
          float dist = length(dd);
          if (dist < 0.001f) continue;
          dd = dd * (1.f / dist);
          float cc = dot(dd, cv.n), cl = dot(-dd, lv.n);
          if (cc <= 0.f || cl <= 0.f) continue;
          float g = (cc * cl) / (dist * dist);
          float3 cb = vertex_brdf(sc, cv, dd, true);
          float3 lb = vertex_brdf(sc, lv, -dd, false);
          float3 c = lv.beta * lb * cb * cv.beta * g;
          if (is_zero(c)) continue;
          Hit hh;
          if (trace<true, false>(sc, cv.p, dd, 0.001f, dist - 0.001f, cv.prim, hh, err)) continue;
          Lc = c;
        }
        if (is_zero(Lc) && !splat) continue;
        float w = mis_weight<MAXV>(sc, P, has ? &sampled : nullptr, s, t);
        if (splat) {
          float3 c = Lc * w;
          float4* dst = film.splat + (size_t)spy * film.width + spx;
          atomicAdd(&dst->x, c.x);
          atomicAdd(&dst->y, c.y);
          atomicAdd(&dst->z, c.z);
        } else {
          total += Lc * w;
        }
      }
    }
    PS.Lout[p] = make_float4(total.x, total.y, total.z, 0.f);
  }
}

}  // namespace

void launch_bdpt(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                 cudaStream_t st) {
  uint32_t n = ch.npix * ch.layers;
  (void)block;
  int grid = launch_grid(n, 128, 0);
  if (sc.max_depth <= 9) k_bdpt<10><<<grid, 128, 0, st>>>(sc, film, P, ch);
  else k_bdpt<18><<<grid, 128, 0, st>>>(sc, film, P, ch);
}

}  // namespace gprt
