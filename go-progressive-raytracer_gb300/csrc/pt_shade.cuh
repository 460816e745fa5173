// pt_shade.cuh - one level of the path tracer for one path, shared by the
// single-job wavefront (kernels_pt.cu) and the multi-job serving wavefront
// (server.cu).
#pragma once

#include "device.cuh"
#include "kernels.h"

namespace gprt {

// What one shading step asks of the queues: continue the path, and/or trace
// a shadow ray whose contribution is added when it is unoccluded.
struct ShadeOut {
  bool cont, shadow;
  float3 sh_o, sh_d, sh_c;
  float sh_t;
  uint32_t sh_skip;
  int root;  // BVH root of the path's scene
};

// One level of rayColorRecursive (pkg/integrator/path_tracing.go:35-104) with
// CalculateDirectLighting (:116-157), CalculateIndirectLighting (:160-189)
// and ApplyRussianRoulette (:193-220), for path p at depth index `bounce`
// (= MaxDepth - depth).  The Russian-roulette draw happens first at every
// level, as in the reference.  Updates the path's radiance, weights, ray and
// sampler position in P.
__device__ __forceinline__ void shade_path(const DevScene& sc, const DevPaths& P, uint32_t p, uint64_t seed,
                                           int bounce, ShadeOut& out) {
  out.cont = false;
  out.shadow = false;
  out.sh_skip = kNoHit;
  out.sh_t = 0.f;
  float4 o4 = P.ray_o[p], d4 = P.ray_d[p], h4 = P.hit[p];
  float3 d = f3(d4);
  out.root = __float_as_int(d4.w);
  float3 W = f3(P.weight[p]), thr = f3(P.thr[p]), L = f3(P.L[p]);
  Rng rng;
  rng.init(seed, P.pixel[p], P.sample[p], P.rng_pos[p]);
  // ApplyRussianRoulette: currentBounce = MaxDepth - depth = bounce
  float u = rng.next();
  bool dead = false;
  if (bounce >= sc.rr_min_bounces) {
    float surv = fminf(0.95f, fmaxf(0.5f, luminance(thr)));
    if (u > surv) dead = true;
    else W *= 1.0f / surv;
  }
  bool cont = false;
  if (!dead) {
    uint32_t prim = __float_as_uint(h4.y);
    if (prim == kNoHit) {
      L += W * background(sc, d);  // infinite-light emission of a missed ray
    } else {
      Hit h{h4.x, prim, h4.z, h4.w};
      Surface s;
      surface_at(sc, f3(o4), d, h, s);
      DevMaterial m = load_material(sc, s.mat);
      L += W * emitted(m, s.front);  // getEmittedLight (:108-113)
      Scatter sc_;
      if (scatter(sc, m, d, s, rng, sc_)) {
        if (sc_.pdf <= 0.f) {
          // calculateSpecularColor (:88-97)
          W *= sc_.att;
          thr *= sc_.att;
          cont = true;
        } else {
          // CalculateDirectLighting: light choice + light sample
          if (sc.n_lights > 0) {
            int li = pick_light(sc, rng.next());
            DevLight Lt = sc.lights[li];
            LightSample ls = light_sample(sc, Lt, s.p, s.n, rng.next2());
            ls.pdf *= Lt.prob;
            if (luminance(ls.emission) > 0.f && ls.pdf > 0.f) {
              float cosine = dot(ls.dir, s.n);
              bool delta;
              float mp = mat_pdf(sc, m, d, ls.dir, s.n, delta);
              if (cosine > 0.f && !delta) {
                float w = power_heuristic(ls.pdf, mp);
                float3 f = brdf(sc, m, d, ls.dir, s, true);
                float3 c = W * (f * ls.emission) * (cosine * w / ls.pdf);
                if (!is_zero(c)) {
                  out.shadow = true;
                  out.sh_o = s.p;
                  out.sh_d = ls.dir;
                  out.sh_t = ls.dist - 0.001f;
                  out.sh_c = c;
                  out.sh_skip = prim;
                }
              }
            }
          }
          // CalculateIndirectLighting
          float3 sd = normalize(sc_.dir);
          float cosine = dot(sd, s.n);
          if (cosine > 0.f) {
            float lp = total_light_pdf(sc, s.p, s.n, sd);
            float w = power_heuristic(sc_.pdf, lp);
            W *= sc_.att * (cosine * w / sc_.pdf);
            thr *= sc_.att * (cosine / sc_.pdf);
            cont = true;
          }
        }
        if (cont) {
          P.ray_o[p] = make_float4(s.p.x, s.p.y, s.p.z, __uint_as_float(prim));
          P.ray_d[p] = make_float4(sc_.dir.x, sc_.dir.y, sc_.dir.z, d4.w);
        }
      }
    }
  }
  cont = cont && (bounce + 1 < sc.max_depth);
  P.L[p] = make_float4(L.x, L.y, L.z, 0.f);
  P.rng_pos[p] = rng.pos;
  if (cont) {
    P.weight[p] = make_float4(W.x, W.y, W.z, 0.f);
    P.thr[p] = make_float4(thr.x, thr.y, thr.z, 0.f);
  }
  out.cont = cont;
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

// Queues the continuation of path p and its shadow ray.
__device__ __forceinline__ void push_shade_out(const DevPaths& P, int cur, uint32_t p, const ShadeOut& o) {
  uint32_t slot = warp_append(&P.counters[cur ^ 1], o.cont);
  if (o.cont) P.queue[cur ^ 1][slot] = p;
  uint32_t ss = warp_append(&P.counters[2], o.shadow);
  if (o.shadow) {
    P.sh_o[ss] = make_float4(o.sh_o.x, o.sh_o.y, o.sh_o.z, o.sh_t);
    P.sh_d[ss] = make_float4(o.sh_d.x, o.sh_d.y, o.sh_d.z, __uint_as_float(o.sh_skip));
    P.sh_c[ss] = make_float4(o.sh_c.x, o.sh_c.y, o.sh_c.z, __uint_as_float(p));
    if (P.sh_root) P.sh_root[ss] = o.root;
  }
}

}  // namespace gprt
