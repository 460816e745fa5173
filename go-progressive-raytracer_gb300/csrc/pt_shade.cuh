// pt_shade.cuh - one level of the path tracer for one path, shared by the
// single-job wavefront (kernels_pt.cu) and the multi-job serving wavefront
// (server.cu).
#pragma once

#include "device.cuh"
#include "kernels.h"

namespace gprt {

// The state a shading step leaves: the continuing path (when `cont`).  Its
// shadow ray is queued as soon as next-event estimation produces it.
struct ShadeOut {
  bool cont;
  float4 o, d, w;  // next ray origin (+ skip prim), direction (+ BVH root), weight (+ origin index)
  float3 thr, L;
  uint4 ids;
};

// One level of rayColorRecursive (pkg/integrator/path_tracing.go:35-104) with
// CalculateDirectLighting (:116-157), CalculateIndirectLighting (:160-189)
// and ApplyRussianRoulette (:193-220), for slot i of queue Q at depth index
// `bounce` (= MaxDepth - depth).  The Russian-roulette draw happens first at
// every level, as in the reference.  The shadow ray of next-event estimation
// goes to P's shadow queue at once (its contribution, when unoccluded, is
// added to the path's radiance at its origin index), so its state is not
// held to the end of the step.
__device__ __forceinline__ void shade_path(const DevScene& sc, const DevPaths& P, const PathBuf& Q,
                                           const float4* hits, uint32_t i, uint64_t seed, int bounce, ShadeOut& out) {
  out.cont = false;
  float4 o4 = Q.ray_o[i], d4 = Q.ray_d[i], h4 = hits[i];
  uint4 ids = Q.ids[i];
  float3 d = f3(d4);
  // at bounce 0 the path state raygen implies (not stored): weight 1, origin
  // index = the slot, roulette throughput 1, radiance 0
  float4 w4 = make_float4(1.f, 1.f, 1.f, __uint_as_float(i));
  float3 thr = f3(1.f, 1.f, 1.f), L = f3(0.f, 0.f, 0.f);
  if (bounce > 0) {
    w4 = Q.weight[i];
    thr = f3(Q.thr[i]);
    L = f3(Q.L[i]);
  }
  float3 W = f3(w4);
  out.o = o4;
  out.d = d4;
  Rng rng;
  rng.init(seed, ids.x, ids.y, ids.z);
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
      L += W * emitted(m, s.front, d);  // getEmittedLight (:108-113)
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
                if (!is_zero(c)) {  // one warp-aggregated append among the lanes here
                  uint32_t ss = warp_append(&P.counters[2], true);
                  P.sh_o[ss] = make_float4(s.p.x, s.p.y, s.p.z, ls.dist - 0.001f);
                  P.sh_d[ss] = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, __uint_as_float(prim));
                  P.sh_c[ss] = make_float4(c.x, c.y, c.z, w4.w);  // w4.w: the origin index
                  if (P.sh_root) P.sh_root[ss] = __float_as_int(d4.w);
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
          out.o = make_float4(s.p.x, s.p.y, s.p.z, __uint_as_float(prim));
          out.d = make_float4(sc_.dir.x, sc_.dir.y, sc_.dir.z, d4.w);
        }
      }
    }
  }
  out.cont = cont && (bounce + 1 < sc.max_depth);
  out.L = L;
  out.w = make_float4(W.x, W.y, W.z, w4.w);
  out.thr = thr;
  out.ids = make_uint4(ids.x, ids.y, rng.pos, ids.w);
}

// Brings the shading inputs of slot i of queue Q (ray, hit, ids and, after
// bounce 0 (`state`), weight, roulette throughput and radiance) into L2
// ahead of their use: a grid-stride shading loop issues this for its next
// slot at the end of the current one, so the next iteration's dependent
// loads meet L2 instead of DRAM.
__device__ __forceinline__ void prefetch_slot(const PathBuf& Q, const float4* hits, uint32_t i, bool state) {
  const void* a[7] = {Q.ray_o + i, Q.ray_d + i, hits + i, Q.ids + i, Q.weight + i, Q.thr + i, Q.L + i};
  const int m = state ? 7 : 4;
  for (int k = 0; k < m; k++) asm volatile("prefetch.global.L2 [%0];" ::"l"(a[k]));
}

// The shading group of primitive p, stored in its record by the builders.
__device__ __forceinline__ int prim_group(const DevScene& sc, uint32_t p) {
  if (p < sc.quad_base) return __float_as_int(__ldg(sc.tris + (size_t)p * 3 + 1).w);
  if (p < sc.sphere_base) return __float_as_int(__ldg(sc.quads + (size_t)(p - sc.quad_base) * 5 + 2).w);
  if (p < sc.quadric_base) return __float_as_int(__ldg(sc.spheres + (size_t)(p - sc.sphere_base) * 2 + 1).y);
  return __float_as_int(__ldg(sc.quadrics + (size_t)(p - sc.quadric_base) * 5 + 4).w);
}

// The slot order the shading kernels read for queue `cur`, by shading group
// (`group(i, prim)` for slot i's hit on primitive prim; missed rays, which
// only look up the background, are group 3): group 0 from the front, then,
// from the back, groups 1, 2 and 3.  Each block of 1,024 slots takes one
// range from the front and one from the back (one atomic each) and lays its
// back range out group by group, so warps run one kind of shading (next-event
// estimation on all lanes or on none; metal, glass or finished paths) instead
// of mixing them lane by lane.  Every path is shaded exactly as in queue
// order.
template <class Group>
__device__ __forceinline__ void order_slots(const DevPaths& P, int cur, Group group) {
  constexpr int G = kShadeGroups;
  __shared__ uint32_t wc[G][32];
  __shared__ uint32_t bfront, bback, boff[G];
  const uint32_t n = P.counters[cur];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  for (uint32_t base = blockIdx.x * 1024u; base < n; base += gridDim.x * 1024u) {
    uint32_t i = base + threadIdx.x;
    bool live = i < n;
    uint32_t prim = live ? __float_as_uint(P.hit[i].y) : kNoHit;
    int g = prim != kNoHit && prim != kOverflowHit ? group(i, prim) : G - 1;
    unsigned mine = 0;  // the lanes of this warp in group g
#pragma unroll
    for (int k = 0; k < G; k++) {
      unsigned m = __ballot_sync(0xffffffffu, live && g == k);
      if (g == k) mine = m;
      if (lane == 0) wc[k][w] = __popc(m);
    }
    __syncthreads();
    if (threadIdx.x < G) {  // exclusive scan of each group's warp counts
      uint32_t acc = 0;
      for (int k = 0; k < 32; k++) {
        uint32_t c = wc[threadIdx.x][k];
        wc[threadIdx.x][k] = acc;
        acc += c;
      }
      boff[threadIdx.x] = acc;  // the group's total, for now
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      // back-range entry j sits at n - 1 - (bback + j): the last group takes
      // the smallest j (the highest positions), group 1 the largest
      uint32_t back = 0;
      for (int k = G - 1; k >= 1; k--) {
        uint32_t t = boff[k];
        boff[k] = back;
        back += t;
      }
      bfront = boff[0] ? atomicAdd(&P.counters[6], boff[0]) : 0u;
      bback = back ? atomicAdd(&P.counters[7], back) : 0u;
    }
    __syncthreads();
    if (live) {
      uint32_t r = wc[g][w] + __popc(mine & below);
      if (g == 0) P.order[bfront + r] = i;
      else P.order[n - 1u - (bback + boff[g] + r)] = i;
    }
    __syncthreads();  // the counts and bases are rewritten for the next range
  }
}

// Moves a continuing path to the next queue; a finished path adds its
// radiance at its origin index (where its unoccluded shadow rays add
// theirs; raygen clears it).  Called by every lane of the warp; `live` is
// false for lanes without a path.
__device__ __forceinline__ void push_shade_out(const DevPaths& P, int cur, bool live, const ShadeOut& o) {
  bool cont = live && o.cont;
  uint32_t slot = warp_append(&P.counters[cur ^ 1], cont);
  if (cont) {
    const PathBuf& N = P.q[cur ^ 1];
    N.ray_o[slot] = o.o;
    N.ray_d[slot] = o.d;
    N.weight[slot] = o.w;
    N.thr[slot] = make_float4(o.thr.x, o.thr.y, o.thr.z, 0.f);
    N.L[slot] = make_float4(o.L.x, o.L.y, o.L.z, 0.f);
    N.ids[slot] = o.ids;
  } else if (live) {
    float4* dst = P.Lout + __float_as_uint(o.w.w);
    float4 a = *dst;
    *dst = make_float4(a.x + o.L.x, a.y + o.L.y, a.z + o.L.z, 0.f);
  }
}

}  // namespace gprt
