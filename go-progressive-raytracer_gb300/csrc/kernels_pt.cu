// kernels_pt.cu - raw ray batches and the wavefront path tracer.
//
// The reference's PathTracingIntegrator.rayColorRecursive
// (pkg/integrator/path_tracing.go:35-104) recurses once per bounce and
// returns emitted + direct + indirect radiance, every level scaled by its
// Russian-roulette compensation, and the indirect term scaled by the BSDF
// MIS weight.  Unrolled, the radiance of a sample is a sum over bounces of
//     W_k * (Le_k + Ld_k)
// where W_k is the product of the per-level factors of the levels above:
// rr compensation, and attenuation (specular) or attenuation*cos*w_bsdf/pdf
// (diffuse).  The wavefront keeps W_k, the Russian-roulette throughput and
// the gathered radiance per path and advances all paths one bounce per
// kernel sequence:  extend (closest hit) -> shade -> shadow (any hit).
#include <algorithm>

#include "device.cuh"
#include "kernels.h"
#include "pt_shade.cuh"

namespace gprt {

int launch_grid(uint32_t n, int block, int max_blocks) {
  uint32_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (max_blocks > 0 && g > (uint32_t)max_blocks) g = (uint32_t)max_blocks;
  return (int)g;
}

// ----------------------------------------------------------------- raw batches
struct BatchSource {
  const gprt_ray* rays;
  gprt_hit* hits;
  uint32_t n;
  __device__ uint32_t count() const { return n; }
  int root;
  int* err;
  __device__ void load(uint32_t i, float3& o, float3& d, float& tmin, float& tmax, uint32_t& skip, int& rt) const {
    rt = root;
    const float4* r = reinterpret_cast<const float4*>(rays + i);
    float4 a = __ldg(r), b = __ldg(r + 1);
    o = f3(a);
    d = f3(b);
    tmin = a.w;
    tmax = b.w;
    skip = kNoHit;
  }
  __device__ void store(uint32_t i, const Hit& h) const {
    bool over = h.prim == kOverflowHit;
    if (over) atomicOr(err, kErrStackOverflow);
    bool any = h.prim != kNoHit && !over;
    reinterpret_cast<float4*>(hits)[i] =
        make_float4(any ? h.t : -1.f, __uint_as_float(any || over ? h.prim : kNoHit), any ? h.u : 0.f,
                    any ? h.v : 0.f);
  }
};

// Batches use static per-warp ranges: calls on different streams share no counter.
template <bool kAny>
__global__ void __launch_bounds__(128, 8) k_intersect(DevScene sc, BatchSource src) {
  trace_persistent<kAny, false>(sc, src, nullptr, nullptr, nullptr);
}

int persistent_grid(int sm_count, int block) { return std::max(1, sm_count * (1024 / block)); }

void launch_intersect(const DevScene& sc, const gprt_ray* rays, uint32_t n, bool any_hit, gprt_hit* hits, int* err,
                      cudaStream_t st) {
  if (n == 0) return;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = launch_grid((n + 31) / 32 * 32, 128, persistent_grid(sms, 128));
  BatchSource src{rays, hits, n, sc.root, err};
  if (any_hit) k_intersect<true><<<grid, 128, 0, st>>>(sc, src);
  else k_intersect<false><<<grid, 128, 0, st>>>(sc, src);
}

// ----------------------------------------------------------------- raygen
// TileRenderer sample loop + Camera.GetRay (tile_renderer.go:55-59,
// camera.go:173-190): path p of the chunk is sample `layer` of pixel i.
__global__ void k_pt_raygen(DevScene sc, DevFilm film, DevPaths P, ChunkDesc ch) {
  uint32_t n = ch.npix * ch.layers;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    uint32_t layer = p / ch.npix, i = p - layer * ch.npix;
    uint32_t pix = ch.pix_list ? ch.pix_list[ch.pix0 + i] : ch.pix0 + i;
    uint32_t sample = film.count[pix] + layer;
    int x = (int)(pix % (uint32_t)film.width), y = (int)(pix / (uint32_t)film.width);
    Rng rng;
    rng.init(ch.seed, pix, sample);
    // Camera.GetRay(i, j, sampler.Get2D(), sampler.Get2D()) (tile_renderer.go:56)
    float2 lens = rng.next2();
    float2 jit = rng.next2();
    float3 o, d;
    camera_ray(sc.cam, x, y, lens, jit, o, d);
    const PathBuf& Q = P.q[0];
    Q.ray_o[p] = make_float4(o.x, o.y, o.z, __uint_as_float(kNoHit));
    Q.ray_d[p] = make_float4(d.x, d.y, d.z, __int_as_float(sc.root));
    // weight 1 with origin index p, roulette throughput 1 and radiance 0 are
    // implied at bounce 0 (not stored)
    Q.ids[p] = make_uint4(pix, sample, rng.pos, 0u);
    P.Lout[p] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.counters[0] = n;
    P.counters[4] = 0;  // ray-fetch counters of the first extend and shadow launches
    P.counters[5] = 0;
  }
}

void launch_pt_raygen(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                      cudaStream_t st) {
  uint32_t n = ch.npix * ch.layers;
  k_pt_raygen<<<launch_grid(n, block, 0), block, 0, st>>>(sc, film, P, ch);
}

// ----------------------------------------------------------------- extend
// scene.BVH.Hit(ray, 0.001, +Inf) for every live path (path_tracing.go:67)

// Adds one thread's traversal work to the job's counters (one atomic per warp).
__device__ __forceinline__ void add_counts(unsigned long long* dst, uint32_t rays, const TraceStats& s) {
  unsigned long long v[4] = {rays, s.nodes, s.boxes, s.prims};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    unsigned long long x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(dst + k, x);
  }
}

// The rays of the current queue; built on the host and passed as a kernel
// argument, so its pointers stay in the constant bank.
struct ExtendSource {
  const float4* ray_o;
  const float4* ray_d;
  float4* hit;
  const uint32_t* n;
  const float4* weight;  // origin index of each path (.w), read when reporting a bound; null at bounce 0 (slot = origin)
  ErrSink err;
  __device__ uint32_t count() const { return *n; }
  __device__ void load(uint32_t i, float3& o, float3& d, float& tmin, float& tmax, uint32_t& skip, int& rt) const {
    float4 a = ray_o[i], b = ray_d[i];
    rt = __float_as_int(b.w);
    o = f3(a);
    d = f3(b);
    tmin = 0.001f;
    tmax = kInfF;
    skip = __float_as_uint(a.w);
  }
  // the marker hit of a stack overflow is stored as a miss and fails the
  // path's job
  __device__ void store(uint32_t i, const Hit& h) const {
    bool any = h.prim != kNoHit;
    if (h.prim == kOverflowHit) {
      err.report(weight ? __float_as_uint(weight[i].w) : i, kErrStackOverflow);
      any = false;
    }
    hit[i] = make_float4(any ? h.t : -1.f, __uint_as_float(any ? h.prim : kNoHit), h.u, h.v);
  }
};

// The error sink of a wavefront's paths (per job, or per item of a multi-job step).
static ErrSink err_sink(const DevPaths& P) { return ErrSink{P.counters + 3, P.item_err, P.item_start, P.n_items}; }

template <bool kCount>
__global__ void __launch_bounds__(128, 8)
    k_pt_extend(DevScene sc, ExtendSource src, uint32_t* counters, int cur, unsigned long long* stats) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    counters[cur ^ 1] = 0;  // next queue and shadow queue start empty
    counters[2] = 0;
    counters[6] = 0;  // hit / miss counts of the slot order built after this launch
    counters[7] = 0;
  }
  TraceStats ts{0, 0, 0};
  uint32_t rays = 0;
  trace_persistent<false, kCount>(sc, src, counters + 4, &ts, &rays);
  if (kCount) add_counts(stats, rays, ts);
}

// One ray per thread (grid-stride), the variant GPRT_JOB_SIMPLE_EXTEND selects.
template <bool kCount>
__global__ void __launch_bounds__(256)
    k_pt_extend_simple(DevScene sc, ExtendSource src, uint32_t* counters, int cur, unsigned long long* stats) {
  uint32_t n = src.count();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    counters[cur ^ 1] = 0;
    counters[2] = 0;
    counters[6] = 0;
    counters[7] = 0;
  }
  TraceStats ts{0, 0, 0};
  uint32_t rays = 0;
  uint32_t end = kCount ? ((n + 31) & ~31u) : n;  // whole warps stay for the count reduction
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
    if (i < n) {
      float3 o, d;
      float tmin, tmax;
      uint32_t skip;
      int root;
      src.load(i, o, d, tmin, tmax, skip, root);
      Hit h;
      trace_from<false, kCount>(sc, root, o, d, tmin, tmax, skip, h, nullptr, &ts);
      src.store(i, h);
      rays++;
    }
  }
  if (kCount) add_counts(stats, rays, ts);
}

static int sm_count_current() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

void launch_pt_extend(const DevScene& sc, const DevPaths& P, int cur, int bounce, int block, int grid, cudaStream_t st) {
  ExtendSource src{P.q[cur].ray_o, P.q[cur].ray_d, P.hit, P.counters + cur, bounce > 0 ? P.q[cur].weight : nullptr,
                   err_sink(P)};
  if (P.variant & GPRT_JOB_SIMPLE_EXTEND) {
    int b = std::min(block, 256);
    if (P.stats) k_pt_extend_simple<true><<<grid, b, 0, st>>>(sc, src, P.counters, cur, P.stats);
    else k_pt_extend_simple<false><<<grid, b, 0, st>>>(sc, src, P.counters, cur, P.stats);
    return;
  }
  int g = persistent_grid(sm_count_current(), 128);
  if (P.stats) k_pt_extend<true><<<g, 128, 0, st>>>(sc, src, P.counters, cur, P.stats);
  else k_pt_extend<false><<<g, 128, 0, st>>>(sc, src, P.counters, cur, P.stats);
}

// ----------------------------------------------------------------- shade
// The shading order of queue `cur` (order_slots) for one scene.
__global__ void __launch_bounds__(1024) k_hit_order(DevScene sc, DevPaths P, int cur) {
  order_slots(P, cur, [&](uint32_t, uint32_t prim) { return prim_group(sc, prim); });
}

void launch_hit_order(const DevScene& sc, const DevPaths& P, int cur, uint32_t cap, int sms, cudaStream_t st) {
  if (!P.order) return;
  int g = std::max(1, std::min((int)((cap + 1023) / 1024), sms * 2));
  k_hit_order<<<g, 1024, 0, st>>>(sc, P, cur);
}

// One level of rayColorRecursive (path_tracing.go:35-104) with
// CalculateDirectLighting (:116-157), CalculateIndirectLighting (:160-189)
// and ApplyRussianRoulette (:193-220).  The Russian-roulette draw happens
// first at every level, as in the reference.
template <int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    k_pt_shade(DevScene sc, DevPaths P, ChunkDesc ch, int cur, int bounce) {
  uint32_t n = P.counters[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.counters[4] = 0;  // ray-fetch counters of the next shadow and extend launches
    P.counters[5] = 0;
  }
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t slot = first < n ? (P.order ? P.order[first] : first) : 0u;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    uint32_t i = base + threadIdx.x;
    // the slot of the next iteration, read now and prefetched into L2 after this one
    uint32_t inext = i + stride;
    uint32_t snext = inext < n ? (P.order ? P.order[inext] : inext) : 0u;
    ShadeOut o;
    o.cont = false;
    bool live = i < n;
    if (live) shade_path(sc, P, P.q[cur], P.hit, slot, ch.seed, bounce, o);
    push_shade_out(P, cur, live, o);
    if (inext < n) prefetch_slot(P.q[cur], P.hit, snext, bounce > 0);
    slot = snext;
  }
}

void launch_pt_shade(const DevScene& sc, const DevPaths& P, const ChunkDesc& ch, int cur, int bounce, int block,
                     int grid, cudaStream_t st) {
  // the shading-group slot order pays where rays escape to an infinite
  // light (missed rays are then a large share) or where specular and
  // diffuse materials mix; in closed all-diffuse scenes it is overhead
  DevPaths Po = P;
  if (sc.has_infinite || sc.has_specular) launch_hit_order(sc, P, cur, P.capacity, sm_count_current(), st);
  else Po.order = nullptr;
  if (P.variant & GPRT_JOB_SHADE_OCCUPANCY) {
    int g = std::max(1, (int)((int64_t)grid * block / 192));
    k_pt_shade<192, 3><<<g, 192, 0, st>>>(sc, Po, ch, cur, bounce);
  } else {
    k_pt_shade<256, 2><<<grid, std::min(block, 256), 0, st>>>(sc, Po, ch, cur, bounce);
  }
}

// ----------------------------------------------------------------- shadow
// scene.BVH.Hit(shadowRay, 0.001, distance - 0.001) used as a boolean
// (path_tracing.go:143-148): the contribution is kept when nothing is hit.
struct ShadowSource {
  const float4* sh_o;
  const float4* sh_d;
  const float4* sh_c;
  const int* sh_root;  // null: every ray starts at `root`
  float4* Lout;        // radiance of the paths, by origin index
  const uint32_t* n;
  int root;
  ErrSink err;
  __device__ uint32_t count() const { return *n; }
  __device__ void load(uint32_t i, float3& o, float3& d, float& tmin, float& tmax, uint32_t& skip, int& rt) const {
    rt = sh_root ? sh_root[i] : root;
    float4 a = sh_o[i], b = sh_d[i];
    o = f3(a);
    d = f3(b);
    tmin = 0.001f;
    tmax = a.w;
    skip = __float_as_uint(b.w);
  }
  // one shadow ray per path and bounce: the read-modify-write of its origin
  // slot meets no other ray of the launch
  __device__ void store(uint32_t i, const Hit& h) const {
    if (h.prim == kOverflowHit) {  // the visibility is unknown: fail the path's job
      err.report(__float_as_uint(sh_c[i].w), kErrStackOverflow);
      return;
    }
    if (h.prim != kNoHit) return;  // occluded
    float4 c = sh_c[i];
    float4* dst = Lout + __float_as_uint(c.w);
    float4 L = *dst;
    *dst = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.f);
  }
};

template <bool kCount>
__global__ void __launch_bounds__(128, 8)
    k_pt_shadow(DevScene sc, ShadowSource src, uint32_t* counters, unsigned long long* stats) {
  TraceStats ts{0, 0, 0};
  uint32_t rays = 0;
  trace_persistent<true, kCount>(sc, src, counters + 5, &ts, &rays);
  if (kCount) add_counts(stats + 4, rays, ts);
}

// One shadow ray per thread (grid-stride), the variant GPRT_JOB_SIMPLE_SHADOW selects.
template <bool kCount>
__global__ void __launch_bounds__(256)
    k_pt_shadow_simple(DevScene sc, ShadowSource src, uint32_t* counters, unsigned long long* stats) {
  uint32_t n = src.count();
  TraceStats ts{0, 0, 0};
  uint32_t rays = 0;
  uint32_t end = kCount ? ((n + 31) & ~31u) : n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
    if (i < n) {
      float3 o, d;
      float tmin, tmax;
      uint32_t skip;
      int root;
      src.load(i, o, d, tmin, tmax, skip, root);
      Hit h;
      trace_from<true, kCount>(sc, root, o, d, tmin, tmax, skip, h, nullptr, &ts);
      src.store(i, h);
      rays++;
    }
  }
  if (kCount) add_counts(stats + 4, rays, ts);
}

void launch_pt_shadow(const DevScene& sc, const DevPaths& P, int cur, int block, int grid, cudaStream_t st) {
  ShadowSource src{P.sh_o, P.sh_d, P.sh_c, P.sh_root, P.Lout, P.counters + 2, sc.root, err_sink(P)};
  if (P.variant & GPRT_JOB_SIMPLE_SHADOW) {
    int b = std::min(block, 256);
    if (P.stats) k_pt_shadow_simple<true><<<grid, b, 0, st>>>(sc, src, P.counters, P.stats);
    else k_pt_shadow_simple<false><<<grid, b, 0, st>>>(sc, src, P.counters, P.stats);
    return;
  }
  int g = persistent_grid(sm_count_current(), 128);
  if (P.stats) k_pt_shadow<true><<<g, 128, 0, st>>>(sc, src, P.counters, P.stats);
  else k_pt_shadow<false><<<g, 128, 0, st>>>(sc, src, P.counters, P.stats);
}

// ----------------------------------------------------------------- accumulate
// PixelStats.AddSample (pkg/renderer/stats.go:41-47), in sample order per pixel
__global__ void k_accumulate(DevFilm film, DevPaths P, ChunkDesc ch) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ch.npix; i += gridDim.x * blockDim.x) {
    uint32_t pix = ch.pix_list ? ch.pix_list[ch.pix0 + i] : ch.pix0 + i;
    float4 acc = film.rgbl[pix];
    float l2 = film.lum2[pix];
    for (uint32_t layer = 0; layer < ch.layers; layer++) {
      float4 c = P.Lout[layer * ch.npix + i];
      float lum = luminance(f3(c));
      acc.x += c.x;
      acc.y += c.y;
      acc.z += c.z;
      acc.w += lum;
      l2 += lum * lum;
    }
    film.rgbl[pix] = acc;
    film.lum2[pix] = l2;
    film.count[pix] += ch.layers;
  }
}

void launch_accumulate(const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block, cudaStream_t st) {
  k_accumulate<<<launch_grid(ch.npix, block, 0), block, 0, st>>>(film, P, ch);
}

}  // namespace gprt

namespace gprt {

void carve_paths(unsigned char* base, uint32_t cap, bool multi, DevPaths& P) {
  size_t f4 = align256((size_t)cap * sizeof(float4)), u4 = align256((size_t)cap * sizeof(uint4));
  unsigned char* p = base;
  auto take = [&](size_t n) {
    unsigned char* r = p;
    p += n;
    return r;
  };
  P.counters = reinterpret_cast<uint32_t*>(take(256));
  for (int k = 0; k < 2; k++) {
    PathBuf& Q = P.q[k];
    Q.ray_o = reinterpret_cast<float4*>(take(f4));
    Q.ray_d = reinterpret_cast<float4*>(take(f4));
    Q.weight = reinterpret_cast<float4*>(take(f4));
    Q.thr = reinterpret_cast<float4*>(take(f4));
    Q.L = reinterpret_cast<float4*>(take(f4));
    Q.ids = reinterpret_cast<uint4*>(take(u4));
  }
  P.hit = reinterpret_cast<float4*>(take(f4));
  P.Lout = reinterpret_cast<float4*>(take(f4));
  P.sh_o = reinterpret_cast<float4*>(take(f4));
  P.sh_d = reinterpret_cast<float4*>(take(f4));
  P.sh_c = reinterpret_cast<float4*>(take(f4));
  P.sh_root = multi ? reinterpret_cast<int*>(take(align256((size_t)cap * sizeof(int)))) : nullptr;
  P.order = reinterpret_cast<uint32_t*>(take(align256((size_t)cap * sizeof(uint32_t))));
  P.capacity = cap;
}

}  // namespace gprt
