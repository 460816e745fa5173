// kernels.h - host-callable launchers of the device kernels
#pragma once

#include <cuda_runtime.h>

#include "../../include/gprt.h"
#include "layout.h"

namespace gprt {

// Film of one job: renderer.PixelStats per pixel (pkg/renderer/stats.go:20-51)
struct DevFilm {
  float4* rgbl;    // ColorAccum.xyz, LuminanceAccum
  float* lum2;     // LuminanceSqAccum
  uint32_t* count; // SampleCount
  float4* splat;   // BDPT t=1 splats of the current pass (xyz)
  int width, height;
};

// Wavefront path state (structure of arrays, capacity = paths per chunk)
struct DevPaths {
  float4* ray_o;   // origin.xyz, skip primitive (as int bits)
  float4* ray_d;   // direction.xyz, BVH root node of the path's scene (as int bits)
  float4* weight;  // radiance weight (rgb)
  float4* thr;     // Russian-roulette throughput (rgb)
  float4* L;       // radiance gathered so far (rgb)
  float4* hit;     // t, prim, u, v
  uint32_t* pixel;
  uint32_t* sample;
  uint32_t* rng_pos;  // uniform numbers consumed so far by the path's sample
  uint32_t* queue[2];
  float4* sh_o;    // shadow ray origin.xyz, tmax
  float4* sh_d;    // shadow ray direction.xyz, skip primitive
  float4* sh_c;    // contribution rgb, path index (int bits)
  int* sh_root;    // BVH root of each shadow ray (multi-scene wavefronts; null: the scene's root)
  uint32_t* item;  // work item (job) of each path (multi-job wavefronts; null otherwise)
  uint32_t* counters;  // [0],[1] path queues, [2] shadow queue, [3] error bits
  unsigned long long* stats;  // traversal counters (extend rays/nodes/boxes/prims, shadow ...) or null
  uint32_t capacity;
  uint32_t variant;  // GPRT_JOB_SIMPLE_EXTEND | GPRT_JOB_SIMPLE_SHADOW
};

// Pixels a chunk covers: `layers` consecutive samples of `npix` pixels,
// pixel i = pix_list ? pix_list[pix0 + i] : pix0 + i.
struct ChunkDesc {
  uint32_t pix0, npix, layers;
  const uint32_t* pix_list;
  uint64_t seed;
  int bounce_base;
};

int launch_grid(uint32_t n, int block, int max_blocks);

void launch_intersect(const DevScene& sc, const gprt_ray* rays, uint32_t n, bool any_hit, gprt_hit* hits, int* err,
                      cudaStream_t st);

// path tracing (pkg/integrator/path_tracing.go) in wavefront form
void launch_pt_raygen(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                      cudaStream_t st);
void launch_pt_extend(const DevScene& sc, const DevPaths& P, int cur, int block, int grid, cudaStream_t st);
void launch_pt_shade(const DevScene& sc, const DevPaths& P, const ChunkDesc& ch, int cur, int bounce, int block,
                     int grid, cudaStream_t st);
void launch_pt_shadow(const DevScene& sc, const DevPaths& P, int block, int grid, cudaStream_t st);
void launch_accumulate(const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block, cudaStream_t st);

// bidirectional path tracing (pkg/integrator/bdpt.go), one sample per thread
void launch_bdpt(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                 cudaStream_t st);

// film
void launch_apply_splats(const DevFilm& film, cudaStream_t st);
void launch_resolve_rgba8(const DevFilm& film, uint8_t* out, cudaStream_t st);
void launch_image_mean(const DevFilm& film, float* out, cudaStream_t st);
void launch_active_pixels(const DevFilm& film, uint32_t target, uint32_t min_samples, float threshold,
                          uint32_t* list, uint32_t* count, cudaStream_t st);

}  // namespace gprt
