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

// Live paths of one bounce, compacted: slot i of the queue holds the whole
// state of one path (structure of arrays), so every kernel of a bounce reads
// and writes contiguous slots.
struct PathBuf {
  float4* ray_o;   // origin.xyz, primitive the ray leaves (uint bits)
  float4* ray_d;   // direction.xyz, BVH root node of the path's scene (int bits)
  float4* weight;  // radiance weight rgb, origin index of the path (uint bits)
  float4* thr;     // Russian-roulette throughput rgb
  float4* L;       // radiance gathered so far rgb
  uint4* ids;      // pixel, sample index, sampler position, work item
};

// Wavefront path state (capacity = paths per chunk).  Paths are generated in
// origin order (origin index = layer * npix + pixel of the chunk) into q[0];
// each shade kernel compacts the continuing paths of q[cur] into q[cur ^ 1]
// and writes the radiance of finished paths to Lout at their origin index.
// BDPT working set of one chunk of samples (see kernels_bdpt.cu): subpath
// vertices as 5 float4 fields, each indexed [vertex * ns + sample] (camera
// vertices 0..maxv-1, light vertices maxv..2 maxv-1), per-sample metadata,
// and one contribution slot per (strategy, sample).
// The subpaths in flight between bounces of the BDPT subpath wavefront, one
// slot per subpath (structure of arrays): the ray (origin = the last vertex,
// the primitive it leaves; direction, the forward pdf of the next vertex),
// the throughput and the MIS prefix through the vertex before the last, the
// last vertex's normal and forward pdf, the sample (index in the chunk,
// sampler position, pixel, sample number) and the state bits (length,
// bounces, camera / light, connectibility of the last two vertices, whether
// the last vertex is on a surface or at infinity; the camera subpath's
// length for a light subpath).
struct BdQueue {
  float4* o;
  float4* d;
  float4* beta;
  float4* last;
  uint4* ids;
  uint2* st;
};

struct DevBdpt {
  float4* v[5];
  float4* pdf;    // per vertex: fwd, flags | (light + 1) << 8 (int bits), rev, the subpath's MIS prefix
  BdQueue q[2];   // the subpath wavefront's two queues
  float4* hit;    // closest hit of each slot of the current queue
  float4* lorig;  // per sample, 3 float4: the light subpath's origin (infinite lights: pdf fix-ups)
  uint4* meta;    // nc | nl << 8, sampler position after the subpaths, pixel, sample index
  uint2* masks;   // strategies that draw samples: light-tracing (bit s), direct-lighting (bit t)
  float4* contrib;
  float2* uv;     // surface UV per vertex (scenes with textures only, else null)
  // Per strategy k, the samples that have it: ns slots from k * ns, one
  // range of kBdWindow slots per window of kBdWindow consecutive samples
  // (window w from k * ns + w * kBdWindow), so that the strategy kernels can
  // take every strategy of one window of samples before the next window.
  uint32_t* slist;
  uint32_t* scount;   // entries of list k in window w at [w * K + k] (K = (maxv + 1) * maxv)
  uint32_t* sprefix;  // per strategy class c, from c * (nw * K + 1): exclusive prefix of its counts over [w * K + k], then the class total
  uint32_t ns;    // samples per chunk
  uint32_t nw;    // sample windows per chunk
  int maxv;       // vertices per subpath (10 or 18)
};

// Samples per window of the BDPT strategy lists: the vertices of a window
// (2 * maxv records of 96 B per sample: 31 MB at maxv = 10) stay in L2 while
// all of its strategies run.  A multiple of the list kernel's 1,024-sample
// block.
constexpr uint32_t kBdWindow = 16384;
inline uint32_t bdpt_windows(uint32_t ns) { return (ns + kBdWindow - 1) / kBdWindow; }

struct DevPaths {
  PathBuf q[2];
  float4* hit;     // closest hit of slot i of the current queue: t, prim, u, v
  float4* Lout;    // radiance of every finished path, by origin index
  float4* sh_o;    // shadow ray origin.xyz, tmax
  float4* sh_d;    // shadow ray direction.xyz, skip primitive
  float4* sh_c;    // contribution rgb, origin index of its path (uint bits)
  int* sh_root;    // BVH root of each shadow ray (multi-scene wavefronts; null: the scene's root)
  uint32_t* order; // slots of the queue by shading group (order_slots; null: queue order)
  uint32_t* counters;  // [0],[1] path queues, [2] shadow queue, [3] error bits, [4],[5] ray fetch, [6],[7] order
  // multi-job wavefronts: one error word per work item and the items' first
  // origin indices (null for a single job: its error word is counters[3])
  uint32_t* item_err;
  const uint32_t* item_start;
  const uint32_t* n_items;
  unsigned long long* stats;  // traversal counters (extend rays/nodes/boxes/prims, shadow ...) or null
  uint32_t capacity;
  uint32_t variant;  // GPRT_JOB_SIMPLE_EXTEND | GPRT_JOB_SIMPLE_SHADOW | GPRT_JOB_SHADE_OCCUPANCY
  DevBdpt bd;        // BDPT jobs only
};

// Subpath vertices per BDPT subpath for a scene depth, and the device bytes
// of the BDPT working set of `ns` samples.
inline int bdpt_maxv(int max_depth) { return max_depth <= 9 ? 10 : 18; }
inline size_t bdpt_bytes(uint32_t ns, int maxv) {
  return (size_t)ns * (6 * 2 * maxv * 16 + 16 + 8 + (size_t)(maxv + 1) * maxv * 16 + 16 + 2 * 88 + 16 + 48) +
         (size_t)5 * (bdpt_windows(ns) * (maxv + 1) * maxv + 1) * 4 + 26 * 256;
}

constexpr uint32_t kVariantBits = GPRT_JOB_SIMPLE_EXTEND | GPRT_JOB_SIMPLE_SHADOW | GPRT_JOB_SHADE_OCCUPANCY;


constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Device bytes of the path state of `cap` paths (one region: counters, two
// queues, hits, origin radiance, shadow rays, slot order; sh_root when multi-scene).
constexpr size_t path_region_bytes(uint32_t cap, bool multi) {
  return 256 + 2 * (5 * align256((size_t)cap * sizeof(float4)) + align256((size_t)cap * sizeof(uint4))) +
         5 * align256((size_t)cap * sizeof(float4)) + align256((size_t)cap * sizeof(uint32_t)) +
         (multi ? align256((size_t)cap * sizeof(int)) : 0);
}

// Points the arrays of P at consecutive 256-byte-aligned ranges of `base`
// (path_region_bytes(cap, multi) bytes, 256-byte aligned).
void carve_paths(unsigned char* base, uint32_t cap, bool multi, DevPaths& P);

// Pixels a chunk covers: `layers` consecutive samples of `npix` pixels,
// pixel i = pix_list ? pix_list[pix0 + i] : pix0 + i.
struct ChunkDesc {
  uint32_t pix0, npix, layers;
  const uint32_t* pix_list;
  uint64_t seed;
};

int launch_grid(uint32_t n, int block, int max_blocks);

void launch_intersect(const DevScene& sc, const gprt_ray* rays, uint32_t n, bool any_hit, gprt_hit* hits, int* err,
                      cudaStream_t st);

// path tracing (pkg/integrator/path_tracing.go) in wavefront form
void launch_pt_raygen(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                      cudaStream_t st);
void launch_pt_extend(const DevScene& sc, const DevPaths& P, int cur, int bounce, int block, int grid, cudaStream_t st);
// Builds P.order for queue `cur` (slots by shading group) before shading.
void launch_hit_order(const DevScene& sc, const DevPaths& P, int cur, uint32_t cap, int sms, cudaStream_t st);
void launch_pt_shade(const DevScene& sc, const DevPaths& P, const ChunkDesc& ch, int cur, int bounce, int block,
                     int grid, cudaStream_t st);
void launch_pt_shadow(const DevScene& sc, const DevPaths& P, int cur, int block, int grid, cudaStream_t st);
void launch_accumulate(const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block, cudaStream_t st);

// bidirectional path tracing (pkg/integrator/bdpt.go): subpaths per sample,
// then one thread per (strategy, sample), then the per-sample sums
void launch_bdpt(const DevScene& sc, const DevFilm& film, const DevPaths& P, const ChunkDesc& ch, int block,
                 cudaStream_t st);

// film
void launch_apply_splats(const DevFilm& film, cudaStream_t st);
void launch_resolve_rgba8(const DevFilm& film, uint8_t* out, cudaStream_t st);
void launch_resolve_tile(const DevFilm& film, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, uint8_t* out,
                         cudaStream_t st);
void launch_image_mean(const DevFilm& film, float* out, cudaStream_t st);
void launch_active_pixels(const DevFilm& film, uint32_t target, uint32_t min_samples, float threshold,
                          uint32_t* list, uint32_t* count, cudaStream_t st);

}  // namespace gprt
