// server.cu - gprt_server: a device-resident request loop with continuous
// batching.  Many progressive path-tracing jobs of different scenes and
// resolutions share every wavefront.
//
// Device data of the server:
//   scene pool   one growable array per primitive type (BVH nodes, triangles +
//                normals, quads, spheres, materials, lights).  A scene admitted
//                for the first time is copied in from its gprt_scene and its
//                node / leaf / light references are rebased to pool indices,
//                so the unchanged traversal kernels walk any scene from its
//                root.  Primitive ids of the pool: triangles [0, 2^30), quads
//                [2^30, 2^31), spheres [2^31, 3 x 2^30), discs / cylinders /
//                cones [3 x 2^30, 2^32 - 1).
//   path state   one set of wavefront arrays (DevPaths) of step capacity,
//                shared by all jobs; each path records its work item.
//   item table   per step: prefix sums of the items' paths and pixels (for a
//                binary search from a path or pixel index to its item) and one
//                DevItem per item (the job's camera, film, seed, pool offsets).
//   films        one per admitted job (sum rgb + lum, lum^2, count per pixel).
// A step: raygen over all items -> [extend -> shade -> shadow] x depth ->
// accumulate, replayed from a CUDA graph captured once per depth (kernel
// arguments are fixed device pointers; what changes per step is the item
// table, copied in before the replay).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <unordered_map>

#include "device.cuh"
#include "handles.h"
#include "pt_shade.cuh"

namespace gprt {
namespace {

// the pool's arrays, one per kind of scene data
constexpr int kNodes = 0, kTris = 1, kQuads = 2, kSpheres = 3, kQuadrics = 4, kMats = 5, kLights = 6, kTexInfo = 7,
              kTexels = 8;
constexpr int kPoolArrays = 9;

constexpr uint32_t kPoolQuadBase = 1u << 30;
constexpr uint32_t kPoolSphereBase = 2u << 30;
constexpr uint32_t kPoolQuadricBase = 3u << 30;

struct StepHdr {
  uint32_t n_items, total_paths, total_pix, dry;
};

struct DevItem {
  uint32_t path0, pix0, npix, layers;
  int root, mat_off, light_off, n_lights;
  int tex_off, texel_off, has_textures, has_tri_uvs;
  int has_infinite, max_depth, rr_min_bounces, width;
  float3 world_center;
  float world_radius;
  unsigned long long seed;
  float4* rgbl;
  float* lum2;
  uint32_t* count;
  const uint32_t* list;  // the item's pixels (a round of an adaptive pass); null: item pixel i is film pixel i
  DevCamera cam;
};

// The shading order of the step's queue `cur` (order_slots), from the group
// stored in each pooled primitive's record.
__global__ void __launch_bounds__(1024) k_srv_hit_order(DevScene pool, DevPaths P, int cur) {
  order_slots(P, cur, [&](uint32_t, uint32_t prim) { return prim_group(pool, prim); });
}

// Camera rays of every item: path p is sample `layer` of pixel i of its item,
// drawn exactly as k_pt_raygen draws them for a single job.
__global__ void k_srv_raygen(DevPaths P, const StepHdr* hdr, const uint32_t* path0, const DevItem* items) {
  uint32_t n = hdr->total_paths, ni = hdr->n_items;
  // the items' error words start clear (read back after the step)
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ni; k += gridDim.x * blockDim.x) P.item_err[k] = 0;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    uint32_t k = find_range(path0, ni, p);
    const DevItem& it = items[k];
    uint32_t rel = p - it.path0;
    uint32_t layer = rel / it.npix, pix = rel - layer * it.npix;
    if (it.list) pix = it.list[pix];
    uint32_t sample = it.count[pix] + layer;
    int x = (int)(pix % (uint32_t)it.width), y = (int)(pix / (uint32_t)it.width);
    Rng rng;
    rng.init(it.seed, pix, sample);
    float2 lens = rng.next2();
    float2 jit = rng.next2();
    float3 o, d;
    camera_ray(it.cam, x, y, lens, jit, o, d);
    const PathBuf& Q = P.q[0];
    Q.ray_o[p] = make_float4(o.x, o.y, o.z, __uint_as_float(kNoHit));
    Q.ray_d[p] = make_float4(d.x, d.y, d.z, __int_as_float(it.root));
    // weight 1 with origin index p, roulette throughput 1 and radiance 0 are
    // implied at bounce 0 (not stored)
    Q.ids[p] = make_uint4(pix, sample, rng.pos, k);
    P.Lout[p] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.counters[0] = n;
    P.counters[4] = 0;
    P.counters[5] = 0;
  }
}

// One bounce of every live path, each shaded with its own job's scene view
// (materials, lights, infinite-light bounds, depth and Russian-roulette
// settings) over the pooled geometry.
__device__ __forceinline__ void srv_shade(const DevScene& pool, const DevPaths& P, const DevItem* items, int cur,
                                          int bounce) {
  uint32_t n = P.counters[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.counters[4] = 0;
    P.counters[5] = 0;
  }
  const PathBuf Q = P.q[cur];
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t slot = first < n ? (P.order ? P.order[first] : first) : 0u;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    uint32_t i = base + threadIdx.x;
    // the slot of the next iteration, read now and prefetched after this one
    // (one iteration ahead: two ahead measured slower)
    uint32_t inext = i + stride;
    uint32_t snext = inext < n ? (P.order ? P.order[inext] : inext) : 0u;
    ShadeOut o;
    o.cont = false;
    bool live = i < n;
    if (live) {
      i = slot;
      const DevItem& it = items[Q.ids[i].w];
      DevScene v = pool;
      v.materials = pool.materials + it.mat_off;
      v.lights = pool.lights + it.light_off;
      v.tex_info = pool.tex_info + it.tex_off;
      v.texels = pool.texels + it.texel_off;
      v.has_textures = it.has_textures;
      v.tri_uvs = it.has_tri_uvs ? pool.tri_uvs : nullptr;
      v.n_lights = it.n_lights;
      v.has_infinite = it.has_infinite;
      v.world_center = it.world_center;
      v.world_radius = it.world_radius;
      v.max_depth = it.max_depth;
      v.rr_min_bounces = it.rr_min_bounces;
      v.root = it.root;
      shade_path(v, P, Q, P.hit, i, it.seed, bounce, o);
    }
    push_shade_out(P, cur, live, o);
    if (inext < n) prefetch_slot(Q, P.hit, snext, bounce > 0);
    slot = snext;
  }
}

// The kernel at 2 blocks of 256 threads per SM (16 warps, 117 registers)
// or, as GPRT_JOB_SHADE_OCCUPANCY, 3 blocks of 192 threads (18 warps at 96
// registers, 64 bytes spilled).  More warps did not pay: the 3-block
// budget measured 8 % slower on the heterogeneous batch (shade 462 vs 428 ms
// per batch), a 112-register cap without spills 28 % slower.
template <int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    k_srv_shade(DevScene pool, DevPaths P, const DevItem* items, int cur, int bounce) {
  srv_shade(pool, P, items, cur, bounce);
}

// PixelStats.AddSample for every pixel of every item, samples in order (the
// same additions as k_accumulate).
__global__ void k_srv_accumulate(DevPaths P, const StepHdr* hdr, const uint32_t* pix0, const DevItem* items) {
  if (hdr->dry) return;
  uint32_t n = hdr->total_pix, ni = hdr->n_items;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    uint32_t k = find_range(pix0, ni, t);
    const DevItem& it = items[k];
    uint32_t i = t - it.pix0;
    uint32_t f = it.list ? it.list[i] : i;  // the film pixel
    float4 acc = it.rgbl[f];
    float l2 = it.lum2[f];
    for (uint32_t layer = 0; layer < it.layers; layer++) {
      float4 c = P.Lout[it.path0 + layer * it.npix + i];
      float lum = luminance(f3(c));
      acc.x += c.x;
      acc.y += c.y;
      acc.z += c.z;
      acc.w += lum;
      l2 += lum * lum;
    }
    it.rgbl[f] = acc;
    it.lum2[f] = l2;
    it.count[f] += it.layers;
  }
}

// Rebases the references of `n` nodes copied to pool index node_off: inner
// children by node_off, leaves by the offset of their primitive type.
__global__ void k_rebase_nodes(float4* nodes, uint32_t n, int node_off, int tri_off, int quad_off, int sph_off,
                               int qdr_off) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n * 4u; c += gridDim.x * blockDim.x) {
    float4* a = nodes + (size_t)(c >> 2) * 8 + 2 * (c & 3);
    int ref = __float_as_int(a->w);
    if (ref == kEmptyChild) continue;
    int meta = __float_as_int(a[1].w);
    int off = node_off;
    if (meta != 0) {
      int type = (meta >> kLeafTypeShift) & 3;
      off = type == kPrimTriangle ? tri_off : type == kPrimQuad ? quad_off : type == kPrimSphere ? sph_off : qdr_off;
    }
    a->w = __int_as_float(ref + off);
  }
}

__global__ void k_rebase_lights(DevLight* L, uint32_t n, int quad_off, int sph_off, int qdr_off) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (L[i].kind == kLightQuad) L[i].prim += quad_off;
    else if (L[i].kind == kLightSphere && L[i].prim >= 0) L[i].prim += sph_off;
    else if (L[i].kind == kLightDisc || L[i].kind == kLightDiscSpot) L[i].prim += qdr_off;
  }
}

double now_ms(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// One growable device array (or two parallel ones) with a first-fit range
// allocator over element indices.
struct PoolArray {
  static constexpr int kBufs = 3;
  size_t elem[kBufs] = {0, 0, 0};  // bytes per element of each parallel buffer (0: unused)
  void* buf[kBufs] = {nullptr, nullptr, nullptr};
  size_t cap = 0;
  std::map<size_t, size_t> free_;  // offset -> length

  size_t bytes_per() const { return elem[0] + elem[1] + elem[2]; }
  size_t bytes() const { return cap * bytes_per(); }
  bool take(size_t n, size_t* off) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        size_t rest = it->second - n, o = it->first + n;
        free_.erase(it);
        if (rest) free_[o] = rest;
        return true;
      }
    }
    return false;
  }
  void give(size_t off, size_t n) {
    if (!n) return;
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && off + n == nx->first) {
      n += nx->second;
      free_.erase(nx);
    }
    auto pv = free_.lower_bound(off);
    if (pv != free_.begin()) {
      --pv;
      if (pv->first + pv->second == off) {
        pv->second += n;
        return;
      }
    }
    free_[off] = n;
  }
  // elements free at the end of the array
  size_t tail_free() const {
    if (free_.empty()) return 0;
    auto last = std::prev(free_.end());
    return last->first + last->second == cap ? last->second : 0;
  }
  bool empty_all() const { return cap == 0 || (free_.size() == 1 && free_.begin()->second == cap); }
};

}  // namespace
}  // namespace gprt

// A scene resident in the pool.
struct PoolScene {
  uint64_t serial = 0;
  size_t off[gprt::kPoolArrays] = {};  // element offsets in the pool arrays (kNodes ... kTexels)
  size_t cnt[gprt::kPoolArrays] = {};
  int refs = 0;
  uint64_t last_use = 0;
  size_t bytes = 0;
  // per-job constants of the scene
  int root = -1;
  int has_infinite = 0, max_depth = 0, rr_min = 0, has_tri_uvs = 0;
  float3 world_center{};
  float world_radius = 0.f;
  DevCamera cam{};
  uint32_t width = 0, height = 0;
};

struct SrvRequest {
  uint64_t ticket;
  gprt_scene* scene;
  uint64_t serial;
  gprt_job_desc desc;
  double submit_ms;
};

struct SrvJob {
  uint64_t ticket = 0;
  PoolScene* ps = nullptr;
  gprt_job_desc desc{};
  uint32_t npix = 0;
  DevFilm film{};
  std::vector<void*> bufs;
  size_t film_bytes = 0;
  uint32_t passes = 0, spp_done = 0, pass_target = 0;
  // adaptive sampling (the scene's AdaptiveMinSamples < 1), as
  // gprt_job_render_pass runs it: per pass the minimum samples of every
  // pixel in bulk, then rounds of one sample for each pixel still active
  // (k_active_pixels: below the pass target and not converged), each round's
  // pixel list built on the device after the step before it; the pass ends
  // when no pixel is active.  spp_done is then the average sample count.
  bool adaptive = false;
  double min_frac = 1.0;       // AdaptiveMinSamples
  float threshold = 0.f;       // AdaptiveThreshold
  uint32_t min_s = 0;          // the pass's minimum samples per pixel
  int64_t uniform = 0;         // the sample count of every pixel while all are equal, else -1
  uint64_t total = 0;          // samples taken over all pixels
  uint32_t* d_list = nullptr;  // npix entries: the pixels of the next round, then their count
  uint32_t active = 0;         // pixels listed for the next round (0: none listed)
  bool running = true;
  double submit_ms = 0, admit_ms = 0;
  uint64_t last_served = 0;
  // BDPT requests: a per-job render on a private copy of the scene (which
  // the caller may destroy meanwhile), one pass between batched steps
  gprt_scene* bd_scene = nullptr;
  gprt_job* bd = nullptr;
};

struct gprt_server {
  gprt_ctx* ctx = nullptr;
  gprt_server_desc desc{};
  std::chrono::steady_clock::time_point t0;
  cudaStream_t stream = nullptr;
  // the BDPT job rendering its first pass runs on this stream, created with
  // the device's greatest priority: its blocks are scheduled ahead of the
  // batched path-tracing wavefront's whenever both wait for an SM
  cudaStream_t bd_first = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // state (smu)
  std::mutex smu;
  gprt::PoolArray pool[gprt::kPoolArrays];
  uint64_t pool_gen = 0;
  std::vector<std::unique_ptr<PoolScene>> scenes;
  std::map<uint64_t, std::unique_ptr<SrvJob>> jobs;  // admitted, by ticket
  DevPaths P{};
  std::vector<void*> path_bufs;
  size_t path_bytes = 0;
  uint64_t bd_rounds = 0;  // BDPT passes run (their least-recently-served order)
  uint32_t firsts_run = 0; // consecutive steps that carried first passes only
  // read-back staging (resolved image before the copy to the host), grown
  // on demand under rmu and kept: a cudaFree per read would synchronise the
  // device while steps run.  Reads run on rb_stream behind rb_ev (recorded
  // on the step stream), one at a time (rmu, taken before smu).
  std::mutex rmu;
  cudaStream_t rb_stream = nullptr;
  cudaEvent_t rb_ev = nullptr;
  // released path-tracing films kept for the next admissions (a cudaMalloc
  // per buffer at admission and a cudaFree at release, which waits for the
  // whole device, cost about 1.5 % of a 256-job batch); counted in
  // bytes_in_use and freed first when the budget is short.  rb_done is
  // recorded on the read-back stream as a film enters the cache, and a
  // reuse waits for it, so a read still queued sees the old image.
  struct CachedFilm {
    uint32_t npix = 0;
    bool adaptive = false;
    std::vector<void*> bufs;
    DevFilm film{};
    uint32_t* d_list = nullptr;
    size_t bytes = 0;
  };
  std::vector<CachedFilm> film_cache;
  size_t film_cache_bytes = 0;
  cudaEvent_t rb_done = nullptr;
  std::vector<void*> rb_bufs;
  size_t rb_bytes = 0;
  unsigned char* rb = nullptr;
  // pinned host staging of read-backs: the device-to-host copy runs at the
  // link's rate, then one host memcpy into the caller's (pageable) buffer
  unsigned char* rb_host = nullptr;
  size_t rb_host_bytes = 0;
  size_t reserve = 0;      // bytes promised to the film being admitted
  uint32_t capacity = 0;   // path capacity allocated
  uint32_t step_paths = 0; // paths per step (<= capacity)
  uint32_t block = 128;
  uint32_t flags = 0;
  // item table: [hdr | path0[max+1] | pix0[max+1]] then items[max]
  unsigned char* d_table = nullptr;
  // then one error word per item at err_off (cleared by the step's raygen)
  unsigned char* h_table = nullptr;  // pinned staging of the table; its error words receive the read-back
  uint32_t* h_err = nullptr;         // pinned: a pageable read-back would block inside the runtime
  uint32_t* h_act = nullptr;         // pinned: active-pixel counts of the adaptive rounds being listed
                                     // until the step ends, stalling other threads' CUDA calls
  size_t table_bytes = 0, prefix_bytes = 0, err_off = 0, act_off = 0;
  std::map<int, cudaGraphExec_t> graphs;  // by depth
  uint64_t graph_gen = ~0ull;
  // instrumentation (GPRT_JOB_TIME_KERNELS / GPRT_JOB_COUNT_TRAVERSAL in flags):
  // event pairs around every kernel of a step, by depth (captured into the
  // graph of that depth), and the device traversal counters
  std::map<int, std::vector<cudaEvent_t>> step_events;
  unsigned long long* d_stats = nullptr;
  gprt_job_counters acc{};
  gprt_server_stats st{};
  // requests and events (qmu)
  std::mutex qmu;
  std::condition_variable cv_work, cv_ev;
  std::deque<SrvRequest> pending;
  std::deque<gprt_event> events;
  uint64_t next_ticket = 1;
  std::atomic<uint32_t> n_running{0};
  uint64_t work_gen = 0;
  // loop thread
  std::thread loop;
  bool stopping = false, loop_running = false;
};

using namespace gprt;

namespace {



void emit(gprt_server* sv, uint64_t ticket, uint32_t kind, uint32_t passes, uint32_t spp, int status,
          double submit_ms) {
  gprt_event e{};
  e.ticket = ticket;
  e.kind = kind;
  e.pass_number = passes;
  e.samples_per_pixel = spp;
  e.status = status;
  e.t_ms = now_ms(sv->t0);
  e.submit_ms = submit_ms;
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    sv->events.push_back(e);
  }
  sv->cv_ev.notify_all();
}

// Released films kept for reuse at most.
constexpr size_t kFilmCacheMax = 1024;

// Frees cached films until `need` more bytes fit the budget (all of them
// with need = SIZE_MAX).
void drop_film_cache(gprt_server* sv, size_t need);

// A path-tracing job's film (+ its active-pixel list and count when the
// scene samples adaptively).
size_t film_bytes_for(uint32_t npix, bool adaptive) {
  return (size_t)npix * (sizeof(float4) + sizeof(float) + sizeof(uint32_t)) +
         (adaptive ? ((size_t)npix + 1) * sizeof(uint32_t) : 0);
}

size_t bytes_in_use(gprt_server* sv) {
  size_t b = sv->path_bytes + sv->table_bytes + sv->reserve + sv->film_cache_bytes;
  for (auto& a : sv->pool) b += a.bytes();
  for (auto& kv : sv->jobs) b += kv.second->film_bytes;
  return b;
}

void drop_film_cache(gprt_server* sv, size_t need) {
  while (!sv->film_cache.empty() &&
         (need == SIZE_MAX || bytes_in_use(sv) + need > sv->desc.hbm_budget_bytes)) {
    gprt_server::CachedFilm& c = sv->film_cache.back();
    free_all(c.bufs);
    sv->film_cache_bytes -= c.bytes;
    sv->film_cache.pop_back();
  }
}

// Element counts of a gprt_scene in the pool's arrays.
void scene_counts(const gprt_scene* s, size_t cnt[kPoolArrays]) {
  const HostScene& h = s->host;
  cnt[kNodes] = h.nodes.size() / 8;
  cnt[kTris] = h.n_tris;
  cnt[kQuads] = h.n_quads;
  cnt[kSpheres] = h.n_spheres;
  cnt[kQuadrics] = h.n_quadrics;
  cnt[kMats] = h.materials.size();
  cnt[kLights] = h.lights.size();
  cnt[kTexInfo] = h.tex_info.size();
  cnt[kTexels] = h.texels.size();
}

size_t scene_bytes(gprt_server* sv, const size_t cnt[kPoolArrays]) {
  size_t b = 0;
  for (int k = 0; k < kPoolArrays; k++) b += cnt[k] * sv->pool[k].bytes_per();
  return b;
}

DevScene pool_view(gprt_server* sv) {
  DevScene d{};
  d.nodes = static_cast<const float4*>(sv->pool[kNodes].buf[0]);
  d.tris = static_cast<const float4*>(sv->pool[kTris].buf[0]);
  d.tri_normals = static_cast<const float4*>(sv->pool[kTris].buf[1]);
  d.tri_uvs = static_cast<const float4*>(sv->pool[kTris].buf[2]);  // a job sees it only when its scene has UVs
  d.quads = static_cast<const float4*>(sv->pool[kQuads].buf[0]);
  d.spheres = static_cast<const float4*>(sv->pool[kSpheres].buf[0]);
  d.quadrics = static_cast<const float4*>(sv->pool[kQuadrics].buf[0]);
  d.materials = static_cast<const DevMaterial*>(sv->pool[kMats].buf[0]);
  d.lights = static_cast<const DevLight*>(sv->pool[kLights].buf[0]);
  d.tex_info = static_cast<const uint4*>(sv->pool[kTexInfo].buf[0]);
  d.texels = static_cast<const float4*>(sv->pool[kTexels].buf[0]);
  d.n_nodes = (int)sv->pool[kNodes].cap;
  d.root = -1;
  d.quad_base = kPoolQuadBase;
  d.sphere_base = kPoolSphereBase;
  d.quadric_base = kPoolQuadricBase;
  d.n_prims = 0xFFFFFFFEu;
  return d;
}

// Grows pool array k to hold at least `need_cap` elements (copying what it
// holds).  Returns false when the budget or the device refuses.
bool grow(gprt_server* sv, int k, size_t need_cap) {
  PoolArray& a = sv->pool[k];
  size_t new_cap = std::max(need_cap, a.cap + a.cap / 2);
  if (k == kTris || k == kQuads) new_cap = std::min<size_t>(new_cap, kPoolQuadBase);
  if (k == kSpheres) new_cap = std::min<size_t>(new_cap, kPoolQuadricBase - kPoolSphereBase);
  if (k == kQuadrics) new_cap = std::min<size_t>(new_cap, (size_t)0xFFFFFFFEu - kPoolQuadricBase);
  if (k == kNodes || k == kMats || k == kLights || k == kTexInfo || k == kTexels)
    new_cap = std::min<size_t>(new_cap, 0x7FFFFFFF);
  if (new_cap < need_cap) return false;
  size_t used = bytes_in_use(sv);
  size_t extra = (new_cap - a.cap) * a.bytes_per();
  if (used + extra > sv->desc.hbm_budget_bytes) {
    new_cap = need_cap;  // exact fit
    extra = (new_cap - a.cap) * a.bytes_per();
    if (used + extra > sv->desc.hbm_budget_bytes) return false;
  }
  void* nb[PoolArray::kBufs] = {nullptr, nullptr, nullptr};
  for (int b = 0; b < PoolArray::kBufs; b++) {
    if (!a.elem[b]) continue;
    if (cudaMalloc(&nb[b], new_cap * a.elem[b]) != cudaSuccess) {
      cudaGetLastError();
      for (int q = 0; q < b; q++)
        if (nb[q]) cudaFree(nb[q]);
      return false;
    }
    if (a.cap) cudaMemcpyAsync(nb[b], a.buf[b], a.cap * a.elem[b], cudaMemcpyDeviceToDevice, sv->stream);
  }
  cudaStreamSynchronize(sv->stream);
  for (int b = 0; b < PoolArray::kBufs; b++)
    if (a.buf[b]) cudaFree(a.buf[b]);
  size_t old = a.cap;
  for (int b = 0; b < PoolArray::kBufs; b++) a.buf[b] = nb[b];
  a.cap = new_cap;
  a.give(old, new_cap - old);
  sv->pool_gen++;
  return true;
}

// Frees the pool's device arrays when no scene is resident.
void shrink_if_empty(gprt_server* sv) {
  if (!sv->scenes.empty()) return;
  bool any = false;
  for (auto& a : sv->pool) {
    for (int b = 0; b < PoolArray::kBufs; b++)
      if (a.buf[b]) {
        cudaFree(a.buf[b]);
        a.buf[b] = nullptr;
        any = true;
      }
    a.cap = 0;
    a.free_.clear();
  }
  if (any) sv->pool_gen++;
}

void evict(gprt_server* sv, PoolScene* ps) {
  for (int k = 0; k < kPoolArrays; k++) sv->pool[k].give(ps->off[k], ps->cnt[k]);
  for (auto it = sv->scenes.begin(); it != sv->scenes.end(); ++it)
    if (it->get() == ps) {
      sv->scenes.erase(it);
      break;
    }
}

// Places the scene's arrays in the pool, evicting unreferenced scenes (least
// recently used first) and growing arrays as the budget allows.
bool place(gprt_server* sv, const size_t cnt[kPoolArrays], size_t off[kPoolArrays]) {
  for (;;) {
    bool ok = true;
    size_t got[kPoolArrays] = {};
    int k = 0;
    for (; k < kPoolArrays; k++) {
      if (cnt[k] == 0) continue;
      if (!sv->pool[k].take(cnt[k], &got[k])) {
        ok = false;
        break;
      }
    }
    if (ok) {
      for (int i = 0; i < kPoolArrays; i++) off[i] = got[i];
      return true;
    }
    for (int i = 0; i < k; i++) sv->pool[i].give(got[i], cnt[i]);
    // grow array k by what its free tail lacks
    PoolArray& a = sv->pool[k];
    if (grow(sv, k, a.cap + cnt[k] - a.tail_free())) continue;
    // evict the least recently used unreferenced scene and retry
    PoolScene* lru = nullptr;
    for (auto& s : sv->scenes)
      if (s->refs == 0 && (!lru || s->last_use < lru->last_use)) lru = s.get();
    if (!lru) return false;
    evict(sv, lru);
    shrink_if_empty(sv);
  }
}

// Copies a gprt_scene into the pool (or finds it there).
PoolScene* make_resident(gprt_server* sv, gprt_scene* s) {
  for (auto& ps : sv->scenes)
    if (ps->serial == s->serial) return ps.get();
  size_t cnt[kPoolArrays], off[kPoolArrays];
  scene_counts(s, cnt);
  if (!place(sv, cnt, off)) return nullptr;
  // node ids stay below the root flag bits, quadric ids below kOverflowHit
  if (off[kNodes] + cnt[kNodes] >= (size_t)kMaxNodes) return nullptr;
  if (kPoolQuadricBase + off[kQuadrics] + cnt[kQuadrics] >= (size_t)kOverflowHit) return nullptr;
  auto ps = std::make_unique<PoolScene>();
  ps->serial = s->serial;
  for (int k = 0; k < kPoolArrays; k++) {
    ps->off[k] = off[k];
    ps->cnt[k] = cnt[k];
  }
  ps->bytes = scene_bytes(sv, cnt);
  const DevScene& d = s->dev;
  cudaStream_t st = sv->stream;
  auto copy = [&](int k, int b, const void* src) {
    if (!cnt[k]) return;
    PoolArray& a = sv->pool[k];
    cudaMemcpyAsync(static_cast<unsigned char*>(a.buf[b]) + off[k] * a.elem[b], src, cnt[k] * a.elem[b],
                    cudaMemcpyDeviceToDevice, st);
  };
  copy(kNodes, 0, d.nodes);
  copy(kTris, 0, d.tris);
  copy(kTris, 1, d.tri_normals);
  if (d.tri_uvs) copy(kTris, 2, d.tri_uvs);
  copy(kQuads, 0, d.quads);
  copy(kSpheres, 0, d.spheres);
  copy(kQuadrics, 0, d.quadrics);
  copy(kMats, 0, d.materials);
  copy(kLights, 0, d.lights);
  copy(kTexInfo, 0, d.tex_info);  // texel indices stay scene-relative: jobs see offset views
  copy(kTexels, 0, d.texels);
  if (cnt[kNodes]) {
    float4* nodes = static_cast<float4*>(sv->pool[kNodes].buf[0]) + off[kNodes] * 8;
    uint32_t n = (uint32_t)cnt[kNodes];
    k_rebase_nodes<<<launch_grid(n * 4, 256, 4096), 256, 0, st>>>(nodes, n, (int)off[kNodes], (int)off[kTris],
                                                                   (int)off[kQuads], (int)off[kSpheres],
                                                                   (int)off[kQuadrics]);
  }
  if (cnt[kLights]) {
    DevLight* L = static_cast<DevLight*>(sv->pool[kLights].buf[0]) + off[kLights];
    k_rebase_lights<<<1, 128, 0, st>>>(L, (uint32_t)cnt[kLights], (int)off[kQuads], (int)off[kSpheres],
                                       (int)off[kQuadrics]);
  }
  ps->root = cnt[kNodes] ? ((int)off[kNodes] | (s->host.test_stack_cap ? kRootStackCap : 0)) : -1;
  ps->has_infinite = d.has_infinite;
  ps->has_tri_uvs = d.tri_uvs ? 1 : 0;
  ps->max_depth = d.max_depth;
  ps->rr_min = d.rr_min_bounces;
  ps->world_center = d.world_center;
  ps->world_radius = d.world_radius;
  ps->cam = d.cam;
  ps->width = s->host.sampling.width;
  ps->height = s->host.sampling.height;
  PoolScene* raw = ps.get();
  sv->scenes.push_back(std::move(ps));
  return raw;
}

void release_job(gprt_server* sv, SrvJob* j) {
  if (j->running) {
    j->running = false;
    sv->n_running--;
  }
  if (j->ps) {
    j->ps->refs--;
    j->ps = nullptr;
  }
  if (!j->bd && !j->bufs.empty() && sv->film_cache.size() < kFilmCacheMax) {
    cudaEventRecord(sv->rb_done, sv->rb_stream);
    gprt_server::CachedFilm c;
    c.npix = j->npix;
    c.adaptive = j->adaptive;
    c.bufs = std::move(j->bufs);
    c.film = j->film;
    c.d_list = j->d_list;
    c.bytes = j->film_bytes;
    sv->film_cache_bytes += c.bytes;
    sv->film_cache.push_back(std::move(c));
    j->bufs.clear();
  }
  free_all(j->bufs);
  if (j->bd_scene) {
    gprt_scene_destroy(j->bd_scene);  // and the job on it
    j->bd_scene = nullptr;
    j->bd = nullptr;
  }
  j->film_bytes = 0;  // freed, or counted in the film cache
}

// Moves the job past passes that need no new samples; finishes it after its
// last pass (RenderProgressive stops at max passes or when the average
// sample count reaches the maximum, progressive.go:339-361).
void advance(gprt_server* sv, SrvJob* j, bool emit_pass) {
  if (emit_pass) {
    j->passes++;
    emit(sv, j->ticket, GPRT_EV_PASS, j->passes, j->spp_done, GPRT_OK, j->submit_ms);
  }
  for (;;) {
    if (j->passes >= j->desc.max_passes || j->spp_done >= j->desc.max_samples_per_pixel) {
      emit(sv, j->ticket, GPRT_EV_DONE, j->passes, j->spp_done, GPRT_OK, j->submit_ms);
      sv->st.finished++;
      if (j->running) {
        j->running = false;
        sv->n_running--;
      }
      if (j->ps) {
        j->ps->refs--;
        j->ps->last_use = sv->st.steps;
        j->ps = nullptr;
      }
      return;
    }
    j->pass_target = samples_for_pass(j->desc, j->passes + 1);
    if (j->adaptive) {
      // shouldStopSampling's minimum (tile_renderer.go:79); the pass ends
      // when a round lists no active pixel
      j->min_s = std::max(1u, (uint32_t)((double)j->pass_target * j->min_frac));
      j->active = 0;
      return;
    }
    if (j->pass_target > j->spp_done) return;
    j->passes++;
    emit(sv, j->ticket, GPRT_EV_PASS, j->passes, j->spp_done, GPRT_OK, j->submit_ms);
  }
}

// Admits pending requests in arrival order while they fit.
void admit(gprt_server* sv) {
  gprt_ctx* ctx = sv->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);  // keeps pending scenes alive
  for (;;) {
    SrvRequest r;
    {
      std::lock_guard<std::mutex> q(sv->qmu);
      if (sv->pending.empty()) return;
      r = sv->pending.front();
    }
    if (sv->jobs.size() >= sv->desc.max_jobs) return;
    gprt_scene* s = r.scene;
    uint32_t npix = s->host.sampling.width * s->host.sampling.height;
    const bool adapt = s->host.sampling.adaptive_min_samples < 1.0;
    size_t cnt[kPoolArrays];
    scene_counts(s, cnt);
    bool resident = false;
    for (auto& ps : sv->scenes) resident |= ps->serial == r.serial;
    size_t fixed = sv->path_bytes + sv->table_bytes;
    size_t need = film_bytes_for(npix, adapt) + (resident ? 0 : scene_bytes(sv, cnt));
    auto pop = [&]() {
      std::lock_guard<std::mutex> q(sv->qmu);
      sv->pending.pop_front();
    };
    if (r.desc.integrator == GPRT_INTEGRATOR_BDPT) {
      // film + subpath working set + the private scene copy
      size_t need_b = bdpt_job_bytes(s, r.desc) + s->bytes;
      if (fixed + need_b > sv->desc.hbm_budget_bytes) {
        pop();
        sv->st.refused++;
        emit(sv, r.ticket, GPRT_EV_REFUSED, 0, 0, GPRT_E_ADMISSION, r.submit_ms);
        continue;
      }
      drop_film_cache(sv, need_b);
      if (bytes_in_use(sv) + need_b > sv->desc.hbm_budget_bytes) {
        bool freed = false;  // unreferenced cached scenes go first
        for (auto& ps : sv->scenes)
          if (ps->refs == 0) {
            evict(sv, ps.get());
            freed = true;
            break;
          }
        if (freed) {
          shrink_if_empty(sv);
          continue;
        }
        return;  // waits for running jobs to finish
      }
      gprt_scene* copy = nullptr;
      gprt_job* bj = nullptr;
      int rc = clone_scene(s, &copy);
      if (rc == GPRT_OK) rc = gprt_job_create(copy, &r.desc, &bj);
      if (rc != GPRT_OK) {
        if (copy) gprt_scene_destroy(copy);
        if (rc == GPRT_E_OOM) return;  // device full: retry next step
        pop();
        sv->st.refused++;
        emit(sv, r.ticket, GPRT_EV_REFUSED, 0, 0, rc, r.submit_ms);
        continue;
      }
      auto j = std::make_unique<SrvJob>();
      j->ticket = r.ticket;
      j->desc = r.desc;
      j->npix = npix;
      j->submit_ms = r.submit_ms;
      j->bd_scene = copy;
      j->bd = bj;
      j->film_bytes = need_b;
      j->adaptive = adapt;
      j->min_frac = s->host.sampling.adaptive_min_samples;
      j->threshold = (float)s->host.sampling.adaptive_threshold;
      j->admit_ms = now_ms(sv->t0);
      pop();
      sv->st.admitted++;
      sv->n_running++;
      emit(sv, r.ticket, GPRT_EV_ADMITTED, 0, 0, GPRT_OK, r.submit_ms);
      SrvJob* raw = j.get();
      sv->jobs[r.ticket] = std::move(j);
      advance(sv, raw, false);
      continue;
    }
    if (npix > sv->capacity || fixed + need > sv->desc.hbm_budget_bytes) {
      pop();
      sv->st.refused++;
      emit(sv, r.ticket, GPRT_EV_REFUSED, 0, 0, GPRT_E_ADMISSION, r.submit_ms);
      continue;
    }
    // films must fit beside everything held now (scene bytes are checked as the pool grows)
    drop_film_cache(sv, film_bytes_for(npix, adapt));
    if (bytes_in_use(sv) + film_bytes_for(npix, adapt) > sv->desc.hbm_budget_bytes) {
      // unreferenced cached scenes go first
      bool freed = false;
      for (auto& ps : sv->scenes)
        if (ps->refs == 0 && ps->serial != r.serial) {
          evict(sv, ps.get());
          freed = true;
          break;
        }
      if (freed) {
        shrink_if_empty(sv);
        continue;
      }
      return;
    }
    auto j = std::make_unique<SrvJob>();
    j->ticket = r.ticket;
    j->desc = r.desc;
    j->npix = npix;
    j->submit_ms = r.submit_ms;
    DevFilm& f = j->film;
    f.width = (int)s->host.sampling.width;
    f.height = (int)s->host.sampling.height;
    int rc = 0;
    bool reused = false;
    for (size_t c = 0; c < sv->film_cache.size(); c++) {
      gprt_server::CachedFilm& cf = sv->film_cache[c];
      if (cf.npix != npix || cf.adaptive != adapt) continue;
      j->bufs = std::move(cf.bufs);
      f.rgbl = cf.film.rgbl;
      f.lum2 = cf.film.lum2;
      f.count = cf.film.count;
      j->d_list = cf.d_list;
      sv->film_cache_bytes -= cf.bytes;
      sv->film_cache.erase(sv->film_cache.begin() + (ptrdiff_t)c);
      cudaStreamWaitEvent(sv->stream, sv->rb_done, 0);  // reads queued before its release end first
      reused = true;
      break;
    }
    if (!reused) {
      rc |= dev_alloc(ctx, j->bufs, &f.rgbl, npix);
      rc |= dev_alloc(ctx, j->bufs, &f.lum2, npix);
      rc |= dev_alloc(ctx, j->bufs, &f.count, npix);
      if (adapt) rc |= dev_alloc(ctx, j->bufs, &j->d_list, (size_t)npix + 1);
    }
    if (rc) {
      free_all(j->bufs);
      return;  // device full: retry next step
    }
    sv->reserve = film_bytes_for(npix, adapt);  // the scene may not take the film's room
    PoolScene* ps = make_resident(sv, s);
    sv->reserve = 0;
    if (!ps) {
      free_all(j->bufs);
      return;  // waits for films and scenes to be released
    }
    cudaMemsetAsync(f.rgbl, 0, (size_t)npix * sizeof(float4), sv->stream);
    cudaMemsetAsync(f.lum2, 0, (size_t)npix * sizeof(float), sv->stream);
    cudaMemsetAsync(f.count, 0, (size_t)npix * sizeof(uint32_t), sv->stream);
    j->film_bytes = film_bytes_for(npix, adapt);
    j->adaptive = adapt;
    j->min_frac = s->host.sampling.adaptive_min_samples;
    j->threshold = (float)s->host.sampling.adaptive_threshold;
    ps->refs++;
    ps->last_use = sv->st.steps;
    j->ps = ps;
    j->admit_ms = now_ms(sv->t0);
    pop();
    sv->st.admitted++;
    sv->n_running++;
    emit(sv, r.ticket, GPRT_EV_ADMITTED, 0, 0, GPRT_OK, r.submit_ms);
    SrvJob* raw = j.get();
    sv->jobs[r.ticket] = std::move(j);
    advance(sv, raw, false);
  }
}

int grid_for(gprt_server* sv, int block) { return std::max(1, sv->ctx->sm_count * (2048 / block)); }

// Kernels of a step of depth D: raygen, D x (extend, shade, shadow), accumulate.
int kernels_per_step(int D) { return 2 + 3 * D; }

// The slot-order kernel runs before each shading launch (timed with it).
bool has_slot_order(const gprt_server* sv) { return sv->P.order != nullptr; }

// Kernel class of launch k of a step (0 extend, 1 shade, 2 shadow, 3 other).
int kernel_class(int k, int D) { return (k == 0 || k == kernels_per_step(D) - 1) ? 3 : (k - 1) % 3; }

// Event pairs bracketing every kernel of a depth-D step (created once).
std::vector<cudaEvent_t>* events_for(gprt_server* sv, int D) {
  auto& v = sv->step_events[D];
  if (v.empty()) {
    v.resize(2 * kernels_per_step(D));
    for (auto& e : v) cudaEventCreate(&e);
  }
  return &v;
}

// The kernel sequence of one step of depth D on the server stream.  While
// the stream is being captured, the timing events become event-record nodes
// of the graph (cudaEventRecordExternal), so they fire on every replay.
void launch_step(gprt_server* sv, int D, cudaStream_t st, bool capturing) {
  DevScene pool = pool_view(sv);
  DevPaths P = sv->P;
  P.variant = sv->flags & kVariantBits;
  P.stats = (sv->flags & GPRT_JOB_COUNT_TRAVERSAL) ? sv->d_stats : nullptr;
  const StepHdr* hdr = reinterpret_cast<const StepHdr*>(sv->d_table);
  const uint32_t* path0 = reinterpret_cast<const uint32_t*>(sv->d_table + 16);
  // device bounds are reported per item: a path's origin index is its index
  // in the step, so path0 maps it to its item
  P.item_err = reinterpret_cast<uint32_t*>(sv->d_table + sv->err_off);
  P.item_start = path0;
  P.n_items = reinterpret_cast<const uint32_t*>(sv->d_table);  // StepHdr::n_items
  const uint32_t* pix0 = path0 + (sv->desc.max_jobs + 1);
  const DevItem* items = reinterpret_cast<const DevItem*>(sv->d_table + sv->prefix_bytes);
  int block = (int)sv->block;
  int grid = grid_for(sv, block);
  std::vector<cudaEvent_t>* ev = (sv->flags & GPRT_JOB_TIME_KERNELS) ? events_for(sv, D) : nullptr;
  int k = 0;
  unsigned rec = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  auto open = [&]() {
    if (ev) cudaEventRecordWithFlags((*ev)[2 * k], st, rec);
  };
  auto close = [&]() {
    if (ev) cudaEventRecordWithFlags((*ev)[2 * k + 1], st, rec);
    k++;
  };
  open();
  k_srv_raygen<<<grid, block, 0, st>>>(P, hdr, path0, items);
  close();
  int cur = 0;
  for (int b = 0; b < D; b++) {
    open();
    launch_pt_extend(pool, P, cur, b, block, grid, st);
    close();
    open();
    k_srv_hit_order<<<std::max(1, std::min((int)((sv->step_paths + 1023) / 1024), sv->ctx->sm_count * 2)), 1024, 0,
                      st>>>(pool, P, cur);
    if (P.variant & GPRT_JOB_SHADE_OCCUPANCY)
      k_srv_shade<192, 3><<<std::max(1, grid * block / 192), 192, 0, st>>>(pool, P, items, cur, b);
    else
      k_srv_shade<256, 2><<<grid, std::min(block, 256), 0, st>>>(pool, P, items, cur, b);
    close();
    open();
    launch_pt_shadow(pool, P, cur, block, grid, st);
    close();
    cur ^= 1;
  }
  open();
  k_srv_accumulate<<<grid, block, 0, st>>>(P, hdr, pix0, items);
  close();
}

// Folds the kernel times of the step just synchronised (and the traversal
// counters) into sv->acc.
void collect_step_counters(gprt_server* sv, int D) {
  if (sv->flags & GPRT_JOB_TIME_KERNELS) {
    auto& ev = *events_for(sv, D);
    for (int k = 0; k < kernels_per_step(D); k++) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      switch (kernel_class(k, D)) {
        case 0: sv->acc.extend_ms += ms; sv->acc.extend_launches++; break;
        case 1: sv->acc.shade_ms += ms; sv->acc.shade_launches++; break;
        case 2: sv->acc.shadow_ms += ms; sv->acc.shadow_launches++; break;
        default: sv->acc.other_ms += ms; sv->acc.other_launches++; break;
      }
    }
  }
  if ((sv->flags & GPRT_JOB_COUNT_TRAVERSAL) && sv->d_stats) {
    unsigned long long v[8];
    cudaMemcpy(v, sv->d_stats, sizeof(v), cudaMemcpyDeviceToHost);
    cudaMemset(sv->d_stats, 0, sizeof(v));
    sv->acc.extend_rays += v[0];
    sv->acc.extend_nodes += v[1];
    sv->acc.extend_boxes += v[2];
    sv->acc.extend_prims += v[3];
    sv->acc.shadow_rays += v[4];
    sv->acc.shadow_nodes += v[5];
    sv->acc.shadow_boxes += v[6];
    sv->acc.shadow_prims += v[7];
  }
}

void drop_graphs(gprt_server* sv) {
  for (auto& kv : sv->graphs) cudaGraphExecDestroy(kv.second);
  sv->graphs.clear();
  cudaGetLastError();
}

int run_step(gprt_server* sv, int D) {
  gprt_ctx* ctx = sv->ctx;
  sv->st.kernels += (uint64_t)kernels_per_step(D) + (has_slot_order(sv) ? (uint64_t)D : 0u);  // + slot orders
  if (sv->flags & GPRT_SERVER_NO_GRAPHS) {
    launch_step(sv, D, sv->stream, false);
    return GPRT_OK;
  }
  if (sv->graph_gen != sv->pool_gen) {
    drop_graphs(sv);
    sv->graph_gen = sv->pool_gen;
  }
  auto it = sv->graphs.find(D);
  if (it == sv->graphs.end()) {
    if (sv->flags & GPRT_JOB_TIME_KERNELS) events_for(sv, D);  // created outside the capture
    cudaGraph_t g = nullptr;
    CK(ctx, cudaStreamBeginCapture(sv->stream, cudaStreamCaptureModeThreadLocal));
    launch_step(sv, D, sv->stream, true);
    CK(ctx, cudaStreamEndCapture(sv->stream, &g));
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph instantiate");
    it = sv->graphs.emplace(D, ex).first;
  }
  CK(ctx, cudaGraphLaunch(it->second, sv->stream));
  sv->st.graph_launches++;
  return GPRT_OK;
}

struct Item {
  SrvJob* j;
  uint32_t layers;
  uint32_t npix;                   // pixels taking `layers` samples each
  const uint32_t* list = nullptr;  // those pixels (an adaptive round), null: every pixel
};

// The next work of a running path-tracing job: `layers` samples for `npix`
// pixels (a pixel list for an adaptive round).  Returns false when the job
// has none until its next round is listed.
bool next_work(const SrvJob* j, uint32_t& layers, uint32_t& npix, const uint32_t*& list) {
  npix = j->npix;
  list = nullptr;
  if (!j->adaptive) {
    layers = j->pass_target - j->spp_done;
    return layers > 0;
  }
  if (j->uniform >= 0 && (uint64_t)j->uniform < j->min_s) {  // nobody stops before the minimum: bulk
    layers = (uint32_t)(j->min_s - (uint64_t)j->uniform);
    return true;
  }
  if (!j->active) return false;
  layers = 1;
  npix = j->active;
  list = j->d_list;
  return true;
}

// Packs the next samples of the running jobs (least recently served first)
// into one wavefront of at most step_paths paths.
std::vector<Item> pack(gprt_server* sv, bool firsts_only) {
  std::vector<SrvJob*> order;
  for (auto& kv : sv->jobs)
    if (kv.second->running && !kv.second->bd && (!firsts_only || kv.second->passes == 0))
      order.push_back(kv.second.get());
  // jobs before their first pass first, the smallest first pass first (a
  // burst of arrivals then shows small images at once and does not wait
  // behind the first pass of a 1024^2 job), then the least recently served
  std::stable_sort(order.begin(), order.end(), [](const SrvJob* a, const SrvJob* b) {
    bool fa = a->passes == 0, fb = b->passes == 0;
    if (fa != fb) return fa;
    if (fa) {
      uint32_t la = 0, na = 0, lb = 0, nb = 0;
      const uint32_t *xa, *xb;
      uint64_t wa = next_work(a, la, na, xa) ? (uint64_t)la * na : 0;
      uint64_t wb = next_work(b, lb, nb, xb) ? (uint64_t)lb * nb : 0;
      if (wa != wb) return wa < wb;
    }
    return a->last_served < b->last_served;
  });
  std::vector<Item> items;
  uint64_t used = 0;
  for (SrvJob* j : order) {
    if (items.size() >= sv->desc.max_jobs) break;
    uint32_t want = 0, np = 0;
    const uint32_t* list = nullptr;
    if (!next_work(j, want, np, list)) continue;
    uint64_t fit = (sv->step_paths - used) / np;
    uint32_t layers = (uint32_t)std::min<uint64_t>(want, fit);
    if (layers == 0) continue;
    items.push_back({j, layers, np, list});
    used += (uint64_t)layers * np;
  }
  return items;
}

// Uploads the item table of a step; returns the depth of the step.
int upload_items(gprt_server* sv, const std::vector<Item>& items, bool dry, uint64_t* paths) {
  uint32_t nmax = sv->desc.max_jobs;
  StepHdr* hdr = reinterpret_cast<StepHdr*>(sv->h_table);
  uint32_t* path0 = reinterpret_cast<uint32_t*>(sv->h_table + 16);
  uint32_t* pix0 = path0 + (nmax + 1);
  DevItem* it = reinterpret_cast<DevItem*>(sv->h_table + sv->prefix_bytes);
  uint32_t pp = 0, px = 0;
  int D = 0;
  for (size_t k = 0; k < items.size(); k++) {
    SrvJob* j = items[k].j;
    PoolScene* ps = j->ps;
    DevItem& d = it[k];
    std::memset(&d, 0, sizeof(d));
    path0[k] = pp;
    pix0[k] = px;
    d.path0 = pp;
    d.pix0 = px;
    d.npix = items[k].npix;
    d.list = items[k].list;
    d.layers = items[k].layers;
    d.root = ps->root;
    d.mat_off = (int)ps->off[kMats];
    d.light_off = (int)ps->off[kLights];
    d.n_lights = (int)ps->cnt[kLights];
    d.tex_off = (int)ps->off[kTexInfo];
    d.texel_off = (int)ps->off[kTexels];
    d.has_textures = ps->cnt[kTexInfo] ? 1 : 0;
    d.has_tri_uvs = ps->has_tri_uvs;
    d.has_infinite = ps->has_infinite;
    d.max_depth = ps->max_depth;
    d.rr_min_bounces = ps->rr_min;
    d.width = (int)ps->width;
    d.world_center = ps->world_center;
    d.world_radius = ps->world_radius;
    d.seed = j->desc.seed;
    d.rgbl = j->film.rgbl;
    d.lum2 = j->film.lum2;
    d.count = j->film.count;
    d.cam = ps->cam;
    pp += items[k].layers * items[k].npix;
    px += items[k].npix;
    D = std::max(D, ps->max_depth);
  }
  uint32_t n = (uint32_t)items.size();
  path0[n] = pp;
  pix0[n] = px;
  hdr->n_items = n;
  hdr->total_paths = pp;
  hdr->total_pix = px;
  hdr->dry = dry ? 1u : 0u;
  *paths = pp;
  cudaMemcpyAsync(sv->d_table, sv->h_table, sv->prefix_bytes, cudaMemcpyHostToDevice, sv->stream);
  cudaMemcpyAsync(sv->d_table + sv->prefix_bytes, sv->h_table + sv->prefix_bytes, n * sizeof(DevItem),
                  cudaMemcpyHostToDevice, sv->stream);
  return D;
}

// Lists the next round of every adaptive job whose bulk samples are taken
// and whose round is not listed yet: one k_active_pixels launch per job on
// the server stream (after the step that took its last samples) and one
// read-back of the counts.  A job with no active pixel has finished its pass
// (then its next pass is listed at once, as gprt_job_render_pass ends a
// pass that needs no sample).
int list_rounds(gprt_server* sv) {
  gprt_ctx* ctx = sv->ctx;
  for (int again = 0; again < 64; again++) {
    std::vector<SrvJob*> js;
    for (auto& kv : sv->jobs) {
      SrvJob* j = kv.second.get();
      if (!j->running || j->bd || !j->adaptive || j->active) continue;
      if (j->uniform >= 0 && (uint64_t)j->uniform < j->min_s) continue;  // its bulk samples come first
      if (js.size() >= sv->desc.max_jobs) break;
      js.push_back(j);
    }
    if (js.empty()) return GPRT_OK;
    for (size_t k = 0; k < js.size(); k++) {
      SrvJob* j = js[k];
      CK(ctx, cudaMemsetAsync(j->d_list + j->npix, 0, sizeof(uint32_t), sv->stream));
      launch_active_pixels(j->film, j->pass_target, j->min_s, j->threshold, j->d_list, j->d_list + j->npix,
                           sv->stream);
      CK(ctx, cudaMemcpyAsync(sv->h_act + k, j->d_list + j->npix, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                              sv->stream));
    }
    CK(ctx, cudaStreamSynchronize(sv->stream));
    bool passed = false;
    for (size_t k = 0; k < js.size(); k++) {
      SrvJob* j = js[k];
      j->active = sv->h_act[k];
      if (j->active == 0) {
        advance(sv, j, true);
        passed = true;
      }
    }
    if (!passed) return GPRT_OK;
  }
  return GPRT_OK;
}

// One batched path-tracing wavefront over the running path-tracing jobs
// (only those before their first pass with `firsts_only`), and its events
// (work queued on other streams before it shares the GPU with it).  Returns
// the number of items run (0: none) or a negative status.
int pt_step(gprt_server* sv, bool dry, double* ms_out, bool firsts_only) {
  gprt_ctx* ctx = sv->ctx;
  if (!dry) {
    int rc = list_rounds(sv);
    if (rc) return rc;
  }
  std::vector<Item> items = pack(sv, firsts_only);
  if (items.empty()) return 0;
  uint64_t paths = 0;
  int D = upload_items(sv, items, dry, &paths);
  CK(ctx, cudaEventRecord(sv->ev0, sv->stream));
  int rc = run_step(sv, D);
  if (rc) return rc;
  CK(ctx, cudaEventRecord(sv->ev1, sv->stream));
  CK(ctx, cudaMemcpyAsync(sv->h_err, sv->d_table + sv->err_off, items.size() * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, sv->stream));
  CK(ctx, cudaStreamSynchronize(sv->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, sv->ev0, sv->ev1);
  if (ms_out) *ms_out = ms;
  if (dry) return (int)items.size();
  collect_step_counters(sv, D);
  sv->st.steps++;
  sv->st.busy_ms += ms;
  sv->st.last_step_ms = ms;
  sv->st.paths += paths;
  // a device bound fails only the jobs whose paths exceeded it (the
  // reference scopes errors to the render they occur in); the others keep
  // this step's samples
  for (size_t k = 0; k < items.size(); k++) {
    SrvJob* j = items[k].j;
    if (!sv->h_err[k]) continue;
    fail(ctx, GPRT_E_BOUND, "device bound exceeded (traversal stack) in job " + std::to_string(j->ticket));
    emit(sv, j->ticket, GPRT_EV_FAILED, j->passes, j->spp_done, GPRT_E_BOUND, j->submit_ms);
    release_job(sv, j);
    items[k].j = nullptr;
  }
  for (const Item& it : items) {
    SrvJob* j = it.j;
    if (!j) continue;
    j->last_served = sv->st.steps;
    sv->st.samples += (uint64_t)it.layers * it.npix;
    if (j->ps) j->ps->last_use = sv->st.steps;
    if (j->adaptive) {
      j->total += (uint64_t)it.layers * it.npix;
      if (j->uniform >= 0) j->uniform = it.npix == j->npix ? j->uniform + it.layers : -1;
      j->spp_done = (uint32_t)(j->total / j->npix);
      j->active = 0;  // the round is taken; list_rounds lists the next one
      continue;
    }
    j->spp_done += it.layers;
    if (j->spp_done >= j->pass_target) advance(sv, j, true);
  }
  return (int)items.size();
}

// BDPT samples rendered per step at most (whole samples per pixel, at least
// one) after a job's first pass: about 3 ms of Cornell-boxes BDPT, so a
// step that carries BDPT work stays short.  A first pass is rendered whole
// in one step (up to kBdptFirstPassSamples; about 11 ms for a 512^2 job at
// 4 spp) on the high-priority stream, instead of one slice per step behind
// the path-tracing wavefront.
constexpr uint64_t kBdptStepSamples = 1u << 18;
constexpr uint64_t kBdptFirstPassSamples = 1u << 22;

// The BDPT job served next: jobs still before their first pass first, the
// oldest request of those first (a burst then finishes its first passes one
// after another instead of all at the end), then the least recently served;
// null when none runs.
SrvJob* next_bdpt(gprt_server* sv) {
  SrvJob* pick = nullptr;
  auto before = [](const SrvJob* a, const SrvJob* b) {
    bool fa = a->passes == 0, fb = b->passes == 0;
    if (fa != fb) return fa;
    if (fa) return a->submit_ms < b->submit_ms || (a->submit_ms == b->submit_ms && a->ticket < b->ticket);
    return a->last_served < b->last_served;
  };
  for (auto& kv : sv->jobs) {
    SrvJob* j = kv.second.get();
    if (j->bd && j->running && (!pick || before(j, pick))) pick = j;
  }
  return pick;
}

// Completes the work queued for BDPT job j (status rc of the launch): `n`
// samples per pixel, or, for an adaptive job, `taken` samples in all (a
// bulk slice or one round; `done`: the round listed no active pixel, so the
// pass is complete); waits for it and emits its events.
void finish_bdpt(gprt_server* sv, SrvJob* j, uint32_t n, uint64_t taken, bool done, int rc, cudaStream_t own) {
  if (rc == GPRT_OK) rc = gprt_job_sync(j->bd);
  if (own) {  // back to the job's own stream (the pass ran on bd_first)
    cudaStreamSynchronize(j->bd->stream);
    j->bd->stream = own;
  }
  if (rc != GPRT_OK) {
    emit(sv, j->ticket, GPRT_EV_FAILED, j->passes, j->spp_done, rc, j->submit_ms);
    release_job(sv, j);
    return;
  }
  j->last_served = ++sv->bd_rounds;
  sv->st.samples += taken;
  if (j->adaptive) {
    j->total += taken;
    j->spp_done = (uint32_t)(j->total / j->npix);
    if (done) advance(sv, j, true);
    return;
  }
  j->spp_done += n;
  if (j->spp_done >= j->pass_target) advance(sv, j, true);
}

// Consecutive steps that may carry first passes only, before one step serves
// the running jobs' later passes again (so that a sustained stream of
// arrivals cannot starve them).
constexpr uint32_t kMaxFirstsSteps = 8;

// BDPT first passes started together in one first-passes step at most.
constexpr size_t kMaxBdptFirsts = 4;

// One step: admission, the next samples of one BDPT job's pass (RenderPass
// of one job, progressive.go:126-223: all pixels take the pass's new
// samples; splats are applied after each slice) and one batched
// path-tracing wavefront beside it; then the events of both.  A BDPT job's
// first pass is rendered whole and queued before the wavefront so that its
// blocks are first in line, the oldest waiting one on the high-priority
// stream and up to kMaxBdptFirsts - 1 more on their own streams beside it;
// later passes go in slices of kBdptStepSamples on the job's own stream.
// While any job waits for its first pass, the step carries first passes
// only (time to first pass before throughput), at most kMaxFirstsSteps
// steps in a row.
// Returns the number of items run (0: nothing to do) or a negative status.
int step_impl(gprt_server* sv, bool dry, double* ms_out) {
  if (!dry) admit(sv);
  SrvJob* bj = dry ? nullptr : next_bdpt(sv);
  bool firsts = false;
  if (!dry) {
    bool waiting = bj && bj->passes == 0;
    for (auto& kv : sv->jobs)
      if (!waiting && kv.second->running && !kv.second->bd && kv.second->passes == 0) waiting = true;
    firsts = waiting && sv->firsts_run < kMaxFirstsSteps;
    sv->firsts_run = firsts ? sv->firsts_run + 1 : 0;
    if (firsts && bj && bj->passes != 0) bj = nullptr;  // its later pass waits too
  }
  // the BDPT work of this step: one job's next slice or adaptive round; in a
  // first-passes step, every BDPT job still before its first pass (up to
  // kMaxBdptFirsts, oldest first), each on its own stream and the oldest on
  // the priority stream, so a burst's BDPT first passes run side by side
  // instead of one step after another
  struct BdWork {
    SrvJob* j;
    uint32_t bn = 0;
    uint64_t taken = 0;
    bool round_empty = false;
    int rc = GPRT_OK;
    cudaStream_t own = nullptr;
  };
  std::vector<BdWork> bw;
  if (bj) {
    bw.push_back({bj});
    if (firsts && bj->passes == 0) {
      std::vector<SrvJob*> more;
      for (auto& kv : sv->jobs)
        if (kv.second->bd && kv.second->running && kv.second->passes == 0 && kv.second.get() != bj)
          more.push_back(kv.second.get());
      std::sort(more.begin(), more.end(), [](const SrvJob* a, const SrvJob* b) {
        return a->submit_ms < b->submit_ms || (a->submit_ms == b->submit_ms && a->ticket < b->ticket);
      });
      for (SrvJob* m : more)
        if (bw.size() < kMaxBdptFirsts) bw.push_back({m});
    }
  }
  for (size_t k = 0; k < bw.size(); k++) {
    BdWork& w = bw[k];
    SrvJob* j = w.j;
    bool first = j->passes == 0;
    uint64_t cap = first ? kBdptFirstPassSamples : kBdptStepSamples;
    uint64_t per = std::max<uint64_t>(1, cap / std::max<uint32_t>(1, j->npix));
    if (first && k == 0 && sv->bd_first) {
      w.own = j->bd->stream;
      j->bd->stream = sv->bd_first;
    }
    const int64_t uni = j->bd->uniform_count;
    if (!j->adaptive || (uni >= 0 && (uint64_t)uni < j->min_s)) {
      // whole samples per pixel: the pass (or, adaptive, its minimum) in slices
      uint32_t want = j->adaptive ? (uint32_t)(j->min_s - (uint64_t)uni) : j->pass_target - j->spp_done;
      w.bn = (uint32_t)std::min<uint64_t>(want, per);
      w.taken = (uint64_t)w.bn * j->npix;
      w.rc = gprt_job_add_samples(j->bd, w.bn);  // queued on the first-pass (or the job's) stream
    } else {
      // one round: a sample for each pixel still active (listed on the device)
      uint32_t active = 0;
      w.rc = job_adaptive_round(j->bd, j->pass_target, j->min_s, j->threshold, &active);
      w.taken = active;
      w.round_empty = active == 0;
    }
  }
  int n = pt_step(sv, dry, ms_out, firsts);
  for (BdWork& w : bw) finish_bdpt(sv, w.j, w.bn, w.taken, w.round_empty, w.rc, w.own);
  if (n < 0) return n;
  return n + (int)bw.size();
}

SrvJob* find_job(gprt_server* sv, uint64_t ticket) {
  auto it = sv->jobs.find(ticket);
  return it == sv->jobs.end() ? nullptr : it->second.get();
}

void loop_main(gprt_server* sv) {
  cudaSetDevice(sv->ctx->device);
  for (;;) {
    uint64_t gen;
    {
      std::unique_lock<std::mutex> lk(sv->qmu);
      sv->cv_work.wait(lk, [&] { return sv->stopping || !sv->pending.empty() || sv->n_running.load() > 0; });
      if (sv->stopping) return;
      gen = sv->work_gen;
    }
    int did;
    {
      std::lock_guard<std::mutex> g(sv->smu);
      did = step_impl(sv, false, nullptr);
    }
    if (did <= 0) {
      // nothing could run (requests wait for memory): sleep until something changes
      std::unique_lock<std::mutex> lk(sv->qmu);
      sv->cv_work.wait_for(lk, std::chrono::milliseconds(5), [&] { return sv->stopping || sv->work_gen != gen; });
    }
  }
}

void notify_work(gprt_server* sv) {
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    sv->work_gen++;
  }
  sv->cv_work.notify_all();
}

int stop_loop(gprt_server* sv) {
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    if (!sv->loop_running) return GPRT_OK;
    sv->stopping = true;
  }
  sv->cv_work.notify_all();
  sv->loop.join();
  std::lock_guard<std::mutex> lk(sv->qmu);
  sv->stopping = false;
  sv->loop_running = false;
  return GPRT_OK;
}

// Read-back of an admitted job's image: kind 0 RGBA8 (vec3ToColor), 1 the
// mean radiance, 2 the RGBA8 of the tile rect = {x0, y0, x1, y1} (only the
// tile's bytes are resolved and copied: extractTileImage,
// progressive.go:225-255).  The resolve and the device-to-host copy are
// queued on the read-back stream behind an event on the step stream (the
// film as of every step queued so far), and the wait and the host copy
// happen outside smu, so the loop thread keeps stepping meanwhile; rmu keeps
// one read at a time on the staging buffers.  A release in between frees the
// film with cudaFree, which waits for the queued resolve.
int read_job(gprt_server* sv, uint64_t ticket, int kind, void* out, const uint32_t* rect = nullptr) {
  std::lock_guard<std::mutex> r(sv->rmu);
  gprt_ctx* ctx = sv->ctx;
  size_t bytes = 0;
  {
    std::lock_guard<std::mutex> g(sv->smu);
    cudaSetDevice(ctx->device);
    SrvJob* j = find_job(sv, ticket);
    if (!j) return fail(ctx, GPRT_E_NOT_FOUND, "unknown or released ticket");
    if (j->bd)  // BDPT: the per-job film (splats included)
      return kind == 0   ? gprt_job_read_rgba8(j->bd, static_cast<uint8_t*>(out))
             : kind == 1 ? gprt_job_read_image(j->bd, static_cast<float*>(out))
                         : gprt_job_read_tile(j->bd, rect[0], rect[1], rect[2], rect[3], static_cast<uint8_t*>(out));
    if (j->bufs.empty()) return fail(ctx, GPRT_E_NOT_FOUND, "the job's film was released");
    if (kind == 2 && (rect[2] <= rect[0] || rect[3] <= rect[1] || rect[2] > (uint32_t)j->film.width ||
                      rect[3] > (uint32_t)j->film.height))
      return fail(ctx, GPRT_E_INVALID, "tile outside the image");
    size_t npix = kind == 2 ? (size_t)(rect[2] - rect[0]) * (rect[3] - rect[1]) : (size_t)j->npix;
    bytes = kind == 1 ? npix * 3 * sizeof(float) : npix * 4;
    if (bytes > sv->rb_bytes) {  // no read is in flight (rmu)
      free_all(sv->rb_bufs);
      sv->rb = nullptr;
      sv->rb_bytes = 0;
      if (dev_alloc(ctx, sv->rb_bufs, &sv->rb, bytes)) return GPRT_E_OOM;
      sv->rb_bytes = bytes;
    }
    if (bytes > sv->rb_host_bytes) {
      if (sv->rb_host) cudaFreeHost(sv->rb_host);
      sv->rb_host = nullptr;
      sv->rb_host_bytes = 0;
      void* h = nullptr;
      if (cudaHostAlloc(&h, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, GPRT_E_OOM, "pinned read-back buffer");
      }
      sv->rb_host = static_cast<unsigned char*>(h);
      sv->rb_host_bytes = bytes;
    }
    uint8_t* d = sv->rb;
    CK(ctx, cudaEventRecord(sv->rb_ev, sv->stream));
    CK(ctx, cudaStreamWaitEvent(sv->rb_stream, sv->rb_ev, 0));
    if (kind == 0) launch_resolve_rgba8(j->film, d, sv->rb_stream);
    else if (kind == 1) launch_image_mean(j->film, reinterpret_cast<float*>(d), sv->rb_stream);
    else launch_resolve_tile(j->film, rect[0], rect[1], rect[2], rect[3], d, sv->rb_stream);
    CK(ctx, cudaMemcpyAsync(sv->rb_host, d, bytes, cudaMemcpyDeviceToHost, sv->rb_stream));
  }
  cudaError_t e = cudaStreamSynchronize(sv->rb_stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "server read-back");
  std::memcpy(out, sv->rb_host, bytes);
  return GPRT_OK;
}

}  // namespace

namespace gprt {
void server_forget_scene(gprt_server* sv, gprt_scene* s) {
  std::vector<SrvRequest> gone;
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    for (auto it = sv->pending.begin(); it != sv->pending.end();) {
      if (it->scene == s) {
        gone.push_back(*it);
        it = sv->pending.erase(it);
      } else {
        ++it;
      }
    }
  }
  for (auto& r : gone) {
    sv->st.cancelled++;
    emit(sv, r.ticket, GPRT_EV_CANCELLED, 0, 0, GPRT_E_CANCELLED, r.submit_ms);
  }
}
}  // namespace gprt

extern "C" {

int gprt_server_create(gprt_ctx* ctx, const gprt_server_desc* desc, gprt_server** out) {
  if (!ctx || !out) return GPRT_E_INVALID;
  *out = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  auto sv = std::make_unique<gprt_server>();
  sv->ctx = ctx;
  if (desc) sv->desc = *desc;
  gprt_server_desc& d = sv->desc;
  if (d.hbm_budget_bytes == 0) d.hbm_budget_bytes = 60ull << 30;
  if (d.max_jobs == 0) d.max_jobs = 1024;
  if (d.step_paths == 0) d.step_paths = 1u << 22;
  if (d.block_size == 0) d.block_size = 128;
  if (d.block_size % 32 || d.block_size > 1024) return fail(ctx, GPRT_E_INVALID, "block_size must be a multiple of 32, <= 1024");
  if (d.max_jobs > (1u << 20)) return fail(ctx, GPRT_E_INVALID, "max_jobs above 2^20");
  sv->t0 = std::chrono::steady_clock::now();
  sv->capacity = d.step_paths;
  sv->step_paths = d.step_paths;
  sv->block = d.block_size;
  sv->flags = d.flags;
  sv->pool[kNodes].elem[0] = 8 * sizeof(float4);
  sv->pool[kTris].elem[0] = 3 * sizeof(float4);
  sv->pool[kTris].elem[1] = sizeof(float4);
  sv->pool[kTris].elem[2] = 2 * sizeof(float4);  // TriangleMeshOptions.VertexUVs
  sv->pool[kQuads].elem[0] = 5 * sizeof(float4);
  sv->pool[kSpheres].elem[0] = 2 * sizeof(float4);
  sv->pool[kQuadrics].elem[0] = 5 * sizeof(float4);
  sv->pool[kMats].elem[0] = sizeof(DevMaterial);
  sv->pool[kLights].elem[0] = sizeof(DevLight);
  sv->pool[kTexInfo].elem[0] = sizeof(uint4);
  sv->pool[kTexels].elem[0] = sizeof(float4);
  // path state of one step
  DevPaths& P = sv->P;
  auto& b = sv->path_bufs;
  uint32_t cap = sv->capacity;
  size_t bytes = path_region_bytes(cap, true);
  unsigned char* region = nullptr;
  int rc = dev_alloc(ctx, b, &region, bytes);
  if (!rc && (d.flags & GPRT_JOB_COUNT_TRAVERSAL)) rc = dev_alloc(ctx, b, &sv->d_stats, 8);
  if (rc) {
    free_all(b);
    return GPRT_E_OOM;
  }
  carve_paths(region, cap, true, P);
  P.capacity = cap;
  P.stats = nullptr;
  sv->path_bytes = bytes;
  sv->prefix_bytes = (16 + 2 * (size_t)(d.max_jobs + 1) * 4 + 255) & ~(size_t)255;
  sv->err_off = (sv->prefix_bytes + (size_t)d.max_jobs * sizeof(DevItem) + 255) & ~(size_t)255;
  sv->act_off = (sv->err_off + (size_t)d.max_jobs * sizeof(uint32_t) + 255) & ~(size_t)255;
  sv->table_bytes = sv->act_off + (size_t)d.max_jobs * sizeof(uint32_t);
  if (sv->path_bytes + sv->table_bytes > d.hbm_budget_bytes) {
    free_all(b);
    return fail(ctx, GPRT_E_ADMISSION, "the budget does not cover the path state of one step");
  }
  if (dev_alloc(ctx, b, &sv->d_table, sv->table_bytes) ||
      cudaMallocHost(reinterpret_cast<void**>(&sv->h_table), sv->table_bytes + 256) != cudaSuccess) {
    cudaGetLastError();
    free_all(b);
    return fail(ctx, GPRT_E_OOM, "item table allocation failed");
  }
  sv->h_err = reinterpret_cast<uint32_t*>(sv->h_table + sv->err_off);
  sv->h_act = reinterpret_cast<uint32_t*>(sv->h_table + sv->act_off);
  if (cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free_all(b);
    cudaFreeHost(sv->h_table);
    return fail(ctx, GPRT_E_DEVICE, "stream creation failed");
  }
  cudaEventCreate(&sv->ev0);
  cudaEventCreate(&sv->ev1);
  if (cudaStreamCreateWithFlags(&sv->rb_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&sv->rb_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&sv->rb_done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    free_all(b);
    cudaFreeHost(sv->h_table);
    cudaStreamDestroy(sv->stream);
    if (sv->rb_stream) cudaStreamDestroy(sv->rb_stream);
    return fail(ctx, GPRT_E_DEVICE, "read-back stream creation failed");
  }
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
      cudaStreamCreateWithPriority(&sv->bd_first, cudaStreamNonBlocking, greatest) != cudaSuccess) {
    cudaGetLastError();
    sv->bd_first = nullptr;  // first passes then run on the job's own stream
  }
  cudaMemsetAsync(P.counters, 0, 8 * sizeof(uint32_t), sv->stream);
  if (sv->d_stats) cudaMemsetAsync(sv->d_stats, 0, 8 * sizeof(unsigned long long), sv->stream);
  cudaError_t e = cudaStreamSynchronize(sv->stream);
  if (e != cudaSuccess) {
    free_all(b);
    cudaFreeHost(sv->h_table);
    if (sv->bd_first) cudaStreamDestroy(sv->bd_first);
    cudaStreamDestroy(sv->rb_stream);
    cudaEventDestroy(sv->rb_ev);
    cudaEventDestroy(sv->rb_done);
    return cuda_fail(ctx, e, "server init");
  }
  ctx->servers.insert(sv.get());
  *out = sv.release();
  return GPRT_OK;
}

int gprt_server_destroy(gprt_server* sv) {
  if (!sv) return GPRT_E_INVALID;
  gprt_ctx* ctx = sv->ctx;
  stop_loop(sv);
  {
    std::lock_guard<std::mutex> r(sv->rmu);  // no read in flight
    std::lock_guard<std::mutex> g(sv->smu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(sv->stream);
    cudaStreamSynchronize(sv->rb_stream);
    for (auto& kv : sv->jobs) {
      kv.second->running = false;  // the server is going: no counters to keep
      release_job(sv, kv.second.get());
    }
    sv->jobs.clear();
    sv->scenes.clear();
    for (auto& a : sv->pool)
      for (int b = 0; b < gprt::PoolArray::kBufs; b++)
        if (a.buf[b]) cudaFree(a.buf[b]);
    drop_graphs(sv);
    for (auto& kv : sv->step_events)
      for (auto e : kv.second) cudaEventDestroy(e);
    drop_film_cache(sv, SIZE_MAX);
    free_all(sv->path_bufs);
    free_all(sv->rb_bufs);
    if (sv->rb_host) cudaFreeHost(sv->rb_host);
    if (sv->h_table) cudaFreeHost(sv->h_table);
    cudaEventDestroy(sv->ev0);
    cudaEventDestroy(sv->ev1);
    cudaStreamDestroy(sv->stream);
    cudaStreamDestroy(sv->rb_stream);
    cudaEventDestroy(sv->rb_ev);
    cudaEventDestroy(sv->rb_done);
    if (sv->bd_first) cudaStreamDestroy(sv->bd_first);
  }
  {
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    ctx->servers.erase(sv);
  }
  delete sv;
  return GPRT_OK;
}

int gprt_server_submit(gprt_server* sv, gprt_scene* s, const gprt_job_desc* desc, uint64_t* ticket) {
  if (!sv || !s || !desc || s->ctx != sv->ctx) return GPRT_E_INVALID;
  gprt_ctx* ctx = sv->ctx;
  if (desc->integrator != GPRT_INTEGRATOR_PATH_TRACING && desc->integrator != GPRT_INTEGRATOR_BDPT)
    return fail(ctx, GPRT_E_INVALID, "unknown integrator");
  gprt_job_desc d = *desc;
  if (d.initial_samples == 0) d.initial_samples = 1;
  if (d.max_samples_per_pixel == 0) d.max_samples_per_pixel = 50;
  if (d.max_passes == 0) d.max_passes = 7;
  if (d.max_samples_per_pixel < d.initial_samples) return fail(ctx, GPRT_E_INVALID, "max samples below initial samples");
  SrvRequest r;
  r.scene = s;
  r.serial = s->serial;
  r.desc = d;
  r.submit_ms = now_ms(sv->t0);
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    r.ticket = sv->next_ticket++;
    sv->pending.push_back(r);
    sv->st.submitted++;
    sv->work_gen++;
  }
  sv->cv_work.notify_all();
  if (ticket) *ticket = r.ticket;
  return GPRT_OK;
}

int gprt_server_cancel(gprt_server* sv, uint64_t ticket) {
  if (!sv) return GPRT_E_INVALID;
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    for (auto it = sv->pending.begin(); it != sv->pending.end(); ++it)
      if (it->ticket == ticket) {
        double sm = it->submit_ms;
        sv->pending.erase(it);
        sv->st.cancelled++;
        gprt_event e{};
        e.ticket = ticket;
        e.kind = GPRT_EV_CANCELLED;
        e.status = GPRT_E_CANCELLED;
        e.t_ms = now_ms(sv->t0);
        e.submit_ms = sm;
        sv->events.push_back(e);
        sv->cv_ev.notify_all();
        return GPRT_OK;
      }
  }
  std::lock_guard<std::mutex> g(sv->smu);
  SrvJob* j = find_job(sv, ticket);
  if (!j) return fail(sv->ctx, GPRT_E_NOT_FOUND, "unknown ticket");
  if (j->running) {
    sv->st.cancelled++;
    emit(sv, ticket, GPRT_EV_CANCELLED, j->passes, j->spp_done, GPRT_E_CANCELLED, j->submit_ms);
  }
  cudaSetDevice(sv->ctx->device);
  cudaStreamSynchronize(sv->stream);
  release_job(sv, j);
  sv->jobs.erase(ticket);
  notify_work(sv);
  return GPRT_OK;
}

int gprt_server_step(gprt_server* sv, uint32_t* busy) {
  if (!sv) return GPRT_E_INVALID;
  int rc;
  {
    std::lock_guard<std::mutex> g(sv->smu);
    cudaSetDevice(sv->ctx->device);
    rc = step_impl(sv, false, nullptr);
  }
  if (busy) {
    std::lock_guard<std::mutex> lk(sv->qmu);
    *busy = sv->n_running.load() + (uint32_t)sv->pending.size();
  }
  return rc < 0 ? rc : GPRT_OK;
}

int gprt_server_start(gprt_server* sv) {
  if (!sv) return GPRT_E_INVALID;
  std::lock_guard<std::mutex> lk(sv->qmu);
  if (sv->loop_running) return GPRT_OK;
  sv->stopping = false;
  sv->loop_running = true;
  sv->loop = std::thread(loop_main, sv);
  return GPRT_OK;
}

int gprt_server_stop(gprt_server* sv) {
  if (!sv) return GPRT_E_INVALID;
  return stop_loop(sv);
}

int gprt_server_poll(gprt_server* sv, gprt_event* events, uint32_t max, uint32_t timeout_ms, uint32_t* n) {
  if (!sv || (max && !events)) return GPRT_E_INVALID;
  std::unique_lock<std::mutex> lk(sv->qmu);
  if (sv->events.empty() && timeout_ms)
    sv->cv_ev.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !sv->events.empty(); });
  uint32_t k = 0;
  while (k < max && !sv->events.empty()) {
    events[k++] = sv->events.front();
    sv->events.pop_front();
  }
  if (n) *n = k;
  return GPRT_OK;
}

int gprt_server_read_film(gprt_server* sv, uint64_t ticket, float* rgb_sum, float* lum_sum, float* lum2_sum,
                          uint32_t* count) {
  if (!sv) return GPRT_E_INVALID;
  std::lock_guard<std::mutex> g(sv->smu);
  gprt_ctx* ctx = sv->ctx;
  cudaSetDevice(ctx->device);
  SrvJob* j = find_job(sv, ticket);
  if (j && j->bd) return gprt_job_read_film(j->bd, rgb_sum, lum_sum, lum2_sum, count);
  if (!j || j->bufs.empty()) return fail(ctx, GPRT_E_NOT_FOUND, "unknown or released ticket");
  uint32_t npix = j->npix;
  CK(ctx, cudaStreamSynchronize(sv->stream));
  if (rgb_sum || lum_sum) {
    std::vector<float4> v(npix);
    CK(ctx, cudaMemcpy(v.data(), j->film.rgbl, (size_t)npix * sizeof(float4), cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < npix; i++) {
      if (rgb_sum) {
        rgb_sum[3 * i] = v[i].x;
        rgb_sum[3 * i + 1] = v[i].y;
        rgb_sum[3 * i + 2] = v[i].z;
      }
      if (lum_sum) lum_sum[i] = v[i].w;
    }
  }
  if (lum2_sum) CK(ctx, cudaMemcpy(lum2_sum, j->film.lum2, (size_t)npix * 4, cudaMemcpyDeviceToHost));
  if (count) CK(ctx, cudaMemcpy(count, j->film.count, (size_t)npix * 4, cudaMemcpyDeviceToHost));
  return GPRT_OK;
}

int gprt_server_read_image(gprt_server* sv, uint64_t ticket, float* rgb_mean) {
  if (!sv || !rgb_mean) return GPRT_E_INVALID;
  return read_job(sv, ticket, 1, rgb_mean);
}

int gprt_server_read_rgba8(gprt_server* sv, uint64_t ticket, uint8_t* rgba) {
  if (!sv || !rgba) return GPRT_E_INVALID;
  return read_job(sv, ticket, 0, rgba);
}

int gprt_server_read_tile(gprt_server* sv, uint64_t ticket, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                          uint8_t* rgba) {
  if (!sv || !rgba) return GPRT_E_INVALID;
  const uint32_t rect[4] = {x0, y0, x1, y1};
  return read_job(sv, ticket, 2, rgba, rect);
}

int gprt_server_release(gprt_server* sv, uint64_t ticket) { return gprt_server_cancel(sv, ticket); }

int gprt_server_get_stats(gprt_server* sv, gprt_server_stats* out) {
  if (!sv || !out) return GPRT_E_INVALID;
  std::lock_guard<std::mutex> g(sv->smu);
  gprt_server_stats s = sv->st;
  {
    std::lock_guard<std::mutex> lk(sv->qmu);
    s.pending_jobs = (uint32_t)sv->pending.size();
    s.submitted = sv->st.submitted;
    s.cancelled = sv->st.cancelled;
  }
  s.active_jobs = sv->n_running.load();
  s.resident_scenes = (uint32_t)sv->scenes.size();
  s.bytes_in_use = bytes_in_use(sv);
  s.bytes_budget = sv->desc.hbm_budget_bytes;
  s.pool_bytes = 0;
  for (auto& a : sv->pool) s.pool_bytes += a.bytes();
  s.path_state_bytes = sv->path_bytes;
  s.step_paths = sv->step_paths;
  s.block_size = sv->block;
  s.flags = sv->flags;
  s.max_jobs = sv->desc.max_jobs;
  *out = s;
  return GPRT_OK;
}

int gprt_server_get_counters(gprt_server* sv, gprt_job_counters* out, int reset) {
  if (!sv || !out) return GPRT_E_INVALID;
  std::lock_guard<std::mutex> g(sv->smu);
  *out = sv->acc;
  if (reset) sv->acc = gprt_job_counters{};
  return GPRT_OK;
}

int gprt_server_stream(gprt_server* sv, void** stream) {
  if (!sv || !stream) return GPRT_E_INVALID;
  *stream = sv->stream;
  return GPRT_OK;
}

int gprt_server_configure(gprt_server* sv, uint32_t step_paths, uint32_t block_size, uint32_t flags) {
  if (!sv) return GPRT_E_INVALID;
  std::lock_guard<std::mutex> g(sv->smu);
  if ((flags & GPRT_JOB_COUNT_TRAVERSAL) && !sv->d_stats) {
    if (dev_alloc(sv->ctx, sv->path_bufs, &sv->d_stats, 8)) return GPRT_E_OOM;
    cudaMemset(sv->d_stats, 0, 8 * sizeof(unsigned long long));
  }
  if (step_paths == 0 || step_paths > sv->capacity) return fail(sv->ctx, GPRT_E_INVALID, "step_paths above the capacity");
  if (block_size == 0 || block_size % 32 || block_size > 1024) return fail(sv->ctx, GPRT_E_INVALID, "bad block_size");
  sv->step_paths = step_paths;
  if (sv->block != block_size || sv->flags != flags) {
    sv->block = block_size;
    sv->flags = flags;
    drop_graphs(sv);
  }
  return GPRT_OK;
}

int gprt_server_autotune(gprt_server* sv, double max_step_ms, gprt_tune_result* out) {
  if (!sv || !out) return GPRT_E_INVALID;
  std::lock_guard<std::mutex> g(sv->smu);
  gprt_ctx* ctx = sv->ctx;
  cudaSetDevice(ctx->device);
  admit(sv);
  if (pack(sv, false).empty()) return fail(ctx, GPRT_E_INVALID, "autotune needs admitted, unfinished jobs");
  uint32_t keep_paths = sv->step_paths, keep_block = sv->block, keep_flags = sv->flags;
  // samples per ms of dry steps (no film is changed) of the current jobs
  auto rate = [&](uint32_t paths, uint32_t block, uint32_t flags, double* step_ms) -> double {
    sv->step_paths = paths;
    if (sv->block != block || sv->flags != flags) {
      sv->block = block;
      sv->flags = flags;
      drop_graphs(sv);
    }
    std::vector<Item> items = pack(sv, false);
    uint64_t n = 0;
    for (auto& it : items) n += (uint64_t)it.layers * it.npix;
    double ms = 0;
    if (step_impl(sv, true, &ms) <= 0) return -1.0;  // warm-up (and graph capture)
    double total = 0;
    for (int r = 0; r < 2; r++) {
      if (step_impl(sv, true, &ms) <= 0) return -1.0;
      total += ms;
    }
    *step_ms = total / 2;
    return *step_ms > 0 ? (double)n / *step_ms : -1.0;
  };
  std::vector<uint32_t> sizes;
  for (uint32_t p = sv->capacity; p >= (1u << 18) && sizes.size() < 5; p >>= 1) sizes.push_back(p);
  double step_ms = 0;
  double best = rate(keep_paths, keep_block, keep_flags, &step_ms);
  double default_ms = step_ms;
  uint32_t bp = keep_paths, bb = keep_block, bf = keep_flags;
  bool best_ok = max_step_ms <= 0 || step_ms <= max_step_ms;
  uint32_t tried = 1;
  auto consider = [&](uint32_t p, uint32_t b, uint32_t f) {
    double ms = 0;
    double r = rate(p, b, f, &ms);
    tried++;
    if (r <= 0) return;
    bool ok = max_step_ms <= 0 || ms <= max_step_ms;
    if ((ok && !best_ok) || (ok == best_ok && r > best)) {
      best = r;
      best_ok = ok;
      bp = p;
      bb = b;
      bf = f;
      out->best_ms = ms;
    }
  };
  out->best_ms = step_ms;
  for (uint32_t p : sizes)
    if (p != keep_paths) consider(p, bb, bf);
  for (uint32_t b : {64u, 128u, 256u})
    if (b != bb) consider(bp, b, bf);
  uint32_t trav_bits = GPRT_JOB_SIMPLE_EXTEND | GPRT_JOB_SIMPLE_SHADOW;
  for (uint32_t v : {0u, (uint32_t)GPRT_JOB_SIMPLE_EXTEND, (uint32_t)GPRT_JOB_SIMPLE_SHADOW})
    if (v != (bf & trav_bits)) consider(bp, bb, (bf & ~trav_bits) | v);
  consider(bp, bb, bf ^ GPRT_JOB_SHADE_OCCUPANCY);
  sv->step_paths = bp;
  if (sv->block != bb || sv->flags != bf) {
    sv->block = bb;
    sv->flags = bf;
    drop_graphs(sv);
  }
  (void)keep_block;
  out->flags = bf;
  out->block_size = bb;
  out->chunk_paths = bp;
  out->candidates = tried;
  out->default_ms = default_ms;
  return GPRT_OK;
}

}  // extern "C"
