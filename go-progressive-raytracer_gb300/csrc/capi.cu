// capi.cu - the C ABI of include/gprt.h: context, scene and job handles and
// the host orchestration of the kernels (chunked wavefront passes).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>

#include "handles.h"

namespace {

// BDPT working set: counters, per-sample radiance and the strategy buffers.
int ensure_bdpt(gprt_job* j) {
  gprt_ctx* ctx = j->scene->ctx;
  uint32_t ns = j->desc.chunk_paths;
  DevPaths& P = j->paths;
  DevBdpt& B = P.bd;
  B.maxv = bdpt_maxv(j->scene->dev.max_depth);
  B.ns = ns;
  auto& b = j->buffers;
  int rc = 0;
  rc |= dev_alloc(ctx, b, &P.counters, 64);
  rc |= dev_alloc(ctx, b, &P.Lout, ns);
  for (int k = 0; k < 5; k++) rc |= dev_alloc(ctx, b, &B.v[k], (size_t)ns * 2 * B.maxv);
  rc |= dev_alloc(ctx, b, &B.pdf, (size_t)ns * 2 * B.maxv);
  for (int k = 0; k < 2; k++) {
    BdQueue& q = B.q[k];
    rc |= dev_alloc(ctx, b, &q.o, ns);
    rc |= dev_alloc(ctx, b, &q.d, ns);
    rc |= dev_alloc(ctx, b, &q.beta, ns);
    rc |= dev_alloc(ctx, b, &q.last, ns);
    rc |= dev_alloc(ctx, b, &q.ids, ns);
    rc |= dev_alloc(ctx, b, &q.st, ns);
  }
  rc |= dev_alloc(ctx, b, &B.hit, ns);
  rc |= dev_alloc(ctx, b, &B.lorig, (size_t)ns * 3);
  rc |= dev_alloc(ctx, b, &B.meta, ns);
  rc |= dev_alloc(ctx, b, &B.masks, ns);
  rc |= dev_alloc(ctx, b, &B.contrib, (size_t)ns * (B.maxv + 1) * B.maxv);
  B.uv = nullptr;
  if (j->scene->dev.has_textures) rc |= dev_alloc(ctx, b, &B.uv, (size_t)ns * 2 * B.maxv);
  rc |= dev_alloc(ctx, b, &B.slist, (size_t)ns * (B.maxv + 1) * B.maxv);
  B.nw = bdpt_windows(ns);
  const size_t nk = (size_t)B.nw * (B.maxv + 1) * B.maxv;
  rc |= dev_alloc(ctx, b, &B.scount, nk);
  rc |= dev_alloc(ctx, b, &B.sprefix, 4 * (nk + 1));
  if (rc) return GPRT_E_OOM;
  P.stats = nullptr;
  P.variant = 0;
  CK(ctx, cudaMemsetAsync(P.counters, 0, 8 * sizeof(uint32_t), j->stream));
  P.capacity = ns;
  return GPRT_OK;
}

int ensure_paths(gprt_job* j) {
  if (j->paths.capacity) return GPRT_OK;
  if (j->desc.integrator == GPRT_INTEGRATOR_BDPT) return ensure_bdpt(j);
  gprt_ctx* ctx = j->scene->ctx;
  uint32_t cap = j->desc.chunk_paths;
  DevPaths& P = j->paths;
  unsigned char* region = nullptr;
  int rc = dev_alloc(ctx, j->buffers, &region, path_region_bytes(cap, false));
  if (!rc && (j->desc.flags & GPRT_JOB_COUNT_TRAVERSAL)) rc = dev_alloc(ctx, j->buffers, &j->d_stats, 8);
  if (rc) return GPRT_E_OOM;
  carve_paths(region, cap, false, P);
  P.stats = j->d_stats;
  P.variant = j->desc.flags & kVariantBits;
  CK(ctx, cudaMemsetAsync(P.counters, 0, 8 * sizeof(uint32_t), j->stream));
  if (j->d_stats) CK(ctx, cudaMemsetAsync(j->d_stats, 0, 8 * sizeof(unsigned long long), j->stream));
  return GPRT_OK;
}

// Runs one chunk: `layers` samples of `npix` pixels starting at pix0.
// CUDA-event bracket of one launch on the job stream (when timing is on).
struct TimedLaunch {
  gprt_job* j;
  size_t idx = (size_t)-1;
  TimedLaunch(gprt_job* job, int cls) : j(job) {
    if (!(j->desc.flags & GPRT_JOB_TIME_KERNELS)) return;
    if (j->timed_used == j->timed.size()) {
      gprt_job::Timed t{cls, nullptr, nullptr};
      cudaEventCreate(&t.a);
      cudaEventCreate(&t.b);
      j->timed.push_back(t);
    }
    idx = j->timed_used++;
    j->timed[idx].cls = cls;
    cudaEventRecord(j->timed[idx].a, j->stream);
  }
  ~TimedLaunch() {
    if (idx != (size_t)-1) cudaEventRecord(j->timed[idx].b, j->stream);
  }
};

// Folds the recorded launch times and the device counters into j->acc.
int collect_counters(gprt_job* j) {
  gprt_ctx* ctx = j->scene->ctx;
  CK(ctx, cudaStreamSynchronize(j->stream));
  for (size_t i = 0; i < j->timed_used; i++) {
    float ms = 0;
    cudaEventElapsedTime(&ms, j->timed[i].a, j->timed[i].b);
    switch (j->timed[i].cls) {
      case 0: j->acc.extend_ms += ms; j->acc.extend_launches++; break;
      case 1: j->acc.shade_ms += ms; j->acc.shade_launches++; break;
      case 2: j->acc.shadow_ms += ms; j->acc.shadow_launches++; break;
      default: j->acc.other_ms += ms; j->acc.other_launches++; break;
    }
  }
  j->timed_used = 0;
  if (j->d_stats) {
    unsigned long long v[8];
    CK(ctx, cudaMemcpy(v, j->d_stats, sizeof(v), cudaMemcpyDeviceToHost));
    CK(ctx, cudaMemset(j->d_stats, 0, sizeof(v)));
    j->acc.extend_rays += v[0];
    j->acc.extend_nodes += v[1];
    j->acc.extend_boxes += v[2];
    j->acc.extend_prims += v[3];
    j->acc.shadow_rays += v[4];
    j->acc.shadow_nodes += v[5];
    j->acc.shadow_boxes += v[6];
    j->acc.shadow_prims += v[7];
  }
  return GPRT_OK;
}

void run_chunk(gprt_job* j, const ChunkDesc& ch) {
  const DevScene& sc = j->scene->dev;
  gprt_ctx* ctx = j->scene->ctx;
  int block = (int)j->desc.block_size;
  int grid = std::max(1, ctx->sm_count * (2048 / block));
  uint32_t n = ch.npix * ch.layers;
  int g = launch_grid(n, block, grid);
  if (j->desc.integrator == GPRT_INTEGRATOR_BDPT) {
    {
      TimedLaunch t(j, 3);
      launch_bdpt(sc, j->film, j->paths, ch, block, j->stream);
    }
    {
      TimedLaunch t(j, 3);
      launch_accumulate(j->film, j->paths, ch, 256, j->stream);
    }
    j->launches += 2;
    return;
  }
  {
    TimedLaunch t(j, 3);
    launch_pt_raygen(sc, j->film, j->paths, ch, block, j->stream);
  }
  int cur = 0;
  for (int b = 0; b < sc.max_depth; b++) {
    {
      TimedLaunch t(j, 0);
      launch_pt_extend(sc, j->paths, cur, b, block, g, j->stream);
    }
    {
      TimedLaunch t(j, 1);
      launch_pt_shade(sc, j->paths, ch, cur, b, block, g, j->stream);
    }
    {
      TimedLaunch t(j, 2);
      launch_pt_shadow(sc, j->paths, cur, block, g, j->stream);
    }
    cur ^= 1;
  }
  {
    TimedLaunch t(j, 3);
    launch_accumulate(j->film, j->paths, ch, 256, j->stream);
  }
  // raygen, accumulate; extend, (slot order,) shade, shadow per bounce
  j->launches += 2 + (uint64_t)(sc.has_infinite || sc.has_specular ? 4 : 3) * sc.max_depth;
}

// Adds `spp` samples to each of `npix` pixels (all pixels, or the list).
int add_samples(gprt_job* j, uint32_t spp, uint32_t npix, const uint32_t* list) {
  if (spp == 0 || npix == 0) return GPRT_OK;
  int rc = ensure_paths(j);
  if (rc) return rc;
  uint32_t cap = j->paths.capacity;
  ChunkDesc ch{};
  ch.pix_list = list;
  ch.seed = j->desc.seed;
  if (npix <= cap) {
    uint32_t per = std::max(1u, cap / npix);
    for (uint32_t done = 0; done < spp;) {
      uint32_t layers = std::min(per, spp - done);
      ch.pix0 = 0;
      ch.npix = npix;
      ch.layers = layers;
      run_chunk(j, ch);
      done += layers;
    }
  } else {
    for (uint32_t s = 0; s < spp; s++)
      for (uint32_t p0 = 0; p0 < npix; p0 += cap) {
        ch.pix0 = p0;
        ch.npix = std::min(cap, npix - p0);
        ch.layers = 1;
        run_chunk(j, ch);
      }
  }
  if (j->desc.integrator == GPRT_INTEGRATOR_BDPT) {
    launch_apply_splats(j->film, j->stream);
    j->launches++;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(j->scene->ctx, e, "kernel launch");
  return GPRT_OK;
}

int check_device_errors(gprt_job* j) {
  gprt_ctx* ctx = j->scene->ctx;
  j->h_words[0] = 0;
  if (j->paths.counters) {
    CK(ctx, cudaMemcpyAsync(j->h_words, j->paths.counters + 3, 4, cudaMemcpyDeviceToHost, j->stream));
  }
  CK(ctx, cudaStreamSynchronize(j->stream));
  uint32_t err = j->h_words[0];
  if (err) {
    return fail(ctx, GPRT_E_BOUND,
                std::string("device bound exceeded:") + ((err & kErrStackOverflow) ? " traversal stack" : ""));
  }
  return GPRT_OK;
}

// Uploads the primitive and node arrays of s->host (host-built BVH, and the
// server's private copies).
int upload_geometry(gprt_ctx* ctx, gprt_scene* s) {
  HostScene& h = s->host;
  DevScene& d = s->dev;
  int rc = 0;
  rc |= upload(ctx, s->buffers, h.nodes, &d.nodes, &s->bytes);
  rc |= upload(ctx, s->buffers, h.tris, &d.tris, &s->bytes);
  rc |= upload(ctx, s->buffers, h.tri_normals, &d.tri_normals, &s->bytes);
  rc |= upload(ctx, s->buffers, h.quads, &d.quads, &s->bytes);
  rc |= upload(ctx, s->buffers, h.spheres, &d.spheres, &s->bytes);
  rc |= upload(ctx, s->buffers, h.quadrics, &d.quadrics, &s->bytes);
  return rc;
}

// Uploads materials, lights and textures, sets the scalar fields of s->dev
// and waits for the copies; frees the scene's buffers on failure.
int upload_rest(gprt_ctx* ctx, gprt_scene* s) {
  HostScene& h = s->host;
  DevScene& d = s->dev;
  int rc = 0;
  rc |= upload(ctx, s->buffers, h.materials, &d.materials, &s->bytes);
  rc |= upload(ctx, s->buffers, h.lights, &d.lights, &s->bytes);
  rc |= upload(ctx, s->buffers, h.tri_uvs, &d.tri_uvs, &s->bytes);
  rc |= upload(ctx, s->buffers, h.tex_info, &d.tex_info, &s->bytes);
  rc |= upload(ctx, s->buffers, h.texels, &d.texels, &s->bytes);
  d.has_textures = h.tex_info.empty() ? 0 : 1;
  if (rc) {
    free_all(s->buffers);
    return rc;
  }
  if (dev_alloc(ctx, s->buffers, &s->d_err, 1)) {
    free_all(s->buffers);
    return GPRT_E_OOM;
  }
  cudaMemsetAsync(s->d_err, 0, sizeof(int), ctx->stream);
  if (h.nodes.size() / 8 >= (size_t)kMaxNodes) {
    free_all(s->buffers);
    return fail(ctx, GPRT_E_INVALID, "the scene's BVH has more than 2^30 nodes");
  }
  d.n_nodes = (int)(h.nodes.size() / 8);
  d.root = d.n_nodes > 0 ? (h.test_stack_cap ? kRootStackCap : 0) : -1;
  d.n_lights = (int)h.lights.size();
  d.quad_base = h.n_tris;
  d.sphere_base = h.n_tris + h.n_quads;
  d.quadric_base = h.n_tris + h.n_quads + h.n_spheres;
  d.n_prims = h.n_tris + h.n_quads + h.n_spheres + h.n_quadrics;
  if ((uint64_t)h.n_tris + h.n_quads + h.n_spheres + h.n_quadrics >= kOverflowHit) {
    free_all(s->buffers);
    return fail(ctx, GPRT_E_INVALID, "the scene has too many primitives for 32-bit primitive ids");
  }
  d.has_infinite = h.has_infinite;
  d.has_specular = 0;
  for (const DevMaterial& m : h.materials) d.has_specular |= m.kind == kMatMetal || m.kind == kMatDielectric;
  d.world_center = make_float3((float)h.world_center[0], (float)h.world_center[1], (float)h.world_center[2]);
  d.world_radius = (float)h.world_radius;
  d.cam = h.cam;
  d.max_depth = (int)h.sampling.max_depth;
  d.rr_min_bounces = (int)h.sampling.rr_min_bounces;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    free_all(s->buffers);
    return cuda_fail(ctx, e, "scene upload");
  }
  return GPRT_OK;
}

}  // namespace

extern "C" {

int gprt_version(void) { return GPRT_ABI_VERSION; }

int gprt_ctx_create(int device, gprt_ctx** out) {
  if (!out) return GPRT_E_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return GPRT_E_DEVICE;
  }
  auto c = std::make_unique<gprt_ctx>();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return GPRT_E_DEVICE;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return GPRT_E_DEVICE;
  if (cudaMallocHost(reinterpret_cast<void**>(&c->h_words), 64) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamDestroy(c->stream);
    return GPRT_E_OOM;
  }
  *out = c.release();
  return GPRT_OK;
}

int gprt_ctx_destroy(gprt_ctx* ctx) {
  if (!ctx) return GPRT_E_INVALID;
  // servers first: their loop threads take the context lock
  for (;;) {
    gprt_server* sv = nullptr;
    {
      std::lock_guard<std::recursive_mutex> lk(ctx->mu);
      if (ctx->servers.empty()) break;
      sv = *ctx->servers.begin();
    }
    gprt_server_destroy(sv);
  }
  {
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    while (!ctx->scenes.empty()) gprt_scene_destroy(*ctx->scenes.begin());
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    cudaFreeHost(ctx->h_words);
  }
  delete ctx;
  return GPRT_OK;
}

const char* gprt_last_error(const gprt_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gprt_scene_create(gprt_ctx* ctx, const gprt_scene_desc* desc, gprt_scene** out) {
  if (!ctx || !out) return GPRT_E_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  *out = nullptr;
  cudaSetDevice(ctx->device);
  auto s = std::make_unique<gprt_scene>();
  s->ctx = ctx;
  static std::atomic<uint64_t> next_serial{1};
  s->serial = next_serial++;
  std::string err;
  if (!build_scene(desc, s->host, err, (desc->build_flags & GPRT_BUILD_DEVICE) != 0))
    return fail(ctx, GPRT_E_INVALID, err);
  HostScene& h = s->host;
  h.test_stack_cap = (desc->build_flags & GPRT_BUILD_TEST_STACK_CAP) != 0;
  DevScene& d = s->dev;
  int rc = 0;
  if (h.device_bvh) {
    // BVH and primitive arrays built on the GPU (also remaps the light indices)
    rc = device_build_bvh(ctx, h, d, s->buffers, &s->bytes);
    if (rc) {
      free_all(s->buffers);
      return rc;
    }
    // mesh normals / UVs by final triangle id, now that the builder has filled the primitive maps
    apply_mesh_options(desc, h);
    if (h.custom_normals && h.n_tris)
      CK(ctx, cudaMemcpyAsync(const_cast<float4*>(d.tri_normals), h.tri_normals.data(), h.tri_normals.size() * 16,
                              cudaMemcpyHostToDevice, ctx->stream));
    // the tree is checked on the host copy before any kernel walks it
    auto tc = std::chrono::steady_clock::now();
    std::string bad = validate_layout(h);
    h.check_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tc).count();
    h.build_ms += h.check_ms;
    if (!bad.empty()) {
      free_all(s->buffers);
      return fail(ctx, GPRT_E_DEVICE, "device BVH build produced an invalid tree: " + bad);
    }
  } else {
    rc = upload_geometry(ctx, s.get());
    if (rc) {
      free_all(s->buffers);
      return rc;
    }
  }
  rc = upload_rest(ctx, s.get());
  if (rc) return rc;
  ctx->scenes.insert(s.get());
  *out = s.release();
  return GPRT_OK;
}

int gprt_scene_destroy(gprt_scene* s) {
  if (!s) return GPRT_E_INVALID;
  gprt_ctx* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  for (gprt_server* sv : ctx->servers) server_forget_scene(sv, s);
  while (!s->jobs.empty()) gprt_job_destroy(*s->jobs.begin());
  cudaStreamSynchronize(ctx->stream);
  free_all(s->buffers);
  ctx->scenes.erase(s);
  delete s;
  return GPRT_OK;
}

int gprt_scene_get_info(const gprt_scene* s, gprt_scene_info* info) {
  if (!s || !info) return GPRT_E_INVALID;
  const HostScene& h = s->host;
  std::memset(info, 0, sizeof(*info));
  for (int k = 0; k < 3; k++) info->world_center[k] = h.world_center[k];
  info->world_radius = h.world_radius;
  info->n_triangles = h.n_tris;
  info->n_quads = h.n_quads;
  info->n_spheres = h.n_spheres;
  info->n_quadrics = h.n_quadrics;
  info->n_primitives = (uint64_t)h.n_tris + h.n_quads + h.n_spheres + h.n_quadrics;
  info->n_nodes = h.nodes.size() / 8;
  info->device_bytes = s->bytes;
  info->image_width = h.sampling.width;
  info->image_height = h.sampling.height;
  info->build_ms = h.build_ms;
  info->flatten_ms = h.flatten_ms;
  info->bvh_ms = h.bvh_ms;
  info->check_ms = h.check_ms;
  return GPRT_OK;
}

int gprt_scene_validate(const gprt_scene_desc* desc, gprt_scene_info* info, char* errbuf, size_t err_len) {
  HostScene h;
  std::string err;
  bool ok = build_scene(desc, h, err);
  if (ok) err = validate_layout(h);
  if (errbuf && err_len) {
    std::strncpy(errbuf, err.c_str(), err_len - 1);
    errbuf[err_len - 1] = 0;
  }
  if (!ok || !err.empty()) return GPRT_E_INVALID;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    for (int k = 0; k < 3; k++) info->world_center[k] = h.world_center[k];
    info->world_radius = h.world_radius;
    info->n_triangles = h.n_tris;
    info->n_quads = h.n_quads;
    info->n_spheres = h.n_spheres;
    info->n_quadrics = h.n_quadrics;
    info->n_primitives = (uint64_t)h.n_tris + h.n_quads + h.n_spheres + h.n_quadrics;
    info->n_nodes = h.nodes.size() / 8;
    info->image_width = h.sampling.width;
    info->image_height = h.sampling.height;
    info->build_ms = h.build_ms;
    info->flatten_ms = h.flatten_ms;
    info->bvh_ms = h.bvh_ms;
  }
  return GPRT_OK;
}

int gprt_scene_primitive_map(const gprt_scene* s, uint32_t* shape_index, uint32_t* sub_index) {
  if (!s) return GPRT_E_INVALID;
  if (shape_index) std::memcpy(shape_index, s->host.prim_shape.data(), s->host.prim_shape.size() * 4);
  if (sub_index) std::memcpy(sub_index, s->host.prim_sub.data(), s->host.prim_sub.size() * 4);
  return GPRT_OK;
}

int gprt_intersect(gprt_scene* s, const gprt_ray* rays, uint32_t n, uint32_t flags, gprt_hit* hits, void* stream) {
  if (!s || (n && (!rays || !hits)) || flags > GPRT_ANY) return GPRT_E_INVALID;
  gprt_ctx* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  launch_intersect(s->dev, rays, n, flags == GPRT_ANY, hits, s->d_err, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "intersect launch");
  return GPRT_OK;
}

int gprt_intersect_host(gprt_scene* s, const gprt_ray* rays, uint32_t n, uint32_t flags, gprt_hit* hits) {
  if (!s || (n && (!rays || !hits)) || flags > GPRT_ANY) return GPRT_E_INVALID;
  gprt_ctx* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (n == 0) return GPRT_OK;
  std::vector<void*> tmp;
  gprt_ray* dr = nullptr;
  gprt_hit* dh = nullptr;
  if (dev_alloc(ctx, tmp, &dr, n) || dev_alloc(ctx, tmp, &dh, n)) {
    free_all(tmp);
    return GPRT_E_OOM;
  }
  cudaError_t e = cudaMemsetAsync(s->d_err, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dr, rays, (size_t)n * sizeof(gprt_ray), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    launch_intersect(s->dev, dr, n, flags == GPRT_ANY, dh, s->d_err, ctx->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hits, dh, (size_t)n * sizeof(gprt_hit), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  free_all(tmp);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "intersect_host");
  if (cudaMemcpyAsync(ctx->h_words, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    return cuda_fail(ctx, cudaGetLastError(), "intersect_host error word");
  if (ctx->h_words[0]) return fail(ctx, GPRT_E_BOUND, "device bound exceeded: traversal stack");
  return GPRT_OK;
}

int gprt_traversal_counts(gprt_scene* s, const gprt_ray* rays, uint32_t n, uint32_t flags, uint64_t* node_visits,
                          uint64_t* box_tests, uint64_t* prim_tests) {
  if (!s || (n && !rays)) return GPRT_E_INVALID;
  uint64_t a, b, c;
  count_traversal(s->host, rays, n, flags == GPRT_ANY, a, b, c);
  if (node_visits) *node_visits = a;
  if (box_tests) *box_tests = b;
  if (prim_tests) *prim_tests = c;
  return GPRT_OK;
}

int gprt_job_create(gprt_scene* s, const gprt_job_desc* desc, gprt_job** out) {
  if (!s || !desc || !out) return GPRT_E_INVALID;
  gprt_ctx* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  *out = nullptr;
  if (desc->integrator > GPRT_INTEGRATOR_BDPT) return fail(ctx, GPRT_E_INVALID, "unknown integrator");
  auto j = std::make_unique<gprt_job>();
  j->scene = s;
  j->desc = *desc;
  gprt_job_desc& d = j->desc;
  // DefaultProgressiveConfig (progressive.go:38-46)
  if (d.tile_size == 0) d.tile_size = 64;
  if (d.initial_samples == 0) d.initial_samples = 1;
  if (d.max_samples_per_pixel == 0) d.max_samples_per_pixel = 50;
  if (d.max_passes == 0) d.max_passes = 7;
  if (d.block_size == 0) d.block_size = 128;
  if (d.block_size % 32 || d.block_size > 1024) return fail(ctx, GPRT_E_INVALID, "block_size must be a multiple of 32, <= 1024");
  uint32_t npix = s->host.sampling.width * s->host.sampling.height;
  if (d.chunk_paths == 0) {
    uint64_t want = (uint64_t)npix * std::max(1u, d.max_samples_per_pixel);
    // path tracing: up to 2^24 paths per wavefront (about 4.6 GB of path
    // state); BDPT: 2^20 samples per chunk (3.5 GB of vertices and strategy
    // contributions at depth <= 9, 8.4 GB up to depth 17)
    d.chunk_paths = (uint32_t)std::min<uint64_t>(want, d.integrator == GPRT_INTEGRATOR_BDPT ? (1u << 20) : (1u << 24));
  }
  if (d.integrator == GPRT_INTEGRATOR_BDPT) d.chunk_paths = std::min(d.chunk_paths, 1u << 20);
  if (d.max_samples_per_pixel < d.initial_samples) return fail(ctx, GPRT_E_INVALID, "max samples below initial samples");
  if (d.integrator == GPRT_INTEGRATOR_BDPT && s->host.sampling.max_depth > 17)
    return fail(ctx, GPRT_E_INVALID, "BDPT supports max_depth <= 17 (18 stored vertices per subpath)");
  DevFilm& f = j->film;
  f.width = (int)s->host.sampling.width;
  f.height = (int)s->host.sampling.height;
  int rc = 0;
  rc |= dev_alloc(ctx, j->buffers, &f.rgbl, npix);
  rc |= dev_alloc(ctx, j->buffers, &f.lum2, npix);
  rc |= dev_alloc(ctx, j->buffers, &f.count, npix);
  rc |= dev_alloc(ctx, j->buffers, &f.splat, npix);
  rc |= dev_alloc(ctx, j->buffers, &j->d_pix_list, npix);
  rc |= dev_alloc(ctx, j->buffers, &j->d_active, 1);
  if (rc) {
    free_all(j->buffers);
    return GPRT_E_OOM;
  }
  if (cudaMallocHost(reinterpret_cast<void**>(&j->h_words), 16) != cudaSuccess) {
    cudaGetLastError();
    free_all(j->buffers);
    return fail(ctx, GPRT_E_OOM, "pinned job words");
  }
  if (cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free_all(j->buffers);
    cudaFreeHost(j->h_words);
    return fail(ctx, GPRT_E_DEVICE, "stream creation failed");
  }
  cudaEventCreate(&j->ev0);
  cudaEventCreate(&j->ev1);
  cudaMemsetAsync(f.rgbl, 0, (size_t)npix * sizeof(float4), j->stream);
  cudaMemsetAsync(f.lum2, 0, (size_t)npix * sizeof(float), j->stream);
  cudaMemsetAsync(f.count, 0, (size_t)npix * sizeof(uint32_t), j->stream);
  cudaMemsetAsync(f.splat, 0, (size_t)npix * sizeof(float4), j->stream);
  cudaError_t e = cudaStreamSynchronize(j->stream);
  if (e != cudaSuccess) {
    free_all(j->buffers);
    cudaFreeHost(j->h_words);
    cudaStreamDestroy(j->stream);
    return cuda_fail(ctx, e, "job init");
  }
  j->uniform_count = 0;
  s->jobs.insert(j.get());
  *out = j.release();
  return GPRT_OK;
}

int gprt_job_destroy(gprt_job* j) {
  if (!j) return GPRT_E_INVALID;
  gprt_ctx* ctx = j->scene->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(j->stream);
  free_all(j->buffers);
  cudaFreeHost(j->h_words);
  cudaStreamDestroy(j->stream);
  cudaEventDestroy(j->ev0);
  cudaEventDestroy(j->ev1);
  for (auto& t : j->timed) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  j->scene->jobs.erase(j);
  delete j;
  return GPRT_OK;
}

int gprt_job_add_samples(gprt_job* j, uint32_t spp) {
  if (!j) return GPRT_E_INVALID;
  gprt_ctx* ctx = j->scene->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  uint32_t npix = (uint32_t)j->film.width * j->film.height;
  int rc = add_samples(j, spp, npix, nullptr);
  if (rc) return rc;
  if (j->uniform_count >= 0) j->uniform_count += spp;
  return GPRT_OK;
}

int gprt_job_sync(gprt_job* j) {
  if (!j) return GPRT_E_INVALID;
  gprt_ctx* ctx = j->scene->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  return check_device_errors(j);
}

int gprt_job_render_pass(gprt_job* j, uint32_t pass, gprt_render_stats* stats) {
  if (!j || pass == 0) return GPRT_E_INVALID;
  gprt_ctx* ctx = j->scene->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const gprt_sampling_desc& sd = j->scene->host.sampling;
  uint32_t target = samples_for_pass(j->desc, pass);
  uint32_t npix = (uint32_t)j->film.width * j->film.height;
  // shouldStopSampling minimum (tile_renderer.go:79)
  uint32_t min_s = std::max(1u, (uint32_t)((double)target * sd.adaptive_min_samples));
  cudaEventRecord(j->ev0, j->stream);
  int rc = GPRT_OK;
  uint64_t before_launches = j->launches;
  if (j->uniform_count >= 0 && (uint64_t)j->uniform_count < min_s) {
    // nobody can stop before min_s: one bulk wave
    rc = add_samples(j, min_s - (uint32_t)j->uniform_count, npix, nullptr);
    if (rc) return rc;
    j->uniform_count = min_s;
  }
  if (min_s < target || j->uniform_count < 0 || (uint64_t)j->uniform_count < target) {
    // adaptive rounds of one sample per still-active pixel
    for (;;) {
      uint32_t active = 0;
      rc = gprt::job_adaptive_round(j, target, min_s, (float)sd.adaptive_threshold, &active);
      if (rc) return rc;
      if (active == 0) break;
    }
  }
  cudaEventRecord(j->ev1, j->stream);
  rc = check_device_errors(j);
  if (rc) return rc;
  float ms = 0;
  cudaEventElapsedTime(&ms, j->ev0, j->ev1);
  // assembleCurrentImage statistics (progressive.go:395-431)
  gprt_render_stats st{};
  st.total_pixels = npix;
  st.max_samples = target;
  st.pass_number = pass;
  st.pass_ms = ms;
  if (j->uniform_count >= 0) {
    st.total_samples = (uint64_t)j->uniform_count * npix;
    st.min_samples = std::min<uint32_t>(j->desc.max_samples_per_pixel, (uint32_t)j->uniform_count);
    st.max_samples_used = (uint32_t)j->uniform_count;
  } else {
    std::vector<uint32_t> cnt(npix);
    CK(ctx, cudaMemcpy(cnt.data(), j->film.count, (size_t)npix * 4, cudaMemcpyDeviceToHost));
    st.min_samples = j->desc.max_samples_per_pixel;
    for (uint32_t c : cnt) {
      st.total_samples += c;
      st.min_samples = std::min(st.min_samples, c);
      st.max_samples_used = std::max(st.max_samples_used, c);
    }
  }
  st.average_samples = (double)st.total_samples / (double)st.total_pixels;
  (void)before_launches;
  j->last = st;
  if (stats) *stats = st;
  return GPRT_OK;
}

int gprt_job_read_film(gprt_job* j, float* rgb_sum, float* lum_sum, float* lum2_sum, uint32_t* count) {
  if (!j) return GPRT_E_INVALID;
  gprt_ctx* ctx = j->scene->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  uint32_t npix = (uint32_t)j->film.width * j->film.height;
  CK(ctx, cudaStreamSynchronize(j->stream));
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

static int read_via_device(gprt_job* j, size_t bytes, int kind, void* out) {
  gprt_ctx* ctx = j->scene->ctx;
  std::vector<void*> tmp;
  uint8_t* d = nullptr;
  if (dev_alloc(ctx, tmp, &d, bytes)) return GPRT_E_OOM;
  if (kind == 0) launch_resolve_rgba8(j->film, d, j->stream);
  else launch_image_mean(j->film, reinterpret_cast<float*>(d), j->stream);
  j->launches++;
  cudaError_t e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, j->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(j->stream);
  free_all(tmp);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "image read-back");
  return GPRT_OK;
}

int gprt_job_read_image(gprt_job* j, float* rgb_mean) {
  if (!j || !rgb_mean) return GPRT_E_INVALID;
  std::lock_guard<std::recursive_mutex> lk(j->scene->ctx->mu);
  cudaSetDevice(j->scene->ctx->device);
  size_t npix = (size_t)j->film.width * j->film.height;
  return read_via_device(j, npix * 3 * sizeof(float), 1, rgb_mean);
}

int gprt_job_read_rgba8(gprt_job* j, uint8_t* rgba) {
  if (!j || !rgba) return GPRT_E_INVALID;
  std::lock_guard<std::recursive_mutex> lk(j->scene->ctx->mu);
  cudaSetDevice(j->scene->ctx->device);
  size_t npix = (size_t)j->film.width * j->film.height;
  return read_via_device(j, npix * 4, 0, rgba);
}

int gprt_job_read_tile(gprt_job* j, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, uint8_t* rgba) {
  if (!j || !rgba || x1 <= x0 || y1 <= y0 || x1 > (uint32_t)j->film.width || y1 > (uint32_t)j->film.height)
    return GPRT_E_INVALID;
  gprt_ctx* ctx = j->scene->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  // resolved on the device: only the tile's bytes cross to the host
  size_t bytes = (size_t)(x1 - x0) * (y1 - y0) * 4;
  std::vector<void*> tmp;
  uint8_t* d = nullptr;
  if (dev_alloc(ctx, tmp, &d, bytes)) return GPRT_E_OOM;
  launch_resolve_tile(j->film, x0, y0, x1, y1, d, j->stream);
  j->launches++;
  cudaError_t e = cudaMemcpyAsync(rgba, d, bytes, cudaMemcpyDeviceToHost, j->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(j->stream);
  free_all(tmp);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "tile read-back");
  return GPRT_OK;
}

int gprt_job_get_stats(gprt_job* j, gprt_render_stats* stats) {
  if (!j || !stats) return GPRT_E_INVALID;
  *stats = j->last;
  return GPRT_OK;
}

int gprt_job_launch_count(const gprt_job* j, uint64_t* launches) {
  if (!j || !launches) return GPRT_E_INVALID;
  *launches = j->launches;
  return GPRT_OK;
}

int gprt_job_get_counters(gprt_job* j, gprt_job_counters* out) {
  if (!j || !out) return GPRT_E_INVALID;
  std::lock_guard<std::recursive_mutex> lk(j->scene->ctx->mu);
  cudaSetDevice(j->scene->ctx->device);
  int rc = collect_counters(j);
  if (rc) return rc;
  *out = j->acc;
  return GPRT_OK;
}

int gprt_job_reset_counters(gprt_job* j) {
  if (!j) return GPRT_E_INVALID;
  std::lock_guard<std::recursive_mutex> lk(j->scene->ctx->mu);
  cudaSetDevice(j->scene->ctx->device);
  int rc = collect_counters(j);
  j->acc = gprt_job_counters{};
  return rc;
}

int gprt_job_stream(gprt_job* j, void** stream) {
  if (!j || !stream) return GPRT_E_INVALID;
  *stream = j->stream;
  return GPRT_OK;
}

}  // extern "C"

// ============================================================================
// Allocation-free rendering (gprt_render_noalloc).
//
// For callers that cannot allocate device memory while rendering: a plugin
// inside a host application whose own allocator owns the GPU's memory, and
// render loops whose device-memory budget is fixed at start-up.  The
// wavefront path state of one call lives in the file-scope device array
// below, sized for GPRT_NOALLOC_MAX_PATHS pixel samples; every GPU that loads
// the library holds it until exit.  In host code the name
// `g_noalloc_scratch` is a host-side stand-in, not a device address: the
// address is looked up with cudaGetSymbolAddress (with the context's device
// current) on the first call through a context, kept in the context, and
// passed to the kernels.  Calls share the array and keep the previous
// call's contents, so every counter and the error word are cleared at the
// start of a call; calls that overlap on the GPU race.
// ============================================================================
namespace {

constexpr size_t kNoAllocPaths = GPRT_NOALLOC_MAX_PATHS;
// the path state of kNoAllocPaths paths (two compacted queues of ray, weight,
// throughput, radiance and sampler ids; hits; origin radiance; shadow rays)
constexpr size_t kNoAllocBytes = path_region_bytes((uint32_t)kNoAllocPaths, false);

__device__ __align__(256) static unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array for this context's device (set-up on
// the first call through the context; the caller holds ctx->mu).
int noalloc_scratch(gprt_ctx* ctx, unsigned char** out) {
  if (!ctx->noalloc_scratch) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    ctx->noalloc_scratch = static_cast<unsigned char*>(p);
  }
  *out = ctx->noalloc_scratch;
  return GPRT_OK;
}

// Mean of the `layers` samples of every pixel: the sums of PixelStats.AddSample
// in sample order, then GetColor (pkg/renderer/stats.go:41-55).  When a
// device bound was exceeded the image is NaN and the error bits go to
// `status` (when given).
__global__ void k_noalloc_mean(DevPaths P, uint32_t npix, uint32_t layers, float* out, uint32_t* status) {
  const uint32_t err = *(volatile uint32_t*)(P.counters + 3);
  if (status && blockIdx.x == 0 && threadIdx.x == 0) *status = err;
  const float nan = __int_as_float(0x7fc00000);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
    if (err) {
      out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = nan;
      continue;
    }
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t l = 0; l < layers; l++) {
      float4 c = P.Lout[l * npix + i];
      acc.x += c.x;
      acc.y += c.y;
      acc.z += c.z;
    }
    float inv = 1.0f / (float)layers;
    out[3 * i] = acc.x * inv;
    out[3 * i + 1] = acc.y * inv;
    out[3 * i + 2] = acc.z * inv;
  }
}

// The film counts a fresh job starts from: all zero, read by raygen as the
// first sample index of every pixel.
__global__ void k_noalloc_zero(uint32_t* p, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
}

}  // namespace

extern "C" int gprt_render_noalloc(gprt_scene* s, uint32_t spp, uint64_t seed, float* rgb_out, uint32_t* status_out,
                                   void* stream) {
  if (!s || !rgb_out || spp == 0) return GPRT_E_INVALID;
  gprt_ctx* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  uint64_t npix = (uint64_t)s->host.sampling.width * s->host.sampling.height;
  if (npix * spp > kNoAllocPaths)
    return fail(ctx, GPRT_E_INVALID,
                "width * height * spp = " + std::to_string(npix * spp) + " exceeds the " +
                    std::to_string(kNoAllocPaths) +
                    " pixel samples of the allocation-free entry point; use gprt_job_* or a smaller request");
  unsigned char* base = nullptr;
  int rc = noalloc_scratch(ctx, &base);
  if (rc) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  DevPaths P{};
  carve_paths(base, (uint32_t)kNoAllocPaths, false, P);
  P.stats = nullptr;
  // queue counters and the error word start at zero
  CK(ctx, cudaMemsetAsync(P.counters, 0, 8 * sizeof(uint32_t), st));
  // a film view whose sample counts are zero: the ids array of the second
  // queue holds them until the first bounce (raygen reads them before any
  // path is moved there)
  DevFilm film{};
  film.width = (int)s->host.sampling.width;
  film.height = (int)s->host.sampling.height;
  film.count = reinterpret_cast<uint32_t*>(P.q[1].ids);
  k_noalloc_zero<<<launch_grid((uint32_t)npix, 256, 0), 256, 0, st>>>(film.count, (uint32_t)npix);
  ChunkDesc ch{};
  ch.pix0 = 0;
  ch.npix = (uint32_t)npix;
  ch.layers = spp;
  ch.pix_list = nullptr;
  ch.seed = seed;
  const DevScene& sc = s->dev;
  const int block = 128;
  int grid = launch_grid((uint32_t)(npix * spp), block, std::max(1, ctx->sm_count * (2048 / block)));
  launch_pt_raygen(sc, film, P, ch, block, st);
  int cur = 0;
  for (int b = 0; b < sc.max_depth; b++) {
    launch_pt_extend(sc, P, cur, b, block, grid, st);
    launch_pt_shade(sc, P, ch, cur, b, block, grid, st);
    launch_pt_shadow(sc, P, cur, block, grid, st);
    cur ^= 1;
  }
  k_noalloc_mean<<<launch_grid((uint32_t)npix, 256, 0), 256, 0, st>>>(P, (uint32_t)npix, spp, rgb_out, status_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "allocation-free render launch");
  return GPRT_OK;
}

// ============================================================================
// Autotuner (gprt_autotune): coordinate descent over the wavefront size, the
// traversal variants and the block size, timing real tuning passes.
// ============================================================================
namespace {

// Device time of `spp` samples per pixel with `d` (after one warm-up pass),
// or a negative value when the configuration cannot run (e.g. out of memory).
double time_config(gprt_scene* s, const gprt_job_desc& d, uint32_t spp) {
  gprt_job* j = nullptr;
  if (gprt_job_create(s, &d, &j) != GPRT_OK) return -1.0;
  double ms = -1.0;
  if (gprt_job_add_samples(j, spp) == GPRT_OK && gprt_job_sync(j) == GPRT_OK) {
    cudaEventRecord(j->ev0, j->stream);
    if (gprt_job_add_samples(j, spp) == GPRT_OK) {
      cudaEventRecord(j->ev1, j->stream);
      if (gprt_job_sync(j) == GPRT_OK) {
        float f = 0;
        cudaEventElapsedTime(&f, j->ev0, j->ev1);
        ms = f;
      }
    }
  }
  gprt_job_destroy(j);
  return ms;
}

}  // namespace

extern "C" int gprt_autotune(gprt_scene* s, const gprt_job_desc* base, uint32_t spp, gprt_tune_result* out) {
  if (!s || !base || !out || spp == 0) return GPRT_E_INVALID;
  gprt_ctx* ctx = s->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  std::memset(out, 0, sizeof(*out));
  gprt_job_desc d = *base;
  d.flags &= ~(GPRT_JOB_TIME_KERNELS | GPRT_JOB_COUNT_TRAVERSAL | kVariantBits);
  d.max_samples_per_pixel = std::max(d.max_samples_per_pixel, 2 * spp);
  uint64_t npix = (uint64_t)s->host.sampling.width * s->host.sampling.height;
  uint64_t work = npix * spp;
  if (d.block_size == 0) d.block_size = 128;
  if (d.chunk_paths == 0) d.chunk_paths = (uint32_t)std::min<uint64_t>(work, 1u << 24);
  double best = time_config(s, d, spp);
  if (best < 0) return fail(ctx, GPRT_E_DEVICE, "autotune: the default configuration failed");
  out->default_ms = best;
  out->candidates = 1;
  auto consider = [&](gprt_job_desc c) {
    double t = time_config(s, c, spp);
    out->candidates++;
    if (t >= 0 && t < best) {
      best = t;
      d = c;
    }
  };
  if (d.integrator == GPRT_INTEGRATOR_PATH_TRACING) {
    // wavefront size: whole pass, a quarter, a sixteenth (at least 64 Ki paths)
    uint32_t base_chunk = d.chunk_paths;
    for (uint32_t div : {4u, 16u}) {
      uint32_t c = base_chunk / div;
      if (c < (1u << 16)) continue;
      gprt_job_desc cand = d;
      cand.chunk_paths = c;
      consider(cand);
    }
    // traversal variants
    uint32_t fl0 = d.flags;
    for (uint32_t v : {GPRT_JOB_SIMPLE_EXTEND, GPRT_JOB_SIMPLE_SHADOW, GPRT_JOB_SIMPLE_EXTEND | GPRT_JOB_SIMPLE_SHADOW}) {
      gprt_job_desc cand = d;
      cand.flags = fl0 | v;
      consider(cand);
    }
    // shading kernel with fewer registers
    gprt_job_desc cand = d;
    cand.flags ^= GPRT_JOB_SHADE_OCCUPANCY;
    consider(cand);
  }
  // block size of the non-persistent kernels
  for (uint32_t b : {64u, 256u}) {
    gprt_job_desc cand = d;
    cand.block_size = b;
    consider(cand);
  }
  out->flags = d.flags & kVariantBits;
  out->block_size = d.block_size;
  out->chunk_paths = d.chunk_paths;
  out->best_ms = best;
  return GPRT_OK;
}

namespace gprt {

int clone_scene(gprt_scene* src, gprt_scene** out) {
  gprt_ctx* ctx = src->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  *out = nullptr;
  auto s = std::make_unique<gprt_scene>();
  s->ctx = ctx;
  s->serial = src->serial;
  s->host = src->host;
  s->dev = DevScene{};
  int rc = upload_geometry(ctx, s.get());
  if (rc) {
    free_all(s->buffers);
    return rc;
  }
  rc = upload_rest(ctx, s.get());
  if (rc) return rc;
  *out = s.release();
  return GPRT_OK;
}

size_t bdpt_job_bytes(const gprt_scene* s, const gprt_job_desc& d) {
  const HostScene& h = s->host;
  uint64_t npix = (uint64_t)h.sampling.width * h.sampling.height;
  uint64_t ns = d.chunk_paths ? d.chunk_paths : npix * std::max(1u, d.max_samples_per_pixel);
  ns = std::min<uint64_t>(ns, 1u << 20);
  int maxv = bdpt_maxv((int)h.sampling.max_depth);
  size_t film = (size_t)npix * (sizeof(float4) * 2 + 3 * sizeof(uint32_t)) + 256;
  size_t work = bdpt_bytes((uint32_t)ns, maxv) + (size_t)ns * sizeof(float4) +               // vertices, Lout
                (size_t)ns * (maxv + 1) * maxv * sizeof(uint32_t) + 64 * sizeof(uint32_t);  // strategy lists
  if (!h.tex_info.empty()) work += (size_t)ns * 2 * maxv * sizeof(float2);
  return film + work;
}


// One round of an adaptive pass: lists the pixels still active for pass
// target `target` and minimum `min_s` (k_active_pixels; waits for j's
// stream), queues one sample for each, and returns their number in *active
// (0: the pass is complete and nothing is queued).
int job_adaptive_round(gprt_job* j, uint32_t target, uint32_t min_s, float threshold, uint32_t* active) {
  gprt_ctx* ctx = j->scene->ctx;
  const uint32_t npix = (uint32_t)j->film.width * j->film.height;
  CK(ctx, cudaMemsetAsync(j->d_active, 0, sizeof(uint32_t), j->stream));
  launch_active_pixels(j->film, target, min_s, threshold, j->d_pix_list, j->d_active, j->stream);
  j->launches++;
  CK(ctx, cudaMemcpyAsync(j->h_words + 1, j->d_active, 4, cudaMemcpyDeviceToHost, j->stream));
  CK(ctx, cudaStreamSynchronize(j->stream));
  *active = j->h_words[1];
  if (*active == 0) return GPRT_OK;
  if (*active != npix) j->uniform_count = -1;
  int rc = add_samples(j, 1, *active, j->d_pix_list);
  if (rc) return rc;
  if (j->uniform_count >= 0) j->uniform_count++;
  return GPRT_OK;
}

}  // namespace gprt
