// handles.h - the handle types behind the opaque pointers of include/gprt.h
// (context, scene, job, server) and the error / allocation helpers the
// translation units of the C ABI share.
#pragma once

#include <condition_variable>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/gprt.h"
#include "kernels.h"
#include "scene.h"

using namespace gprt;

// Ownership: a context owns its scenes and a scene owns its jobs, so
// destroying a parent releases whatever children the caller did not.
struct gprt_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  // pinned words for small read-backs (counts, error flags): a copy into
  // pageable memory blocks inside the runtime until the stream drains and
  // stalls other threads' CUDA calls meanwhile
  uint32_t* h_words = nullptr;
  std::recursive_mutex mu;
  std::string err;
  std::set<gprt_scene*> scenes;
  std::set<gprt_server*> servers;
  // device address of the allocation-free entry point's static array,
  // looked up on its first call through this context
  unsigned char* noalloc_scratch = nullptr;
};

struct gprt_scene {
  gprt_ctx* ctx = nullptr;
  HostScene host;
  DevScene dev{};
  std::vector<void*> buffers;
  size_t bytes = 0;
  int* d_err = nullptr;
  std::set<gprt_job*> jobs;
  uint64_t serial = 0;  // unique per scene created in this process
};

struct gprt_job {
  gprt_scene* scene = nullptr;
  uint32_t* h_words = nullptr;  // pinned: [0] error bits, [1] active pixels
  gprt_job_desc desc{};
  DevFilm film{};
  DevPaths paths{};
  std::vector<void*> buffers;
  cudaStream_t stream = nullptr;
  uint32_t* d_pix_list = nullptr;
  uint32_t* d_active = nullptr;
  uint64_t launches = 0;
  int64_t uniform_count = 0;  // every pixel holds this many samples (-1: differs)
  uint64_t sample_index_base = 0;
  gprt_render_stats last{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // instrumentation (GPRT_JOB_TIME_KERNELS / GPRT_JOB_COUNT_TRAVERSAL)
  struct Timed {
    int cls;  // 0 extend, 1 shade, 2 shadow, 3 other
    cudaEvent_t a, b;
  };
  std::vector<Timed> timed;
  size_t timed_used = 0;
  unsigned long long* d_stats = nullptr;
  gprt_job_counters acc{};
};

namespace gprt {


inline int fail(gprt_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

inline int cuda_fail(gprt_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, GPRT_E_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(ctx, call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

template <class T>
int dev_alloc(gprt_ctx* ctx, std::vector<void*>& bufs, T** out, size_t count, size_t* bytes = nullptr) {
  *out = nullptr;
  if (count == 0) return GPRT_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, GPRT_E_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  bufs.push_back(p);
  *out = static_cast<T*>(p);
  if (bytes) *bytes += count * sizeof(T);
  return GPRT_OK;
}

template <class T>
int upload(gprt_ctx* ctx, std::vector<void*>& bufs, const std::vector<T>& src, const T** out, size_t* bytes) {
  T* d = nullptr;
  int rc = dev_alloc(ctx, bufs, &d, src.size(), bytes);
  if (rc) return rc;
  if (!src.empty()) CK(ctx, cudaMemcpyAsync(d, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  *out = d;
  return GPRT_OK;
}

inline void free_all(std::vector<void*>& bufs) {
  for (void* p : bufs) cudaFree(p);
  bufs.clear();
}

// getSamplesForPass (pkg/renderer/progressive.go:98-123)
// Builds the BVH and the primitive arrays of `h` on the GPU from h.pending
// (bvh_build.cu); the device arrays are allocated into `bufs`.
int device_build_bvh(gprt_ctx* ctx, HostScene& h, DevScene& d, std::vector<void*>& bufs, size_t* bytes);

// Cancels the server's pending requests for a scene that is being destroyed
// (server.cu).  Called with the scene's context locked.
void server_forget_scene(gprt_server* sv, gprt_scene* s);
// A private copy of scene `src` (the same host description, its own device
// arrays), not listed among the context's scenes; gprt_scene_destroy
// releases it with the jobs on it.  The server renders BDPT requests on one.
int clone_scene(gprt_scene* src, gprt_scene** out);
// One round of an adaptive pass of job j (gprt_job_render_pass's loop body,
// capi.cu): one sample for every pixel still active for pass target
// `target` and minimum `min_s`; *active = their number (0: pass complete).
int job_adaptive_round(gprt_job* j, uint32_t target, uint32_t min_s, float threshold, uint32_t* active);
// Device bytes of a BDPT job on scene `s`: film, and the subpath vertices and
// strategy buffers of one chunk as gprt_job_create and its first pass allocate them.
size_t bdpt_job_bytes(const gprt_scene* s, const gprt_job_desc& d);

inline uint32_t samples_for_pass(const gprt_job_desc& d, uint32_t pass) {
  if (d.max_passes == 1) return d.max_samples_per_pixel;
  if (pass == 1) return d.initial_samples;
  uint32_t rem = d.max_samples_per_pixel - d.initial_samples;
  uint32_t per = rem / (d.max_passes - 1);
  uint32_t t = d.initial_samples + (pass - 1) * per;
  if (pass == d.max_passes) t = d.max_samples_per_pixel;
  return t;
}

}  // namespace gprt
