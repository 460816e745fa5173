// kernels_film.cu - per-pixel film kernels: splat application, image
// resolve and the adaptive-sampling pixel list.
#include "device.cuh"
#include "kernels.h"

namespace gprt {

// processSplats: PixelStats.AddSplat adds to ColorAccum only
// (pkg/renderer/progressive.go:371-391, stats.go:36-38)
__global__ void k_apply_splats(DevFilm film) {
  uint32_t n = (uint32_t)film.width * film.height;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 s = film.splat[i];
    if (s.x != 0.f || s.y != 0.f || s.z != 0.f) {
      float4 a = film.rgbl[i];
      film.rgbl[i] = make_float4(a.x + s.x, a.y + s.y, a.z + s.z, a.w);
      film.splat[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

void launch_apply_splats(const DevFilm& film, cudaStream_t st) {
  uint32_t n = (uint32_t)film.width * film.height;
  k_apply_splats<<<launch_grid(n, 256, 0), 256, 0, st>>>(film);
}

// PixelStats.GetColor (stats.go:50-55)
__device__ __forceinline__ float3 pixel_color(const DevFilm& film, uint32_t i) {
  uint32_t c = film.count[i];
  if (c == 0) return f3(0.f, 0.f, 0.f);
  float4 a = film.rgbl[i];
  float inv = 1.0f / (float)c;
  return f3(a.x * inv, a.y * inv, a.z * inv);
}

// vec3ToColor: gamma 2, clamp [0,1], uint8(255 * v) truncation
// (pkg/renderer/progressive.go:482-495)
__global__ void k_resolve_rgba8(DevFilm film, uchar4* out) {
  uint32_t n = (uint32_t)film.width * film.height;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float3 c = pixel_color(film, i);
    float r = fminf(1.f, fmaxf(0.f, sqrtf(c.x)));
    float g = fminf(1.f, fmaxf(0.f, sqrtf(c.y)));
    float b = fminf(1.f, fmaxf(0.f, sqrtf(c.z)));
    out[i] = make_uchar4((unsigned char)(255.f * r), (unsigned char)(255.f * g), (unsigned char)(255.f * b), 255);
  }
}

void launch_resolve_rgba8(const DevFilm& film, uint8_t* out, cudaStream_t st) {
  uint32_t n = (uint32_t)film.width * film.height;
  k_resolve_rgba8<<<launch_grid(n, 256, 0), 256, 0, st>>>(film, reinterpret_cast<uchar4*>(out));
}

// extractTileImage (progressive.go:225-255): the tile's pixels resolved on
// the device, pixels without samples left at zero (alpha included)
__global__ void k_resolve_tile(DevFilm film, uint32_t x0, uint32_t y0, uint32_t tw, uint32_t th, uchar4* out) {
  uint32_t n = tw * th;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    uint32_t tx = k % tw, ty = k / tw;
    uint32_t i = (y0 + ty) * (uint32_t)film.width + (x0 + tx);
    if (film.count[i] == 0) {
      out[k] = make_uchar4(0, 0, 0, 0);
      continue;
    }
    float3 c = pixel_color(film, i);
    float r = fminf(1.f, fmaxf(0.f, sqrtf(c.x)));
    float g = fminf(1.f, fmaxf(0.f, sqrtf(c.y)));
    float b = fminf(1.f, fmaxf(0.f, sqrtf(c.z)));
    out[k] = make_uchar4((unsigned char)(255.f * r), (unsigned char)(255.f * g), (unsigned char)(255.f * b), 255);
  }
}

void launch_resolve_tile(const DevFilm& film, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, uint8_t* out,
                         cudaStream_t st) {
  uint32_t tw = x1 - x0, th = y1 - y0;
  k_resolve_tile<<<launch_grid(tw * th, 256, 0), 256, 0, st>>>(film, x0, y0, tw, th, reinterpret_cast<uchar4*>(out));
}

__global__ void k_image_mean(DevFilm film, float* out) {
  uint32_t n = (uint32_t)film.width * film.height;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float3 c = pixel_color(film, i);
    out[3 * i] = c.x;
    out[3 * i + 1] = c.y;
    out[3 * i + 2] = c.z;
  }
}

void launch_image_mean(const DevFilm& film, float* out, cudaStream_t st) {
  uint32_t n = (uint32_t)film.width * film.height;
  k_image_mean<<<launch_grid(n, 256, 0), 256, 0, st>>>(film, out);
}

// Pixels that still sample in this pass: SampleCount < target and not
// shouldStopSampling (pkg/renderer/tile_renderer.go:55, :77-101).  The list
// is compacted in pixel order within each warp.
__global__ void k_active_pixels(DevFilm film, uint32_t target, uint32_t min_samples, float threshold,
                                uint32_t* list, uint32_t* count) {
  uint32_t n = (uint32_t)film.width * film.height;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    uint32_t i = base + threadIdx.x;
    bool active = false;
    if (i < n) {
      uint32_t c = film.count[i];
      if (c < target) {
        active = true;
        if (c >= min_samples) {
          float4 a = film.rgbl[i];
          float mean = a.w / (float)c, meanSq = film.lum2[i] / (float)c;
          float var = fmaxf(0.f, meanSq - mean * mean);
          bool stop = mean <= 1e-8f ? var < 1e-6f : sqrtf(var) / mean < threshold;
          active = !stop;
        }
      }
    }
    unsigned mask = __ballot_sync(0xffffffffu, active);
    int lane = threadIdx.x & 31;
    uint32_t off = 0;
    if (lane == 0 && mask) off = atomicAdd(count, (uint32_t)__popc(mask));
    off = __shfl_sync(0xffffffffu, off, 0);
    if (active) list[off + __popc(mask & ((1u << lane) - 1u))] = i;
  }
}

void launch_active_pixels(const DevFilm& film, uint32_t target, uint32_t min_samples, float threshold,
                          uint32_t* list, uint32_t* count, cudaStream_t st) {
  uint32_t n = (uint32_t)film.width * film.height;
  k_active_pixels<<<launch_grid(n, 256, 0), 256, 0, st>>>(film, target, min_samples, threshold, list, count);
}

}  // namespace gprt
