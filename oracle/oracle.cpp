// oracle.cpp - scene construction from the C scene description, the
// progressive renderer (pkg/renderer) restated on host threads, and the C
// entry points the tests and the CPU baseline call through ctypes.
// TEST INFRASTRUCTURE ONLY (see oracle.hpp).
#include "oracle.hpp"

#include <chrono>
#include <cstring>
#include <mutex>
#include <thread>

#include "../include/gprt.h"

namespace ref {

// Builds a reference Scene from the flat description; returns nullptr and an
// error message on unsupported content.  Shape constructors follow
// pkg/geometry (NewSphere, NewQuad, NewBox, NewTriangleMesh, NewTriangle) and
// lights follow pkg/scene/scene.go:102-141.
Scene* buildScene(const gprt_scene_desc* d, std::string& err) {
  auto s = std::make_unique<Scene>();
  auto v3 = [](const double* p) { return Vec3(p[0], p[1], p[2]); };
  // textures (image_texture.go:17-23)
  for (uint32_t i = 0; i < d->n_textures; i++) {
    const gprt_texture_desc& t = d->textures[i];
    if (t.width == 0 || t.height == 0 || !t.pixels) {
      err = "texture needs a size and pixels";
      return nullptr;
    }
    auto tex = std::make_unique<ImageTexture>();
    tex->width = (int)t.width;
    tex->height = (int)t.height;
    tex->pixels.resize((size_t)t.width * t.height);
    for (size_t k = 0; k < tex->pixels.size(); k++) tex->pixels[k] = v3(t.pixels + 3 * k);
    s->textures.push_back(std::move(tex));
  }
  auto texture = [&](uint32_t k) -> const ImageTexture* { return k == 0 ? nullptr : s->textures[k - 1].get(); };
  // materials (two passes so Layered can reference later entries)
  s->materials.resize(d->n_materials);
  for (uint32_t i = 0; i < d->n_materials; i++) {
    const gprt_material_desc& m = d->materials[i];
    if ((m.kind == GPRT_MAT_LAMBERTIAN || m.kind == GPRT_MAT_METAL) && m.texture > d->n_textures) {
      err = "material texture index out of range";
      return nullptr;
    }
    switch (m.kind) {
      case GPRT_MAT_LAMBERTIAN: s->materials[i] = std::make_unique<Lambertian>(v3(m.albedo), texture(m.texture)); break;
      case GPRT_MAT_METAL: s->materials[i] = std::make_unique<Metal>(v3(m.albedo), m.fuzz, texture(m.texture)); break;
      case GPRT_MAT_DIELECTRIC: s->materials[i] = std::make_unique<Dielectric>(m.ior); break;
      case GPRT_MAT_EMISSIVE: s->materials[i] = std::make_unique<Emissive>(v3(m.emission)); break;
      case GPRT_MAT_SPOT_EMISSIVE:
        s->materials[i] = std::make_unique<SpotEmissive>(v3(m.emission), v3(m.albedo).normalize());
        break;
      case GPRT_MAT_LAYERED: break;
      case GPRT_MAT_MIX: break;
      default: err = "unknown material kind"; return nullptr;
    }
  }
  for (uint32_t i = 0; i < d->n_materials; i++) {
    const gprt_material_desc& m = d->materials[i];
    if (m.kind == GPRT_MAT_MIX) {
      auto basic = [&](uint32_t k) {
        return k < d->n_materials && d->materials[k].kind != GPRT_MAT_LAYERED && d->materials[k].kind != GPRT_MAT_MIX;
      };
      if (!basic(m.outer) || !basic(m.inner)) {
        err = "mix material must reference two non-layered, non-mix materials";
        return nullptr;
      }
      s->materials[i] = std::make_unique<Mix>(s->materials[m.outer].get(), s->materials[m.inner].get(), m.fuzz);
      continue;
    }
    if (m.kind != GPRT_MAT_LAYERED) continue;
    if (m.outer >= d->n_materials || m.inner >= d->n_materials || !s->materials[m.outer] ||
        !s->materials[m.inner]) {
      err = "layered material references an invalid material";
      return nullptr;
    }
    s->materials[i] = std::make_unique<Layered>(s->materials[m.outer].get(), s->materials[m.inner].get());
  }
  auto mat = [&](uint32_t i) -> const Material* { return i < s->materials.size() ? s->materials[i].get() : nullptr; };
  for (uint32_t i = 0; i < d->n_shapes; i++) {
    const gprt_shape_desc& sh = d->shapes[i];
    const double* p = sh.p;
    std::unique_ptr<Shape> shape;
    switch (sh.kind) {
      case GPRT_SHAPE_SPHERE: shape = std::make_unique<Sphere>(v3(p), p[3], mat(sh.material)); break;
      case GPRT_SHAPE_QUAD: shape = std::make_unique<Quad>(v3(p), v3(p + 3), v3(p + 6), mat(sh.material)); break;
      case GPRT_SHAPE_TRIANGLE: shape = std::make_unique<Triangle>(v3(p), v3(p + 3), v3(p + 6), mat(sh.material)); break;
      case GPRT_SHAPE_DISC: shape = std::make_unique<Disc>(v3(p), v3(p + 3), p[6], mat(sh.material)); break;
      case GPRT_SHAPE_CYLINDER:
        shape = std::make_unique<Cylinder>(v3(p), v3(p + 3), p[6], p[7] != 0, mat(sh.material));
        break;
      case GPRT_SHAPE_CONE:
        // NewCone's checks (cone.go:28-50)
        if (!(p[6] > 0) || p[7] < 0 || p[6] <= p[7] || !(v3(p + 3).sub(v3(p)).length() > 0)) {
          err = "invalid cone";
          return nullptr;
        }
        shape = std::make_unique<Cone>(v3(p), p[6], v3(p + 3), p[7], p[8] != 0, mat(sh.material));
        break;
      case GPRT_SHAPE_BOX: {
        auto b = std::make_unique<Box>(v3(p), v3(p + 3), v3(p + 6), mat(sh.material));
        b->setId((int)i);
        shape = std::move(b);
        break;
      }
      case GPRT_SHAPE_MESH: {
        if (sh.mesh >= d->n_meshes) {
          err = "mesh index out of range";
          return nullptr;
        }
        const gprt_mesh_desc& m = d->meshes[sh.mesh];
        std::vector<Vec3> verts(m.n_vertices);
        for (uint32_t k = 0; k < m.n_vertices; k++) verts[k] = v3(m.vertices + 3 * k);
        std::vector<uint32_t> idx(m.indices, m.indices + 3 * (size_t)m.n_triangles);
        std::vector<const Material*> mats(m.n_triangles);
        for (uint32_t k = 0; k < m.n_triangles; k++)
          mats[k] = mat(m.tri_materials ? m.tri_materials[k] : sh.material);
        auto tm = std::make_unique<TriangleMesh>(verts, idx, mats, m.tri_normals, m.vertex_uvs);
        tm->setId((int)i);
        shape = std::move(tm);
        break;
      }
      default: err = "unknown shape kind"; return nullptr;
    }
    shape->id = (int)i;
    s->shapes.push_back(shape.get());
    s->ownedShapes.push_back(std::move(shape));
  }
  std::vector<double> weights;
  for (uint32_t i = 0; i < d->n_lights; i++) {
    const gprt_light_desc& l = d->lights[i];
    std::unique_ptr<Light> light;
    switch (l.kind) {
      case GPRT_LIGHT_QUAD: {
        if (l.shape >= d->n_shapes || d->shapes[l.shape].kind != GPRT_SHAPE_QUAD) {
          err = "quad light must reference a quad shape";
          return nullptr;
        }
        light = std::make_unique<QuadLight>(static_cast<const Quad*>(s->shapes[l.shape]));
        break;
      }
      case GPRT_LIGHT_SPHERE: {
        if (l.shape == GPRT_NO_SHAPE) {  // its sphere is not a scene shape (not in the BVH)
          auto sph = std::make_unique<Sphere>(v3(l.from), l.radius, nullptr);
          auto em = std::make_unique<Emissive>(v3(l.color_a));
          sph->material = em.get();
          light = std::make_unique<SphereLight>(sph.get());
          s->ownedShapes.push_back(std::move(sph));
          s->materials.push_back(std::move(em));
          break;
        }
        if (l.shape >= d->n_shapes || d->shapes[l.shape].kind != GPRT_SHAPE_SPHERE) {
          err = "sphere light must reference a sphere shape";
          return nullptr;
        }
        light = std::make_unique<SphereLight>(static_cast<const Sphere*>(s->shapes[l.shape]));
        break;
      }
      case GPRT_LIGHT_DISC:
      case GPRT_LIGHT_DISC_SPOT: {
        if (l.shape >= d->n_shapes || d->shapes[l.shape].kind != GPRT_SHAPE_DISC) {
          err = "disc lights must reference a disc shape";
          return nullptr;
        }
        const Disc* disc = static_cast<const Disc*>(s->shapes[l.shape]);
        if (l.kind == GPRT_LIGHT_DISC)
          light = std::make_unique<DiscLight>(disc);
        else
          light = std::make_unique<DiscSpotLight>(disc, v3(l.from), v3(l.to), v3(l.color_a), l.cone_deg, l.cone_delta_deg);
        break;
      }
      case GPRT_LIGHT_POINT_SPOT:
        light = std::make_unique<PointSpotLight>(v3(l.from), v3(l.to), v3(l.color_a), l.cone_deg, l.cone_delta_deg);
        break;
      case GPRT_LIGHT_UNIFORM_INFINITE: light = std::make_unique<UniformInfiniteLight>(v3(l.color_a)); break;
      case GPRT_LIGHT_GRADIENT_INFINITE:
        light = std::make_unique<GradientInfiniteLight>(v3(l.color_a), v3(l.color_b));
        break;
      default: err = "unknown light kind"; return nullptr;
    }
    s->lights.push_back(light.get());
    s->ownedLights.push_back(std::move(light));
    weights.push_back(l.weight);
  }
  if (d->weighted_sampler) s->lightSampler = std::make_unique<LightSampler>(LightSampler::weighted(s->lights, weights));
  CameraConfig cc;
  cc.center = v3(d->camera.center);
  cc.lookAt = v3(d->camera.look_at);
  cc.up = v3(d->camera.up);
  cc.width = (int)d->camera.width;
  cc.aspectRatio = d->camera.aspect_ratio;
  cc.vfov = d->camera.vfov_deg;
  cc.aperture = d->camera.aperture;
  cc.focusDistance = d->camera.focus_distance;
  s->camera = std::make_unique<Camera>(cc);
  s->sampling.width = (int)d->sampling.width;
  s->sampling.height = (int)d->sampling.height;
  s->sampling.samplesPerPixel = (int)d->sampling.samples_per_pixel;
  s->sampling.maxDepth = (int)d->sampling.max_depth;
  s->sampling.rrMinBounces = (int)d->sampling.rr_min_bounces;
  s->sampling.adaptiveMinSamples = d->sampling.adaptive_min_samples;
  s->sampling.adaptiveThreshold = d->sampling.adaptive_threshold;
  s->preprocess();
  return s.release();
}

// PixelStats (pkg/renderer/stats.go:20-55)
struct PixelStats {
  Vec3 color;
  double lum = 0, lum2 = 0;
  int count = 0;
  void addSample(const Vec3& c) {
    color = color.add(c);
    double l = c.luminance();
    lum += l;
    lum2 += l * l;
    count++;
  }
  void addSplat(const Vec3& c) { color = color.add(c); }
  Vec3 getColor() const { return count == 0 ? Vec3() : color.mul(1.0 / (double)count); }
};

struct RenderStatsR {
  long long totalPixels = 0, totalSamples = 0;
  double averageSamples = 0;
  int maxSamples = 0, minSamples = 0, maxSamplesUsed = 0;
};

// The progressive renderer (pkg/renderer/progressive.go, tile_renderer.go)
struct Renderer {
  const Scene* scene;
  int integratorKind;  // 0 PT, 1 BDPT
  int tileSize, initialSamples, maxSamples, maxPasses, threads;
  uint64_t seed;
  int width, height;
  bool counterStream = false;  // draw from the GPU's per-sample counter stream
  std::vector<PixelStats> stats;
  struct Tile {
    int id, x0, y0, x1, y1;
    std::unique_ptr<PcgSampler> sampler;
  };
  std::vector<Tile> tiles;
  RenderStatsR last;

  Renderer(const Scene* s, int integ, int tile, int init, int maxSpp, int passes, uint64_t sd, int th)
      : scene(s), integratorKind(integ), tileSize(tile), initialSamples(init), maxSamples(maxSpp),
        maxPasses(passes), threads(th), seed(sd) {
    width = scene->sampling.width;
    height = scene->sampling.height;
    stats.resize((size_t)width * height);
    // NewTileGrid (progressive.go:455-479); per-tile stream seeded from the tile id
    int tx = (width + tileSize - 1) / tileSize, ty = (height + tileSize - 1) / tileSize;
    int id = 0;
    for (int y = 0; y < ty; y++)
      for (int x = 0; x < tx; x++) {
        Tile t;
        t.id = id;
        t.x0 = x * tileSize;
        t.y0 = y * tileSize;
        t.x1 = std::min(t.x0 + tileSize, width);
        t.y1 = std::min(t.y0 + tileSize, height);
        t.sampler = std::make_unique<PcgSampler>(seed, (uint64_t)(id + 42));
        tiles.push_back(std::move(t));
        id++;
      }
  }
  // getSamplesForPass (progressive.go:98-123)
  int samplesForPass(int pass) const {
    if (maxPasses == 1) return maxSamples;
    if (pass == 1) return initialSamples;
    int rem = maxSamples - initialSamples;
    int per = rem / (maxPasses - 1);
    int target = initialSamples + (pass - 1) * per;
    if (pass == maxPasses) target = maxSamples;
    return target;
  }
  // shouldStopSampling (tile_renderer.go:77-101)
  bool shouldStop(const PixelStats& ps, int maxS) const {
    int minS = std::max(1, (int)((double)maxS * scene->sampling.adaptiveMinSamples));
    if (ps.count < minS) return false;
    double mean = ps.lum / ps.count, meanSq = ps.lum2 / ps.count;
    double var = std::max(0.0, meanSq - mean * mean);
    if (mean <= 1e-8) return var < 1e-6;
    return std::sqrt(var) / mean < scene->sampling.adaptiveThreshold;
  }
  // RenderTileBounds + adaptiveSamplePixelWithSplats (tile_renderer.go:28-74)
  void renderTile(Tile& t, int target, std::vector<std::pair<int, Vec3>>& splats) {
    PathTracingIntegrator pt(scene->sampling);
    BDPTIntegrator bd(scene->sampling);
    std::vector<SplatRay> sr;
    for (int j = t.y0; j < t.y1; j++)
      for (int i = t.x0; i < t.x1; i++) {
        PixelStats& ps = stats[(size_t)j * width + i];
        while (ps.count < target && !shouldStop(ps, target)) {
          CounterSampler cs(seed, (uint32_t)(j * width + i), (uint32_t)ps.count);
          Sampler& s = counterStream ? static_cast<Sampler&>(cs) : static_cast<Sampler&>(*t.sampler);
          Vec2 a = s.get2D();
          Vec2 b = s.get2D();
          Ray ray = scene->camera->getRay(i, j, a, b);
          Vec3 c;
          if (integratorKind == 0) {
            c = pt.rayColor(ray, *scene, s);
          } else {
            sr.clear();
            c = bd.rayColor(ray, *scene, s, sr);
            for (auto& x : sr) {
              int px, py;
              if (scene->camera->mapRayToPixel(x.ray, px, py)) splats.push_back({py * width + px, x.color});
            }
          }
          ps.addSample(c);
        }
      }
  }
  // RenderPass (progressive.go:126-223) with processSplats (:371-391) and
  // assembleCurrentImage statistics (:395-431)
  RenderStatsR renderPass(int pass, int onlyTiles = -1) {
    int nt = onlyTiles >= 0 ? std::min(onlyTiles, (int)tiles.size()) : (int)tiles.size();
    std::vector<int> ids(nt);
    for (int k = 0; k < nt; k++) ids[k] = k;
    return renderTiles(pass, ids);
  }
  // The same pass over the listed tiles only (fixed windows of a frame:
  // path tracing has no cross-tile terms, so a window's pixels equal the
  // whole frame's; BDPT splats from the other tiles are left out).
  RenderStatsR renderTiles(int pass, const std::vector<int>& ids) {
    int target = samplesForPass(pass);
    int nt = (int)ids.size();
    for (int k : ids)
      if (k < 0 || k >= (int)tiles.size()) throw std::runtime_error("tile id out of range");
    std::vector<std::vector<std::pair<int, Vec3>>> tileSplats(nt);
    std::atomic<int> next{0};
    auto worker = [&]() {
      for (;;) {
        int k = next.fetch_add(1);
        if (k >= nt) break;
        renderTile(tiles[ids[k]], target, tileSplats[k]);
      }
    };
    int th = std::max(1, threads);
    std::vector<std::thread> pool;
    for (int i = 0; i < th; i++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    for (auto& v : tileSplats)
      for (auto& sp : v) stats[sp.first].addSplat(sp.second);
    RenderStatsR r;
    r.totalPixels = (long long)width * height;
    r.maxSamples = target;
    r.minSamples = maxSamples;
    for (auto& ps : stats) {
      r.totalSamples += ps.count;
      r.minSamples = std::min(r.minSamples, ps.count);
      r.maxSamplesUsed = std::max(r.maxSamplesUsed, ps.count);
    }
    r.averageSamples = (double)r.totalSamples / (double)r.totalPixels;
    last = r;
    return r;
  }
};

}  // namespace ref

using namespace ref;

namespace {
std::mutex g_err_mu;
std::string g_err;
void setErr(const std::string& e) {
  std::lock_guard<std::mutex> l(g_err_mu);
  g_err = e;
}
}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

void* oracle_scene_create(const gprt_scene_desc* d) {
  try {
    std::string err;
    Scene* s = buildScene(d, err);
    if (!s) setErr(err);
    return s;
  } catch (const std::exception& e) {
    setErr(e.what());
    return nullptr;
  }
}

void oracle_scene_destroy(void* s) { delete static_cast<Scene*>(s); }

// World center/radius (bvh.go:39-48) and image size
int oracle_scene_info(void* sp, double* center, double* radius, int* width, int* height) {
  Scene* s = static_cast<Scene*>(sp);
  center[0] = s->bvh->center.x;
  center[1] = s->bvh->center.y;
  center[2] = s->bvh->center.z;
  *radius = s->bvh->radius;
  *width = s->camera->imageWidth;
  *height = s->camera->imageHeight;
  return 0;
}

// BVH.Hit over a ray batch (float rays widened to float64).  Outputs t,
// shape index, sub index (-1 on miss), uv and the front-face shading normal.
int oracle_intersect(void* sp, const gprt_ray* rays, uint32_t n, double* t, int32_t* shape,
                     int32_t* sub, double* uv, double* normal, int threads) {
  Scene* s = static_cast<Scene*>(sp);
  std::atomic<uint32_t> next{0};
  auto work = [&]() {
    for (;;) {
      uint32_t b = next.fetch_add(4096);
      if (b >= n) break;
      uint32_t e = std::min(n, b + 4096);
      for (uint32_t i = b; i < e; i++) {
        const gprt_ray& r = rays[i];
        Ray ray(Vec3(r.ox, r.oy, r.oz), Vec3(r.dx, r.dy, r.dz));
        SurfaceInteraction h;
        double tmax = std::isinf(r.tmax) ? kInf : (double)r.tmax;
        if (s->bvh->hit(ray, r.tmin, tmax, h)) {
          t[i] = h.t;
          shape[i] = h.shape;
          sub[i] = h.sub;
          if (uv) {
            uv[2 * i] = h.uv.x;
            uv[2 * i + 1] = h.uv.y;
          }
          if (normal) {
            normal[3 * i] = h.normal.x;
            normal[3 * i + 1] = h.normal.y;
            normal[3 * i + 2] = h.normal.z;
          }
        } else {
          t[i] = -1;
          shape[i] = -1;
          sub[i] = -1;
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < std::max(1, threads); i++) pool.emplace_back(work);
  for (auto& x : pool) x.join();
  return 0;
}

// counter_stream != 0: every pixel sample draws from CounterSampler(seed,
// pixel, sample index), the GPU library's stream; otherwise a PCG32 stream
// per 64x64 tile.
void* oracle_renderer_create(void* sp, int integrator, int tile, int initial, int maxSpp, int passes,
                             uint64_t seed, int threads, int counter_stream) {
  Renderer* r = new Renderer(static_cast<Scene*>(sp), integrator, tile > 0 ? tile : 64,
                             initial > 0 ? initial : 1, maxSpp, passes > 0 ? passes : 1, seed, threads);
  r->counterStream = counter_stream != 0;
  return r;
}
void oracle_renderer_destroy(void* r) { delete static_cast<Renderer*>(r); }

// RenderPass; only_tiles >= 0 renders the first only_tiles tiles (bounded
// CPU-baseline samples).  stats_out: total_pixels, total_samples, min, max_used.
int oracle_render_pass(void* rp, int pass, int only_tiles, double* seconds, long long* stats_out) {
  Renderer* r = static_cast<Renderer*>(rp);
  try {
    auto t0 = std::chrono::steady_clock::now();
    RenderStatsR st = r->renderPass(pass, only_tiles);
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    if (stats_out) {
      stats_out[0] = st.totalPixels;
      stats_out[1] = st.totalSamples;
      stats_out[2] = st.minSamples;
      stats_out[3] = st.maxSamplesUsed;
    }
    return 0;
  } catch (const std::exception& e) {
    setErr(e.what());
    return -1;
  }
}

// RenderPass over the `n` listed tile ids only (row-major 64x64 tile grid of
// NewTileGrid, progressive.go:455-479).
int oracle_render_tiles(void* rp, int pass, const int32_t* ids, int n, double* seconds, long long* stats_out) {
  Renderer* r = static_cast<Renderer*>(rp);
  try {
    auto t0 = std::chrono::steady_clock::now();
    RenderStatsR st = r->renderTiles(pass, std::vector<int>(ids, ids + n));
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    if (stats_out) {
      stats_out[0] = st.totalPixels;
      stats_out[1] = st.totalSamples;
      stats_out[2] = st.minSamples;
      stats_out[3] = st.maxSamplesUsed;
    }
    return 0;
  } catch (const std::exception& e) {
    setErr(e.what());
    return -1;
  }
}

// Film read-back: mean color (GetColor), luminance sums and counts.
int oracle_renderer_read(void* rp, double* rgb_mean, double* rgb_sum, double* lum, double* lum2,
                         int32_t* count) {
  Renderer* r = static_cast<Renderer*>(rp);
  for (size_t i = 0; i < r->stats.size(); i++) {
    const PixelStats& ps = r->stats[i];
    Vec3 c = ps.getColor();
    if (rgb_mean) {
      rgb_mean[3 * i] = c.x;
      rgb_mean[3 * i + 1] = c.y;
      rgb_mean[3 * i + 2] = c.z;
    }
    if (rgb_sum) {
      rgb_sum[3 * i] = ps.color.x;
      rgb_sum[3 * i + 1] = ps.color.y;
      rgb_sum[3 * i + 2] = ps.color.z;
    }
    if (lum) lum[i] = ps.lum;
    if (lum2) lum2[i] = ps.lum2;
    if (count) count[i] = ps.count;
  }
  return 0;
}

// assembleCurrentImage / vec3ToColor (progressive.go:395-495)
int oracle_renderer_rgba8(void* rp, uint8_t* out) {
  Renderer* r = static_cast<Renderer*>(rp);
  for (size_t i = 0; i < r->stats.size(); i++) {
    Vec3 c = r->stats[i].getColor().gammaCorrect(2.0).clamp(0.0, 1.0);
    out[4 * i] = (uint8_t)(255 * c.x);
    out[4 * i + 1] = (uint8_t)(255 * c.y);
    out[4 * i + 2] = (uint8_t)(255 * c.z);
    out[4 * i + 3] = 255;
  }
  return 0;
}

int oracle_samples_for_pass(void* rp, int pass) { return static_cast<Renderer*>(rp)->samplesForPass(pass); }

// Camera.GetRay for a batch of (i, j, lens sample, jitter) inputs.
int oracle_camera_rays(void* sp, uint32_t n, const int32_t* ij, const double* samples, double* out) {
  Scene* s = static_cast<Scene*>(sp);
  for (uint32_t k = 0; k < n; k++) {
    Ray r = s->camera->getRay(ij[2 * k], ij[2 * k + 1], Vec2(samples[4 * k], samples[4 * k + 1]),
                              Vec2(samples[4 * k + 2], samples[4 * k + 3]));
    out[6 * k] = r.origin.x;
    out[6 * k + 1] = r.origin.y;
    out[6 * k + 2] = r.origin.z;
    out[6 * k + 3] = r.direction.x;
    out[6 * k + 4] = r.direction.y;
    out[6 * k + 5] = r.direction.z;
  }
  return 0;
}

// One path-traced sample per input ray with an injected sample list per ray
// (TestSampler semantics), for deterministic integrator comparisons.
int oracle_pt_ray_color(void* sp, const double* ray, const double* v1, int n1, const double* v2,
                        int n2, const double* v3, int n3, double* out) {
  Scene* s = static_cast<Scene*>(sp);
  std::vector<double> a(v1, v1 + n1);
  std::vector<Vec2> b;
  for (int i = 0; i < n2; i++) b.emplace_back(v2[2 * i], v2[2 * i + 1]);
  std::vector<Vec3> c;
  for (int i = 0; i < n3; i++) c.emplace_back(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]);
  ListSampler ls(a, b, c);
  PathTracingIntegrator pt(s->sampling);
  try {
    Vec3 r = pt.rayColor(Ray(Vec3(ray[0], ray[1], ray[2]), Vec3(ray[3], ray[4], ray[5])), *s, ls);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
  } catch (const std::exception& e) {
    setErr(e.what());
    return -1;
  }
  return 0;
}

}  // extern "C"
