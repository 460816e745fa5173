/*
 * gprt.h - C ABI of the GB300-native rendering hot path of go-progressive-raytracer.
 *
 * The Go reference keeps its rendering path behind four seams (all paths are
 * relative to the reference project root):
 *   - scene.Scene + scene.SamplingConfig            pkg/scene/scene.go:11-30
 *   - integrator.Integrator (PT and BDPT)           pkg/integrator/integrator.go:15-19,
 *                                                   pkg/integrator/path_tracing.go:40,
 *                                                   pkg/integrator/bdpt.go:64
 *   - renderer.ProgressiveRaytracer                 pkg/renderer/progressive.go:62-223,286
 *   - geometry.BVH.Hit (raw ray batches)            pkg/geometry/bvh.go:183-239
 * This header is what a cgo binding of those seams calls.  Every entry point
 * below cites the reference function it replaces.
 *
 * Conventions (mirroring the reference's Go conventions):
 *   - Every function returns an int status: 0 = OK, negative = error
 *     (GPRT_E_*).  No exception or abort crosses this boundary.  The message of
 *     the last error of a context is returned by gprt_last_error().
 *   - Host pointers passed in are borrowed for the duration of the call only
 *     (cgo pointer rules: Go memory is never retained).  Scene descriptions are
 *     copied.
 *   - All device memory is owned by handles (context, scene, job).  A context
 *     serialises the calls made on it and on its scenes and jobs with an
 *     internal mutex, so handles may be used from several goroutines.
 *   - Arithmetic on the device is FP32; descriptions are float64 like the
 *     reference's core.Vec3 (pkg/core/vec3.go:9-11) and are rounded once.
 */
#ifndef GPRT_H
#define GPRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPRT_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define GPRT_OK 0
#define GPRT_E_INVALID (-1)      /* invalid argument or unsupported scene content */
#define GPRT_E_OOM (-2)          /* device allocation failed */
#define GPRT_E_DEVICE (-3)       /* CUDA error (launch, copy, sync) */
#define GPRT_E_BOUND (-4)        /* a device-side bound (stack, queue, wait) was exceeded */
#define GPRT_E_CANCELLED (-5)    /* job cancelled (context.Context cancellation analogue) */
#define GPRT_E_ADMISSION (-6)    /* serving: request refused by the HBM budget */
#define GPRT_E_NOT_FOUND (-7)    /* serving: unknown ticket */

/* ---- scene description ----------------------------------------------------
 * A flattened scene.Scene (pkg/scene/scene.go:11-19).  Shapes are listed in
 * scene.Shapes order; lights in scene.Lights order.  An area light names the
 * shape that holds its geometry (scene.AddQuadLight / AddSphereLight append
 * both, pkg/scene/scene.go:102-115).
 */

enum gprt_material_kind {
  GPRT_MAT_LAMBERTIAN = 0, /* pkg/material/lambertian.go (SolidColor albedo) */
  GPRT_MAT_METAL = 1,      /* pkg/material/metal.go (fuzz clamped to [0,1]) */
  GPRT_MAT_DIELECTRIC = 2, /* pkg/material/dielectric.go */
  GPRT_MAT_EMISSIVE = 3,   /* pkg/material/emissive.go */
  GPRT_MAT_LAYERED = 4,    /* pkg/material/layered.go (outer, inner) */
  GPRT_MAT_SPOT_EMISSIVE = 5, /* the disc spot light's directional emitter (pkg/lights/disc_spot_light.go:13-51):
                                 emission, albedo = spot direction (normalised by the library) */
  GPRT_MAT_MIX = 6             /* pkg/material/mix.go: outer = material 1, inner = material 2 (neither layered nor
                                  mix), fuzz = ratio (clamped to [0,1]; 0 = all material 1) */
};

/* material.ImageTexture (pkg/material/image_texture.go:8-52): a row-major
 * RGB image, pixels[3 * (y * width + x) + c] (the memory of []core.Vec3) */
typedef struct gprt_texture_desc {
  uint32_t width;
  uint32_t height;
  const double* pixels;
} gprt_texture_desc;

typedef struct gprt_material_desc {
  uint32_t kind;     /* gprt_material_kind */
  uint32_t outer;    /* LAYERED: material index of the outer layer; MIX: material 1 */
  uint32_t inner;    /* LAYERED: material index of the inner layer; MIX: material 2 */
  uint32_t texture;  /* LAMBERTIAN, METAL: 0 = the solid albedo; k = textures[k-1] (NewTexturedLambertian,
                        NewTexturedMetal), evaluated at the hit's UV */
  double albedo[3];  /* LAMBERTIAN, METAL */
  double fuzz;       /* METAL; MIX: the ratio */
  double ior;        /* DIELECTRIC */
  double emission[3];/* EMISSIVE, SPOT_EMISSIVE */
} gprt_material_desc;

enum gprt_shape_kind {
  GPRT_SHAPE_SPHERE = 0,   /* p[0..2] center, p[3] radius (negative = inward normal) */
  GPRT_SHAPE_QUAD = 1,     /* p[0..2] corner, p[3..5] u, p[6..8] v */
  GPRT_SHAPE_BOX = 2,      /* p[0..2] center, p[3..5] half extents, p[6..8] rotation (rad, X->Y->Z) */
  GPRT_SHAPE_MESH = 3,     /* mesh = index into gprt_scene_desc.meshes */
  GPRT_SHAPE_TRIANGLE = 4, /* p[0..2] v0, p[3..5] v1, p[6..8] v2 */
  GPRT_SHAPE_DISC = 5,     /* pkg/geometry/disc.go: p[0..2] centre, p[3..5] normal, p[6] radius */
  GPRT_SHAPE_CYLINDER = 6, /* pkg/geometry/cylinder.go: p[0..2] base, p[3..5] top, p[6] radius, p[7] capped */
  GPRT_SHAPE_CONE = 7      /* pkg/geometry/cone.go: p[0..2] base, p[3..5] top, p[6] base radius,
                              p[7] top radius (< base radius; 0 = pointed), p[8] capped */
};

typedef struct gprt_shape_desc {
  uint32_t kind;     /* gprt_shape_kind */
  uint32_t material; /* material index (ignored for MESH with per-triangle materials) */
  uint32_t mesh;     /* MESH only */
  uint32_t reserved;
  double p[9];
} gprt_shape_desc;

/* geometry.NewTriangleMesh(vertices, faces, material, &TriangleMeshOptions{...})
 * pkg/geometry/triangle_mesh.go:33-146.  Rotation / Center only transform
 * the vertices and are applied by the caller. */
typedef struct gprt_mesh_desc {
  const double* vertices;      /* 3 * n_vertices */
  const uint32_t* indices;     /* 3 * n_triangles */
  const uint32_t* tri_materials; /* n_triangles material indices, or NULL (Materials) */
  uint32_t n_vertices;
  uint32_t n_triangles;
  const double* tri_normals;   /* 3 * n_triangles custom normals (normalised here), or NULL (Normals) */
  const double* vertex_uvs;    /* 2 * n_vertices texture coordinates, or NULL (VertexUVs) */
} gprt_mesh_desc;

enum gprt_light_kind {
  GPRT_LIGHT_QUAD = 0,              /* pkg/lights/quad_light.go; shape = a QUAD shape */
  GPRT_LIGHT_SPHERE = 1,            /* pkg/lights/sphere_light.go; shape = a SPHERE shape, or GPRT_NO_SHAPE for a
                                       light whose sphere is not a scene shape (from = centre, radius, color_a =
                                       emission; the PBRT point light, pkg/scene/pbrt_scene.go:340-349) */
  GPRT_LIGHT_UNIFORM_INFINITE = 2,  /* pkg/lights/uniform_infinite_light.go; color_a = emission */
  GPRT_LIGHT_GRADIENT_INFINITE = 3, /* pkg/lights/gradient_infinite_light.go; color_a = top, color_b = bottom */
  GPRT_LIGHT_DISC = 4,              /* pkg/lights/disc_light.go; shape = a DISC shape with an emissive material */
  GPRT_LIGHT_DISC_SPOT = 5,         /* pkg/lights/disc_spot_light.go (scene.AddSpotLight); shape = the DISC at
                                       `from` facing `to` whose material is SPOT_EMISSIVE; color_a = emission,
                                       from, to, cone_deg, cone_delta_deg */
  GPRT_LIGHT_POINT_SPOT = 6         /* pkg/lights/point_spot_light.go (scene.AddPointSpotLight); no shape;
                                       color_a = emission, from, to, cone_deg, cone_delta_deg */
};

#define GPRT_NO_SHAPE 0xFFFFFFFFu

typedef struct gprt_light_desc {
  uint32_t kind;   /* gprt_light_kind */
  uint32_t shape;  /* QUAD / SPHERE / DISC / DISC_SPOT: index of the shape holding the geometry and material */
  double color_a[3];
  double color_b[3];
  double weight;   /* light-sampler weight; used when gprt_scene_desc.weighted_sampler != 0 */
  double from[3];  /* spot lights: position (disc centre) */
  double to[3];    /* spot lights: the point aimed at */
  double cone_deg;       /* spot lights: total cone angle, degrees */
  double cone_delta_deg; /* spot lights: falloff transition angle, degrees */
  double radius;         /* SPHERE with GPRT_NO_SHAPE: the sphere's radius */
} gprt_light_desc;

/* geometry.CameraConfig, pkg/geometry/camera.go:18-32 */
typedef struct gprt_camera_desc {
  double center[3];
  double look_at[3];
  double up[3];
  double aspect_ratio;
  double vfov_deg;
  double aperture;
  double focus_distance; /* <= 0: |center - look_at| */
  uint32_t width;
  uint32_t reserved;
} gprt_camera_desc;

/* scene.SamplingConfig, pkg/scene/scene.go:22-30 */
typedef struct gprt_sampling_desc {
  uint32_t width;
  uint32_t height;
  uint32_t samples_per_pixel;
  uint32_t max_depth;
  uint32_t rr_min_bounces;
  uint32_t reserved;
  double adaptive_min_samples; /* fraction of the pass target; 1.0 = fixed spp */
  double adaptive_threshold;
} gprt_sampling_desc;

typedef struct gprt_scene_desc {
  const gprt_material_desc* materials;
  const gprt_shape_desc* shapes;
  const gprt_mesh_desc* meshes;
  const gprt_light_desc* lights;
  uint32_t n_materials;
  uint32_t n_shapes;
  uint32_t n_meshes;
  uint32_t n_lights;
  uint32_t weighted_sampler; /* 0: lights.NewUniformLightSampler; 1: NewWeightedLightSampler(weights) */
  uint32_t build_flags;      /* GPRT_BUILD_* */
  gprt_camera_desc camera;
  gprt_sampling_desc sampling;
  const gprt_texture_desc* textures;
  uint32_t n_textures;
  uint32_t reserved;
} gprt_scene_desc;

/* ---- ray batches ----------------------------------------------------------
 * Layout of a ray batch for gprt_intersect: 32 bytes per ray, two 16-byte
 * vectors per ray.  tmin/tmax are the Hit(ray, tMin, tMax) interval of
 * geometry.BVH.Hit. */
/* BVH construction.  Default: binned-SAH BVH built on the host (best
 * traversal speed).  GPRT_BUILD_DEVICE builds it on the GPU instead: Morton
 * codes, radix sort, a linear BVH (Karras 2012) collapsed to the same
 * 4-wide node layout, in milliseconds for millions of triangles (for scenes
 * that arrive while a server is running); its tree traverses somewhat
 * slower.  Scenes of fewer than 8 primitives always build on the host. */
#define GPRT_BUILD_DEVICE 1u
/* Tests only: every ray of this scene gets a 1-entry traversal stack instead
 * of 64, so that rays overflow it and the scene's jobs fail with GPRT_E_BOUND
 * (the device-bound path: the kernels set the error bits and carry on, and
 * only the jobs whose rays overflowed fail). */
#define GPRT_BUILD_TEST_STACK_CAP 2u

typedef struct gprt_ray {
  float ox, oy, oz, tmin;
  float dx, dy, dz, tmax;
} gprt_ray;

/* Hit record: t, primitive id (GPRT_NO_HIT when missed), barycentric /
 * parametric (u, v) as in SurfaceInteraction.UV for triangles and quads.
 * A ray whose traversal stack overflowed (a device bound: the closest hit is
 * unknown) gets prim = GPRT_BOUND_HIT and t = -1. */
typedef struct gprt_hit {
  float t;
  uint32_t prim;
  float u, v;
} gprt_hit;

#define GPRT_NO_HIT 0xFFFFFFFFu
#define GPRT_BOUND_HIT 0xFFFFFFFEu
#define GPRT_CLOSEST 0u /* closest hit (BVH.Hit with the hit record used) */
#define GPRT_ANY 1u     /* any hit in (tmin, tmax): the shadow-ray use of BVH.Hit */

typedef struct gprt_scene_info {
  double world_center[3]; /* BVH.Center, pkg/geometry/bvh.go:39-48 */
  double world_radius;    /* BVH.Radius */
  uint64_t n_primitives;
  uint64_t n_triangles;
  uint64_t n_quads;
  uint64_t n_spheres;
  uint64_t n_nodes;       /* 4-wide BVH nodes */
  uint64_t device_bytes;  /* device memory held by the scene */
  uint32_t image_width;
  uint32_t image_height;
  double build_ms;        /* scene construction time (flatten + BVH + checks) */
  double flatten_ms;      /* of which: flattening the description into primitives */
  double bvh_ms;          /* of which: BVH build and primitive arrays (host SAH or device) */
  double check_ms;        /* of which: layout check of a device-built tree */
  uint64_t n_quadrics;    /* discs, cylinders, cones */
} gprt_scene_info;

/* ---- progressive jobs ---------------------------------------------------- */
enum gprt_integrator_kind {
  GPRT_INTEGRATOR_PATH_TRACING = 0, /* integrator.NewPathTracingIntegrator */
  GPRT_INTEGRATOR_BDPT = 1          /* integrator.NewBDPTIntegrator */
};

/* renderer.ProgressiveConfig (pkg/renderer/progressive.go:29-46) plus the
 * integrator choice and the counter-based sampler seed. */
typedef struct gprt_job_desc {
  uint32_t integrator;           /* gprt_integrator_kind */
  uint32_t tile_size;            /* 0 -> 64 */
  uint32_t initial_samples;      /* 0 -> 1 */
  uint32_t max_samples_per_pixel;/* 0 -> 50 */
  uint32_t max_passes;           /* 0 -> 7 */
  uint32_t chunk_paths;          /* wavefront size; 0 -> automatic */
  uint32_t block_size;           /* threads per block; 0 -> automatic */
  uint32_t flags;                /* GPRT_JOB_* instrumentation flags */
  uint64_t seed;
} gprt_job_desc;

#define GPRT_JOB_TIME_KERNELS 1u     /* CUDA-event timing of every kernel launch, per kernel class */
#define GPRT_JOB_COUNT_TRAVERSAL 2u  /* count BVH node / box / primitive tests (slower kernels) */
/* Kernel variants (normally chosen by gprt_autotune): the closest-hit and the
 * shadow traversal run either persistent (warps refill finished lanes with
 * new rays) or one ray per thread. */
#define GPRT_JOB_SIMPLE_EXTEND 4u
#define GPRT_JOB_SIMPLE_SHADOW 8u
/* Shading kernel compiled for 3 resident 192-thread blocks per SM (18 warps,
 * at most 96 registers) instead of 2 blocks of 256 threads (16 warps). */
#define GPRT_JOB_SHADE_OCCUPANCY 32u

/* Instrumentation of a job (GPRT_JOB_* flags), summed since the last reset.
 * "extend" is the closest-hit traversal of the live paths (one launch per
 * bounce), "shadow" the any-hit traversal of the shadow rays, "shade" the
 * material / light sampling kernel. */
typedef struct gprt_job_counters {
  uint64_t extend_launches, shade_launches, shadow_launches, other_launches;
  double extend_ms, shade_ms, shadow_ms, other_ms;
  uint64_t extend_rays, shadow_rays;
  uint64_t extend_nodes, extend_boxes, extend_prims;
  uint64_t shadow_nodes, shadow_boxes, shadow_prims;
} gprt_job_counters;

/* renderer.RenderStats, pkg/renderer/stats.go:10-17 */
typedef struct gprt_render_stats {
  uint64_t total_pixels;
  uint64_t total_samples;
  double average_samples;
  uint32_t max_samples;
  uint32_t min_samples;
  uint32_t max_samples_used;
  uint32_t pass_number;
  double pass_ms;       /* device time of the pass */
  uint64_t splats;      /* BDPT t=1 splats applied in the pass */
} gprt_render_stats;

typedef struct gprt_ctx gprt_ctx;
typedef struct gprt_scene gprt_scene;
typedef struct gprt_job gprt_job;
typedef struct gprt_server gprt_server;

/* ---- context ------------------------------------------------------------ */
int gprt_version(void);
/* Creates a context on CUDA device `device`. */
int gprt_ctx_create(int device, gprt_ctx** out);
int gprt_ctx_destroy(gprt_ctx* ctx);
/* Message of the last failed call on this context ("" when none). */
const char* gprt_last_error(const gprt_ctx* ctx);

/* ---- scene ---------------------------------------------------------------
 * Replaces scene.Scene.Preprocess (pkg/scene/scene.go:45-78): flattens the
 * shapes into device primitive arrays, builds the device BVH (the reference
 * builds geometry.NewBVH, pkg/geometry/bvh.go:26-109), computes the world
 * center/radius used by the infinite lights (bvh.go:39-48,
 * uniform_infinite_light.go:128-132) and the light sampler
 * (weighted_light_sampler.go:57-78).  Unsupported content -> GPRT_E_INVALID. */
int gprt_scene_create(gprt_ctx* ctx, const gprt_scene_desc* desc, gprt_scene** out);
int gprt_scene_destroy(gprt_scene* scene);
int gprt_scene_get_info(const gprt_scene* scene, gprt_scene_info* info);
/* Maps primitive ids to (index in scene.Shapes, sub-index: box face 0..5 or
 * mesh triangle index, 0 otherwise).  Arrays of n_primitives entries. */
int gprt_scene_primitive_map(const gprt_scene* scene, uint32_t* shape_index, uint32_t* sub_index);

/* Host-only check of a description: flattens it and builds the BVH on the
 * host, verifies the layout invariants (every primitive in exactly one leaf,
 * every box containing what it bounds) and fills `info` (n_nodes, counts,
 * world center/radius).  Needs no GPU.  Returns GPRT_E_INVALID with a message
 * in `err` (size err_len) on failure. */
int gprt_scene_validate(const gprt_scene_desc* desc, gprt_scene_info* info, char* err, size_t err_len);

/* ---- raw ray batches -----------------------------------------------------
 * Replaces geometry.BVH.Hit / hitNode (pkg/geometry/bvh.go:183-239) for a
 * batch.  `rays` and `hits` are DEVICE pointers; `stream` is a cudaStream_t
 * (NULL = the context stream).  Asynchronous. */
int gprt_intersect(gprt_scene* scene, const gprt_ray* rays, uint32_t n, uint32_t flags,
                   gprt_hit* hits, void* stream);
/* Same with HOST pointers; copies in, traces and copies out, synchronously.
 * Returns GPRT_E_BOUND when a ray's traversal stack overflowed (its hit
 * record holds GPRT_BOUND_HIT). */
int gprt_intersect_host(gprt_scene* scene, const gprt_ray* rays, uint32_t n, uint32_t flags,
                        gprt_hit* hits);
/* Algorithmic work of a host ray batch on this scene's BVH, counted by a CPU
 * walk of the device layout: per-ray node visits (4-wide nodes), child-box
 * tests and primitive tests, summed.  Instrumentation for roofline figures. */
int gprt_traversal_counts(gprt_scene* scene, const gprt_ray* rays, uint32_t n, uint32_t flags,
                          uint64_t* node_visits, uint64_t* box_tests, uint64_t* prim_tests);

/* ---- progressive jobs ----------------------------------------------------
 * Replaces renderer.NewProgressiveRaytracer + integrator constructors
 * (pkg/renderer/progressive.go:62-95).  The job owns its film
 * (PixelStats per pixel, pkg/renderer/stats.go:20-55) on the device. */
int gprt_job_create(gprt_scene* scene, const gprt_job_desc* desc, gprt_job** out);
int gprt_job_destroy(gprt_job* job);
/* (*ProgressiveRaytracer).RenderPass (progressive.go:126-223): brings every
 * pixel to the pass target of getSamplesForPass (progressive.go:98-123) with
 * the adaptive stop of tile_renderer.go:51-101, then applies the pass's BDPT
 * splats (progressive.go:371-391).  Synchronous. */
int gprt_job_render_pass(gprt_job* job, uint32_t pass_number, gprt_render_stats* stats);
/* Adds exactly `spp` samples to every pixel (no adaptive stop).  Asynchronous
 * on the job stream; splats are applied. */
int gprt_job_add_samples(gprt_job* job, uint32_t spp);
int gprt_job_sync(gprt_job* job);
/* Film read-back (host pointers): per-pixel ColorAccum (3 floats), luminance
 * sum, luminance-squared sum and sample count; any pointer may be NULL. */
int gprt_job_read_film(gprt_job* job, float* rgb_sum, float* lum_sum, float* lum2_sum,
                       uint32_t* count);
/* PixelStats.GetColor for every pixel: ColorAccum / SampleCount (3 floats/pixel). */
int gprt_job_read_image(gprt_job* job, float* rgb_mean);
/* assembleCurrentImage + vec3ToColor (progressive.go:395-495): RGBA8, gamma 2. */
int gprt_job_read_rgba8(gprt_job* job, uint8_t* rgba);
/* extractTileImage (progressive.go:225-255) for pixel bounds [x0,x1) x [y0,y1). */
int gprt_job_read_tile(gprt_job* job, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                       uint8_t* rgba);
/* Stats of the last pass (assembleCurrentImage statistics). */
int gprt_job_get_stats(gprt_job* job, gprt_render_stats* stats);
/* Kernel launches issued by this job so far (instrumentation). */
int gprt_job_launch_count(const gprt_job* job, uint64_t* launches);
/* Synchronises the job and returns / clears its instrumentation. */
int gprt_job_get_counters(gprt_job* job, gprt_job_counters* out);
int gprt_job_reset_counters(gprt_job* job);
/* The cudaStream_t every kernel of the job is launched on. */
int gprt_job_stream(gprt_job* job, void** stream);

/* ---- autotuning ------------------------------------------------------------
 * No counterpart in the reference (its worker count is the only knob,
 * pkg/renderer/worker_pool.go:49-52).  Times candidate wavefront sizes,
 * traversal variants (GPRT_JOB_SIMPLE_*) and block sizes on tuning passes of
 * `spp` samples per pixel of `scene` with the integrator of `base`
 * (coordinate descent, each candidate timed with CUDA events after one
 * warm-up pass) and returns the fastest configuration; apply it by copying
 * flags / block_size / chunk_paths into the gprt_job_desc of later jobs. */
typedef struct gprt_tune_result {
  uint32_t flags;        /* GPRT_JOB_SIMPLE_* bits of the fastest configuration */
  uint32_t block_size;
  uint32_t chunk_paths;
  uint32_t candidates;   /* configurations timed */
  double best_ms;        /* one tuning pass with the chosen configuration */
  double default_ms;     /* the same pass with the default configuration */
} gprt_tune_result;
int gprt_autotune(gprt_scene* scene, const gprt_job_desc* base, uint32_t spp, gprt_tune_result* out);

/* ---- allocation-free rendering ---------------------------------------------
 * No counterpart in the reference.  Some callers cannot allocate device
 * memory when they render: a plugin inside a host application that owns the
 * GPU's memory through its own allocator (a cudaMalloc behind that
 * allocator's back can fail or fragment what it manages), and render loops
 * whose device-memory budget is fixed when they start, which must not grow
 * or fail later.  This entry point allocates nothing.  It path-traces `spp`
 * samples per pixel of `scene` (samples 0..spp-1 of the counter-based
 * sampler keyed by `seed`, the same samples a fresh job with that seed
 * takes) and writes the per-pixel mean radiance, 3 floats per pixel
 * (PixelStats.GetColor), into the caller's DEVICE buffer `rgb_out`.  The
 * path state lives in one statically sized device array inside the library
 * (GPRT_NOALLOC_MAX_PATHS paths, about 34 MB, held by every GPU that loads
 * the library until the process exits); requests with
 * width * height * spp > GPRT_NOALLOC_MAX_PATHS return GPRT_E_INVALID.  It
 * calls no cudaMalloc or cudaFree.  The first call through a context looks
 * up the array's device address (cudaGetSymbolAddress, with the context's
 * device current) and keeps it in the context, so make that first call
 * before any stream capture; a device reset invalidates the address together
 * with the context, so contexts made before a reset must not be used after
 * it.  All calls share the array and a call starts by clearing the counters
 * it keeps there: calls that overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.  Asynchronous on
 * `stream` (NULL = the context stream).
 * Device bounds: when a path overflowed its traversal stack the image is not
 * valid.  The call then fills `rgb_out` with NaN and, when `status_out` (a
 * DEVICE pointer to one uint32, may be NULL) is given, writes the device
 * error bits there (0: the image is valid; bit 0: traversal stack).  Read it
 * after synchronising `stream`; the return code only covers the launches. */
#define GPRT_NOALLOC_MAX_PATHS 131072u
int gprt_render_noalloc(gprt_scene* scene, uint32_t spp, uint64_t seed, float* rgb_out, uint32_t* status_out,
                        void* stream);

/* ---- serving ---------------------------------------------------------------
 * The reference serves concurrent progressive renders from its web server:
 * one ProgressiveRaytracer per HTTP request, each with its own NumCPU worker
 * pool, no admission control and no batching (web/server/render.go:45-82,
 * 183-227; the pass loop is RenderProgressive, progressive.go:286-368).
 * A gprt_server is the device-resident equivalent with continuous batching:
 *   - requests (a scene + a gprt_job_desc pass schedule) are submitted from
 *     any thread and queue in arrival order;
 *   - admission copies the scene's BVH and primitives into a device pool
 *     shared by all jobs (scenes submitted several times are held once) and
 *     gives the job its film; a request is admitted when its bytes fit the
 *     HBM budget (refused at once when they never can);
 *   - every step packs the next samples of many admitted jobs into ONE
 *     wavefront (raygen -> [extend -> shade -> shadow] x depth ->
 *     accumulate, the bounce sequence replayed as a captured CUDA graph),
 *     so jobs of any size share each launch; jobs admitted while others are
 *     in flight join the next step;
 *   - a pass of a job completes when all its samples are accumulated; events
 *     report admission, every pass (with host timestamps for time-to-first-
 *     pass and per-pass latency), completion, refusal and cancellation.
 * Passes follow getSamplesForPass (progressive.go:98-123) over
 * initial_samples / max_samples_per_pixel / max_passes of the request's
 * gprt_job_desc, with the scene's adaptive stop as gprt_job_render_pass
 * applies it (tile_renderer.go:51-101): a scene with adaptive_min_samples <
 * 1 brings every pixel to the pass minimum, then takes rounds of one sample
 * per pixel still active (below the pass target and not converged), one
 * round per step, until no pixel is; the pass event then reports the
 * average sample count, and the job ends when that reaches
 * max_samples_per_pixel or after max_passes (progressive.go:339-361).  A
 * job's film equals, bit for bit, the film of a gprt_job with the same
 * scene and seed given the same samples (gprt_job_add_samples, or
 * gprt_job_render_pass per pass): each sample is keyed by (seed, pixel,
 * sample index) and each pixel accumulates its samples in order, whatever
 * else shares the wavefront.  BDPT requests
 * (integrator = GPRT_INTEGRATOR_BDPT) are admitted with a private copy of
 * the scene and the BDPT working set of one chunk (both counted against the
 * budget, held until release); each step renders, beside the batched
 * path-tracing wavefront and on the job's own stream, up to 2^18 samples
 * (whole samples per pixel) of one BDPT job's pass, or one round of its
 * adaptive pass: jobs before their first pass first, then the least
 * recently served.  Their film equals that of a
 * gprt_job on the same scene given the same samples, up to the summation
 * order of the light-tracing splats (float atomics; applied after each
 * slice). */
typedef struct gprt_server_desc {
  uint64_t hbm_budget_bytes; /* device bytes held at most: path state + scene pool + films (0: 60 GiB) */
  uint32_t max_jobs;         /* admitted (unreleased) jobs at most (0: 1024) */
  uint32_t step_paths;       /* path capacity of one step's wavefront (0: 1 << 22) */
  uint32_t block_size;       /* threads per block of raygen / shade / accumulate (0: 128) */
  uint32_t flags;            /* GPRT_SERVER_* and GPRT_JOB_* bits (variants and instrumentation) */
} gprt_server_desc;
#define GPRT_SERVER_NO_GRAPHS 16u /* launch each bounce kernel instead of replaying a captured graph */

enum {
  GPRT_EV_ADMITTED = 1,  /* the request holds a film and its scene is resident */
  GPRT_EV_PASS = 2,      /* a pass completed (PassResult, progressive.go:258-263) */
  GPRT_EV_DONE = 3,      /* the last pass completed; the film stays until released */
  GPRT_EV_REFUSED = 4,   /* never fits the budget, or invalid (status = GPRT_E_*) */
  GPRT_EV_CANCELLED = 5, /* gprt_server_cancel, or its scene was destroyed before admission */
  GPRT_EV_FAILED = 6     /* a device error ended the job (status = GPRT_E_*) */
};
typedef struct gprt_event {
  uint64_t ticket;
  uint32_t kind;              /* GPRT_EV_* */
  uint32_t pass_number;       /* passes completed */
  uint32_t samples_per_pixel; /* samples every pixel of the film holds (adaptive scenes: their average, truncated) */
  int32_t status;
  double t_ms;                /* host time of the event, ms since the server was created */
  double submit_ms;           /* host time the request was submitted */
} gprt_event;

typedef struct gprt_server_stats {
  uint64_t steps, graph_launches, kernels, samples, paths;
  uint64_t submitted, admitted, finished, refused, cancelled;
  uint32_t active_jobs, pending_jobs, resident_scenes, reserved;
  uint64_t bytes_in_use, bytes_budget, pool_bytes, path_state_bytes;
  double busy_ms;             /* device time of all steps (CUDA events) */
  double last_step_ms;
  uint32_t step_paths, block_size, flags, max_jobs;
} gprt_server_stats;

int gprt_server_create(gprt_ctx* ctx, const gprt_server_desc* desc, gprt_server** out);
/* Stops the loop thread, cancels what is pending and frees every film and the pool. */
int gprt_server_destroy(gprt_server* server);
/* Queues a request; the scene must stay alive until the request is admitted
 * (destroying it earlier cancels the request).  Thread-safe. */
int gprt_server_submit(gprt_server* server, gprt_scene* scene, const gprt_job_desc* desc, uint64_t* ticket);
/* Cancels a pending or running request (its film is released). */
int gprt_server_cancel(gprt_server* server, uint64_t ticket);
/* Runs one step on the calling thread: admission, one batched wavefront,
 * events.  *busy = admitted-but-unfinished plus pending requests after it. */
int gprt_server_step(gprt_server* server, uint32_t* busy);
/* Starts / stops a loop thread that steps whenever there is work. */
int gprt_server_start(gprt_server* server);
int gprt_server_stop(gprt_server* server);
/* Takes up to `max` events, waiting up to timeout_ms for the first one. */
int gprt_server_poll(gprt_server* server, gprt_event* events, uint32_t max, uint32_t timeout_ms, uint32_t* n);
/* Film / image of an admitted job (in flight or done), as gprt_job_read_*.
 * The image reads (rgb mean, RGBA8, tile) resolve and copy on the server's
 * own read-back stream after the steps queued so far, and wait without
 * holding up the server's loop thread: a front door reads each image as its
 * event arrives while the other jobs keep rendering (one read at a time). */
int gprt_server_read_film(gprt_server* server, uint64_t ticket, float* rgb_sum, float* lum_sum, float* lum2_sum,
                          uint32_t* count);
int gprt_server_read_image(gprt_server* server, uint64_t ticket, float* rgb_mean);
int gprt_server_read_rgba8(gprt_server* server, uint64_t ticket, uint8_t* rgba);
/* The RGBA8 bytes of tile [x0, x1) x [y0, y1) of a job's current image
 * (extractTileImage, pkg/renderer/progressive.go:225-255): resolved on the
 * device, only the tile's bytes cross to the host, row-major, 4 bytes per
 * pixel.  Every tile of a pass is complete when the job's GPRT_EV_PASS event
 * is emitted, so a front door streams TileCompletionResult events
 * (progressive.go:266-276) by reading the tiles after each pass event. */
int gprt_server_read_tile(gprt_server* server, uint64_t ticket, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                          uint8_t* rgba);
/* Frees the film of a finished (or cancels and frees a running) job. */
int gprt_server_release(gprt_server* server, uint64_t ticket);
int gprt_server_get_stats(gprt_server* server, gprt_server_stats* stats);
/* Per-kernel-class launch times and traversal counters of the steps run with
 * GPRT_JOB_TIME_KERNELS / GPRT_JOB_COUNT_TRAVERSAL in the server's flags
 * (summed since the last reset; reset != 0 clears them after reading). */
int gprt_server_get_counters(gprt_server* server, gprt_job_counters* out, int reset);
/* The cudaStream_t every kernel and copy of the server runs on. */
int gprt_server_stream(gprt_server* server, void** stream);
/* Changes the step size / block size / GPRT_JOB_SIMPLE_* variant between steps
 * (step_paths up to the capacity given at creation). */
int gprt_server_configure(gprt_server* server, uint32_t step_paths, uint32_t block_size, uint32_t flags);
/* Autotuner of the batched loop: times candidate step sizes, block sizes and
 * traversal variants on steps of the jobs currently admitted, without adding
 * their samples to any film, and applies the configuration with the highest
 * samples per second among those whose step takes at most max_step_ms
 * (0: no limit).  Needs admitted, unfinished jobs. */
int gprt_server_autotune(gprt_server* server, double max_step_ms, gprt_tune_result* out);

/* ---- loaders ------------------------------------------------------------
 * PBRT-v4 subset scenes (loaders.LoadPBRT / ParsePBRT, pkg/loaders/pbrt.go)
 * converted as scene.NewPBRTScene does (pkg/scene/pbrt_scene.go): the
 * loaded handle owns a gprt_scene_desc (and its arrays) valid until
 * gprt_loaded_free, ready for gprt_scene_create.  camera_override may be
 * NULL (its non-zero fields win, MergeCameraConfig).  gprt_pbrt_load keeps
 * the reference's path rules (validateFilePath, pbrt.go:391-433: under a
 * scenes/ directory or the temporary directory, .pbrt, at most 512 bytes).
 * Errors: GPRT_E_INVALID with the reference's message in errbuf.  Needs no
 * GPU. */
typedef struct gprt_loaded gprt_loaded;
int gprt_pbrt_parse(const char* text, size_t len, const gprt_camera_desc* camera_override,
                    gprt_loaded** out, char* errbuf, size_t err_len);
int gprt_pbrt_load(const char* path, const gprt_camera_desc* camera_override, gprt_loaded** out,
                   char* errbuf, size_t err_len);
const gprt_scene_desc* gprt_loaded_desc(const gprt_loaded* loaded);
void gprt_loaded_free(gprt_loaded* loaded);

/* Binary little-endian PLY meshes (loaders.LoadPLY, pkg/loaders/ply.go):
 * float x, y, z (and nx, ny, nz / u, v; uchar red, green, blue as [0,1]),
 * triangular faces.  The arrays (3 doubles per vertex, 3 indices per
 * triangle, 2 doubles per texture coordinate) feed gprt_mesh_desc directly
 * and stay valid until gprt_ply_free; absent attributes return NULL. */
typedef struct gprt_ply gprt_ply;
typedef struct gprt_ply_info {
  uint32_t n_vertices;
  uint32_t n_triangles;
  uint32_t has_normals;
  uint32_t has_colors;
  uint32_t has_texcoords;
  uint32_t reserved;
} gprt_ply_info;
int gprt_ply_load(const char* path, gprt_ply** out, char* errbuf, size_t err_len);
int gprt_ply_get(const gprt_ply* ply, gprt_ply_info* info, const double** vertices,
                 const uint32_t** indices, const double** normals, const double** colors,
                 const double** texcoords);
void gprt_ply_free(gprt_ply* ply);

#ifdef __cplusplus
}
#endif
#endif /* GPRT_H */
