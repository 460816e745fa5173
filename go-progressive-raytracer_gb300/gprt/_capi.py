"""ctypes binding of include/gprt.h.

Loads the in-tree ``_build/libgprt.so`` (or the build named by the GPRT_LIB
environment variable); there is no other implementation, so a missing
library is an error (build it with ``build.py`` or ``__graft_entry__.build()``).
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libgprt.so")

GPRT_OK = 0
GPRT_E_INVALID = -1
GPRT_E_OOM = -2
GPRT_E_DEVICE = -3
GPRT_E_BOUND = -4
GPRT_E_CANCELLED = -5
GPRT_E_ADMISSION = -6
GPRT_E_NOT_FOUND = -7

MAT_LAMBERTIAN, MAT_METAL, MAT_DIELECTRIC, MAT_EMISSIVE, MAT_LAYERED, MAT_SPOT_EMISSIVE, MAT_MIX = range(7)
SHAPE_SPHERE, SHAPE_QUAD, SHAPE_BOX, SHAPE_MESH, SHAPE_TRIANGLE, SHAPE_DISC, SHAPE_CYLINDER, SHAPE_CONE = range(8)
NO_SHAPE = 0xFFFFFFFF
(LIGHT_QUAD, LIGHT_SPHERE, LIGHT_UNIFORM_INFINITE, LIGHT_GRADIENT_INFINITE, LIGHT_DISC, LIGHT_DISC_SPOT,
 LIGHT_POINT_SPOT) = range(7)
INTEGRATOR_PATH_TRACING, INTEGRATOR_BDPT = 0, 1
CLOSEST, ANY = 0, 1
NO_HIT = 0xFFFFFFFF
BOUND_HIT = 0xFFFFFFFE  # GPRT_BOUND_HIT: the ray's traversal stack overflowed
BUILD_DEVICE = 1
BUILD_TEST_STACK_CAP = 2  # tests only: 1-entry traversal stack, so the scene's rays overflow it
NOALLOC_MAX_PATHS = 131072  # GPRT_NOALLOC_MAX_PATHS


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("pixels", C.POINTER(C.c_double))]


class MaterialDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("outer", C.c_uint32), ("inner", C.c_uint32), ("texture", C.c_uint32),
                ("albedo", C.c_double * 3), ("fuzz", C.c_double), ("ior", C.c_double),
                ("emission", C.c_double * 3)]


class ShapeDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("material", C.c_uint32), ("mesh", C.c_uint32), ("reserved", C.c_uint32),
                ("p", C.c_double * 9)]


class MeshDesc(C.Structure):
    _fields_ = [("vertices", C.POINTER(C.c_double)), ("indices", C.POINTER(C.c_uint32)),
                ("tri_materials", C.POINTER(C.c_uint32)), ("n_vertices", C.c_uint32), ("n_triangles", C.c_uint32),
                ("tri_normals", C.POINTER(C.c_double)), ("vertex_uvs", C.POINTER(C.c_double))]


class LightDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("shape", C.c_uint32), ("color_a", C.c_double * 3),
                ("color_b", C.c_double * 3), ("weight", C.c_double), ("from_", C.c_double * 3), ("to", C.c_double * 3),
                ("cone_deg", C.c_double), ("cone_delta_deg", C.c_double), ("radius", C.c_double)]


class CameraDesc(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("look_at", C.c_double * 3), ("up", C.c_double * 3),
                ("aspect_ratio", C.c_double), ("vfov_deg", C.c_double), ("aperture", C.c_double),
                ("focus_distance", C.c_double), ("width", C.c_uint32), ("reserved", C.c_uint32)]


class SamplingDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("samples_per_pixel", C.c_uint32),
                ("max_depth", C.c_uint32), ("rr_min_bounces", C.c_uint32), ("reserved", C.c_uint32),
                ("adaptive_min_samples", C.c_double), ("adaptive_threshold", C.c_double)]


class SceneDesc(C.Structure):
    _fields_ = [("materials", C.POINTER(MaterialDesc)), ("shapes", C.POINTER(ShapeDesc)),
                ("meshes", C.POINTER(MeshDesc)), ("lights", C.POINTER(LightDesc)),
                ("n_materials", C.c_uint32), ("n_shapes", C.c_uint32), ("n_meshes", C.c_uint32),
                ("n_lights", C.c_uint32), ("weighted_sampler", C.c_uint32), ("build_flags", C.c_uint32),
                ("camera", CameraDesc), ("sampling", SamplingDesc), ("textures", C.POINTER(TextureDesc)),
                ("n_textures", C.c_uint32), ("reserved", C.c_uint32)]


class Ray(C.Structure):
    _fields_ = [("ox", C.c_float), ("oy", C.c_float), ("oz", C.c_float), ("tmin", C.c_float),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("tmax", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_uint32), ("u", C.c_float), ("v", C.c_float)]


class SceneInfo(C.Structure):
    _fields_ = [("world_center", C.c_double * 3), ("world_radius", C.c_double), ("n_primitives", C.c_uint64),
                ("n_triangles", C.c_uint64), ("n_quads", C.c_uint64), ("n_spheres", C.c_uint64),
                ("n_nodes", C.c_uint64), ("device_bytes", C.c_uint64), ("image_width", C.c_uint32),
                ("image_height", C.c_uint32), ("build_ms", C.c_double), ("flatten_ms", C.c_double),
                ("bvh_ms", C.c_double), ("check_ms", C.c_double), ("n_quadrics", C.c_uint64)]


class JobDesc(C.Structure):
    _fields_ = [("integrator", C.c_uint32), ("tile_size", C.c_uint32), ("initial_samples", C.c_uint32),
                ("max_samples_per_pixel", C.c_uint32), ("max_passes", C.c_uint32), ("chunk_paths", C.c_uint32),
                ("block_size", C.c_uint32), ("flags", C.c_uint32), ("seed", C.c_uint64)]


JOB_TIME_KERNELS = 1
JOB_COUNT_TRAVERSAL = 2
JOB_SIMPLE_EXTEND = 4
JOB_SIMPLE_SHADOW = 8
JOB_SHADE_OCCUPANCY = 32


class TuneResult(C.Structure):
    _fields_ = [("flags", C.c_uint32), ("block_size", C.c_uint32), ("chunk_paths", C.c_uint32),
                ("candidates", C.c_uint32), ("best_ms", C.c_double), ("default_ms", C.c_double)]


class JobCounters(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("extend_launches", "shade_launches", "shadow_launches", "other_launches")] + \
        [(n, C.c_double) for n in ("extend_ms", "shade_ms", "shadow_ms", "other_ms")] + \
        [(n, C.c_uint64) for n in ("extend_rays", "shadow_rays", "extend_nodes", "extend_boxes", "extend_prims",
                                   "shadow_nodes", "shadow_boxes", "shadow_prims")]


class RenderStats(C.Structure):
    _fields_ = [("total_pixels", C.c_uint64), ("total_samples", C.c_uint64), ("average_samples", C.c_double),
                ("max_samples", C.c_uint32), ("min_samples", C.c_uint32), ("max_samples_used", C.c_uint32),
                ("pass_number", C.c_uint32), ("pass_ms", C.c_double), ("splats", C.c_uint64)]


class ServerDesc(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_jobs", C.c_uint32), ("step_paths", C.c_uint32),
                ("block_size", C.c_uint32), ("flags", C.c_uint32)]


SERVER_NO_GRAPHS = 16
EV_ADMITTED, EV_PASS, EV_DONE, EV_REFUSED, EV_CANCELLED, EV_FAILED = range(1, 7)
EVENT_NAMES = {EV_ADMITTED: "admitted", EV_PASS: "pass", EV_DONE: "done", EV_REFUSED: "refused",
               EV_CANCELLED: "cancelled", EV_FAILED: "failed"}


class Event(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("kind", C.c_uint32), ("pass_number", C.c_uint32),
                ("samples_per_pixel", C.c_uint32), ("status", C.c_int32), ("t_ms", C.c_double),
                ("submit_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("steps", "graph_launches", "kernels", "samples", "paths", "submitted",
                                           "admitted",
                                           "finished", "refused", "cancelled")] + \
        [(n, C.c_uint32) for n in ("active_jobs", "pending_jobs", "resident_scenes", "reserved")] + \
        [(n, C.c_uint64) for n in ("bytes_in_use", "bytes_budget", "pool_bytes", "path_state_bytes")] + \
        [(n, C.c_double) for n in ("busy_ms", "last_step_ms")] + \
        [(n, C.c_uint32) for n in ("step_paths", "block_size", "flags", "max_jobs")]


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
F32P = C.POINTER(C.c_float)
U32P = C.POINTER(C.c_uint32)
U64P = C.POINTER(C.c_uint64)
U8P = C.POINTER(C.c_uint8)
F64PP = C.POINTER(C.POINTER(C.c_double))
U32PP = C.POINTER(C.POINTER(C.c_uint32))


class PlyInfo(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("n_vertices", "n_triangles", "has_normals", "has_colors", "has_texcoords",
                                         "reserved")]


# name -> (restype, argtypes); every symbol the header declares
SIGNATURES = {
    "gprt_version": (C.c_int, []),
    "gprt_ctx_create": (C.c_int, [C.c_int, PP]),
    "gprt_ctx_destroy": (C.c_int, [P]),
    "gprt_last_error": (C.c_char_p, [P]),
    "gprt_scene_create": (C.c_int, [P, C.POINTER(SceneDesc), PP]),
    "gprt_scene_destroy": (C.c_int, [P]),
    "gprt_scene_get_info": (C.c_int, [P, C.POINTER(SceneInfo)]),
    "gprt_scene_primitive_map": (C.c_int, [P, U32P, U32P]),
    "gprt_scene_validate": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(SceneInfo), C.c_char_p, C.c_size_t]),
    "gprt_intersect": (C.c_int, [P, P, C.c_uint32, C.c_uint32, P, P]),
    "gprt_intersect_host": (C.c_int, [P, P, C.c_uint32, C.c_uint32, P]),
    "gprt_traversal_counts": (C.c_int, [P, P, C.c_uint32, C.c_uint32, U64P, U64P, U64P]),
    "gprt_job_create": (C.c_int, [P, C.POINTER(JobDesc), PP]),
    "gprt_job_destroy": (C.c_int, [P]),
    "gprt_job_render_pass": (C.c_int, [P, C.c_uint32, C.POINTER(RenderStats)]),
    "gprt_job_add_samples": (C.c_int, [P, C.c_uint32]),
    "gprt_job_sync": (C.c_int, [P]),
    "gprt_job_read_film": (C.c_int, [P, F32P, F32P, F32P, U32P]),
    "gprt_job_read_image": (C.c_int, [P, F32P]),
    "gprt_job_read_rgba8": (C.c_int, [P, U8P]),
    "gprt_job_read_tile": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, U8P]),
    "gprt_job_get_stats": (C.c_int, [P, C.POINTER(RenderStats)]),
    "gprt_job_launch_count": (C.c_int, [P, U64P]),
    "gprt_job_get_counters": (C.c_int, [P, C.POINTER(JobCounters)]),
    "gprt_job_reset_counters": (C.c_int, [P]),
    "gprt_job_stream": (C.c_int, [P, PP]),
    "gprt_render_noalloc": (C.c_int, [P, C.c_uint32, C.c_uint64, P, P, P]),
    "gprt_autotune": (C.c_int, [P, C.POINTER(JobDesc), C.c_uint32, C.POINTER(TuneResult)]),
    "gprt_server_create": (C.c_int, [P, C.POINTER(ServerDesc), PP]),
    "gprt_server_destroy": (C.c_int, [P]),
    "gprt_server_submit": (C.c_int, [P, P, C.POINTER(JobDesc), U64P]),
    "gprt_server_cancel": (C.c_int, [P, C.c_uint64]),
    "gprt_server_step": (C.c_int, [P, U32P]),
    "gprt_server_start": (C.c_int, [P]),
    "gprt_server_stop": (C.c_int, [P]),
    "gprt_server_poll": (C.c_int, [P, C.POINTER(Event), C.c_uint32, C.c_uint32, U32P]),
    "gprt_server_read_film": (C.c_int, [P, C.c_uint64, F32P, F32P, F32P, U32P]),
    "gprt_server_read_image": (C.c_int, [P, C.c_uint64, F32P]),
    "gprt_server_read_rgba8": (C.c_int, [P, C.c_uint64, U8P]),
    "gprt_server_read_tile": (C.c_int, [P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, U8P]),
    "gprt_server_release": (C.c_int, [P, C.c_uint64]),
    "gprt_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "gprt_server_get_counters": (C.c_int, [P, C.POINTER(JobCounters), C.c_int]),
    "gprt_server_stream": (C.c_int, [P, PP]),
    "gprt_server_configure": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32]),
    "gprt_server_autotune": (C.c_int, [P, C.c_double, C.POINTER(TuneResult)]),
    "gprt_pbrt_parse": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(CameraDesc), PP, C.c_char_p, C.c_size_t]),
    "gprt_pbrt_load": (C.c_int, [C.c_char_p, C.POINTER(CameraDesc), PP, C.c_char_p, C.c_size_t]),
    "gprt_loaded_desc": (C.POINTER(SceneDesc), [P]),
    "gprt_loaded_free": (None, [P]),
    "gprt_ply_load": (C.c_int, [C.c_char_p, PP, C.c_char_p, C.c_size_t]),
    "gprt_ply_get": (C.c_int, [P, C.POINTER(PlyInfo), F64PP, U32PP, F64PP, F64PP, F64PP]),
    "gprt_ply_free": (None, [P]),
}

_lib = None


def load(path=None):
    """Loads libgprt.so and declares every entry point; raises when missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("GPRT_LIB") or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libgprt.so is not built (%s); run go-progressive-raytracer_gb300/build.py" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class GprtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gprt error %d: %s" % (code, msg))
        self.code = code


def check(rc, ctx=None):
    if rc != GPRT_OK:
        msg = ""
        if ctx is not None:
            m = load().gprt_last_error(ctx)
            msg = m.decode() if m else ""
        raise GprtError(rc, msg)
