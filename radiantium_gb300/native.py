"""ctypes view of the C ABI in include/radiantium.h and the loader of the CUDA library.

The structures below are field-for-field copies of the C declarations.  The
loader never falls back to anything: if the compiled library is missing the
import of :func:`lib` raises, naming the build step.
"""
from __future__ import annotations

import ctypes as C
import os

ABI_VERSION = 2

RT_OK = 0
RT_ERR_INVALID_ARG = -1
RT_ERR_OOM = -2
RT_ERR_CUDA = -3
RT_ERR_ITER_CAP = -4
RT_ERR_CANCELLED = -5
RT_ERR_NO_SCENE = -6
RT_ERR_UNSUPPORTED = -7
RT_ERR_STACK = -8
RT_ERR_BOUNDS = -9

WRAP_CLAMP, WRAP_REPEAT = 0, 1
FILTER_NEAREST, FILTER_LINEAR = 0, 1
MAT_DIFFUSE, MAT_ROUGH_METAL, MAT_ROUGH_GLASS, MAT_ROUGH_PLASTIC, MAT_PERFECT_MIRROR, MAT_PERFECT_GLASS = range(6)
DIST_BECKMANN, DIST_GGX = 0, 1
GROUP_MESH, GROUP_SPHERE, GROUP_INSTANCE, GROUP_INFINITE_LIGHT = range(4)
INTEGRATOR_PATH, INTEGRATOR_VOL_PATH, INTEGRATOR_PARTICLE = 0, 1, 2
PARTICLE_STREAM = 0x80000000
METHOD_BXDF, METHOD_NEE, METHOD_MIS = 0, 1, 2
STRATEGY_UNIFORM, STRATEGY_ALL = 0, 1
HIT_TIE = 1

FloatP = C.POINTER(C.c_float)
IntP = C.POINTER(C.c_int32)


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("wrap", C.c_int32), ("filter", C.c_int32),
                ("data", FloatP)]


class MaterialDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("dist", C.c_int32), ("two_sided", C.c_int32), ("tex_r", C.c_int32),
                ("tex_t", C.c_int32), ("tex_roughness", C.c_int32), ("tex_anisotropic", C.c_int32),
                ("eta_a", C.c_float), ("eta_b", C.c_float), ("kd", C.c_float), ("ks", C.c_float),
                ("eta", C.c_float * 3), ("k", C.c_float * 3)]


class MediumDesc(C.Structure):
    _fields_ = [("sigma_a", C.c_float * 3), ("sigma_s", C.c_float * 3), ("g", C.c_float), ("scale", C.c_float)]


class MeshDesc(C.Structure):
    _fields_ = [("vertex_count", C.c_int32), ("triangle_count", C.c_int32), ("positions", FloatP),
                ("normals", FloatP), ("uvs", FloatP), ("indices", IntP)]


class SphereDesc(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("model_to_world", C.c_float * 16),
                ("world_to_model", C.c_float * 16)]


class GroupDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ref", C.c_int32), ("material", C.c_int32), ("medium_inside", C.c_int32),
                ("medium_outside", C.c_int32), ("emissive", C.c_int32), ("le", C.c_float * 3),
                ("model_to_world", C.c_float * 16), ("world_to_model", C.c_float * 16)]


class CameraDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("near_z", C.c_float), ("far_z", C.c_float),
                ("clip_to_camera", C.c_float * 16), ("camera_to_world", C.c_float * 16),
                ("camera_to_clip", C.c_float * 16), ("world_to_camera", C.c_float * 16)]


class SceneDescC(C.Structure):
    _fields_ = [("abi_version", C.c_int32),
                ("mesh_count", C.c_int32), ("meshes", C.POINTER(MeshDesc)),
                ("sphere_count", C.c_int32), ("spheres", C.POINTER(SphereDesc)),
                ("texture_count", C.c_int32), ("textures", C.POINTER(TextureDesc)),
                ("material_count", C.c_int32), ("materials", C.POINTER(MaterialDesc)),
                ("medium_count", C.c_int32), ("media", C.POINTER(MediumDesc)),
                ("blas_group_count", C.c_int32), ("blas_groups", C.POINTER(GroupDesc)),
                ("blas_count", C.c_int32), ("blas_ranges", IntP),
                ("group_count", C.c_int32), ("groups", C.POINTER(GroupDesc)),
                ("global_medium", C.c_int32),
                ("camera", CameraDesc),
                ("bvh_max_prims", C.c_int32)]


class Ray(C.Structure):
    _fields_ = [("o", C.c_float * 3), ("d", C.c_float * 3), ("min_t", C.c_float), ("max_t", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("prim", C.c_int32), ("sub", C.c_int32),
                ("flags", C.c_uint32)]


class RenderParams(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("method", C.c_int32), ("strategy", C.c_int32),
                ("max_depth", C.c_int32), ("min_depth", C.c_int32), ("rr_threshold", C.c_float),
                ("spp", C.c_int32), ("sample_begin", C.c_int32), ("seed", C.c_uint64),
                ("x0", C.c_int32), ("y0", C.c_int32), ("width", C.c_int32), ("height", C.c_int32)]


class AdjointDesc(C.Structure):
    _fields_ = [("albedo_texture", C.c_int32), ("alpha_count", C.c_int32),
                ("alpha_materials", C.POINTER(C.c_int32))]


class BatchItem(C.Structure):
    _fields_ = [("scene_ctx", C.c_void_p), ("params", RenderParams), ("out_rgb", C.c_void_p)]


class TuneResult(C.Structure):
    _fields_ = [("capacity", C.c_int32), ("refill", C.c_int32), ("renderer", C.c_int32), ("ms", C.c_float),
                ("ms_default", C.c_float)]


class Stats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("rays_closest", C.c_uint64), ("rays_shadow", C.c_uint64),
                ("node_visits", C.c_uint64), ("prim_tests", C.c_uint64), ("instance_visits", C.c_uint64),
                ("invalid_samples", C.c_uint64), ("kernel_launches", C.c_uint64), ("render_launches", C.c_uint64),
                ("render_kernel_ms", C.c_double), ("shade_kernel_ms", C.c_double), ("h2d_bytes", C.c_uint64)]

    def as_dict(self):
        d = {k: int(getattr(self, k)) for k, _ in self._fields_ if k not in ("render_kernel_ms", "shade_kernel_ms")}
        d["render_kernel_ms"] = float(self.render_kernel_ms)
        d["shade_kernel_ms"] = float(self.shade_kernel_ms)
        return d


# numpy structured dtypes with the same layout (rays/hits are passed as arrays)
def ray_dtype():
    import numpy as np
    return np.dtype([("o", "<f4", 3), ("d", "<f4", 3), ("min_t", "<f4"), ("max_t", "<f4")])


def hit_dtype():
    import numpy as np
    return np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<i4"), ("sub", "<i4"), ("flags", "<u4")])


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
# RADIANTIUM_GB300_LIB selects another build of the library (e.g. a debug-bounds variant)
LIB_PATH = os.environ.get("RADIANTIUM_GB300_LIB") or os.path.join(PKG_DIR, "_lib", "libradiantium_gb300.so")

# every symbol include/radiantium.h declares
EXPORTED_SYMBOLS = [
    "rt_abi_version", "rt_create", "rt_destroy", "rt_last_error", "rt_upload_scene",
    "rt_trace_closest", "rt_trace_any", "rt_trace_closest_device", "rt_trace_any_device",
    "rt_render", "rt_render_device", "rt_adjoint_forward", "rt_adjoint_backward", "rt_update_texture", "rt_render_device_noalloc", "rt_render_batch", "rt_render_batch_device", "rt_autotune", "rt_get_stats", "rt_set_counting",
    "rt_set_renderer", "rt_set_traversal", "rt_get_traversal", "rt_set_light_sampling", "rt_get_light_sampling", "rt_cancel", "rt_render_particles", "rt_render_particles_device",
]
RENDERER_AUTO, RENDERER_MEGAKERNEL, RENDERER_WAVEFRONT, RENDERER_WAVEFRONT_GRAPH = 0, 1, 2, 3
TRAVERSAL_EXACT, TRAVERSAL_WIDE = 0, 1
LIGHT_SAMPLING_CDF, LIGHT_SAMPLING_ALIAS = 0, 1
MAX_BATCH = 256
ADJ_MAX_ALPHA = 1024
MAX_SLOTS = 1 << 21       # path slots in flight (wavefront)
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024   # RT_NOALLOC_SCRATCH_BYTES

_lib = None


def _declare(lib):
    vp = C.c_void_p
    lib.rt_abi_version.restype = C.c_int
    lib.rt_abi_version.argtypes = []
    lib.rt_create.restype = C.c_int
    lib.rt_create.argtypes = [C.c_int, C.POINTER(vp)]
    lib.rt_destroy.restype = None
    lib.rt_destroy.argtypes = [vp]
    lib.rt_last_error.restype = C.c_char_p
    lib.rt_last_error.argtypes = [vp]
    lib.rt_upload_scene.restype = C.c_int
    lib.rt_upload_scene.argtypes = [vp, C.POINTER(SceneDescC)]
    lib.rt_trace_closest.restype = C.c_int
    lib.rt_trace_closest.argtypes = [vp, vp, C.c_int64, vp]
    lib.rt_trace_any.restype = C.c_int
    lib.rt_trace_any.argtypes = [vp, vp, C.c_int64, vp]
    lib.rt_trace_closest_device.restype = C.c_int
    lib.rt_trace_closest_device.argtypes = [vp, vp, C.c_int64, vp, vp]
    lib.rt_trace_any_device.restype = C.c_int
    lib.rt_trace_any_device.argtypes = [vp, vp, C.c_int64, vp, vp]
    lib.rt_render.restype = C.c_int
    lib.rt_render.argtypes = [vp, C.POINTER(RenderParams), vp]
    lib.rt_render_device.restype = C.c_int
    lib.rt_render_device.argtypes = [vp, C.POINTER(RenderParams), vp, vp]
    lib.rt_render_device_noalloc.restype = C.c_int
    lib.rt_render_device_noalloc.argtypes = [vp, C.POINTER(RenderParams), vp, vp]
    lib.rt_get_stats.restype = C.c_int
    lib.rt_get_stats.argtypes = [vp, C.POINTER(Stats)]
    lib.rt_set_counting.restype = C.c_int
    lib.rt_set_counting.argtypes = [vp, C.c_int]
    lib.rt_adjoint_forward.restype = C.c_int
    lib.rt_adjoint_forward.argtypes = [vp, C.POINTER(RenderParams), vp]
    lib.rt_adjoint_backward.restype = C.c_int
    lib.rt_adjoint_backward.argtypes = [vp, C.POINTER(RenderParams), C.POINTER(AdjointDesc), vp, vp, vp]
    lib.rt_update_texture.restype = C.c_int
    lib.rt_update_texture.argtypes = [vp, C.c_int, vp]
    lib.rt_autotune.restype = C.c_int
    lib.rt_autotune.argtypes = [vp, C.POINTER(BatchItem), C.c_int, C.POINTER(TuneResult)]
    lib.rt_render_batch.restype = C.c_int
    lib.rt_render_batch.argtypes = [vp, C.POINTER(BatchItem), C.c_int]
    lib.rt_render_batch_device.restype = C.c_int
    lib.rt_render_batch_device.argtypes = [vp, C.POINTER(BatchItem), C.c_int, vp]
    lib.rt_set_renderer.restype = C.c_int
    lib.rt_set_renderer.argtypes = [vp, C.c_int]
    lib.rt_set_traversal.restype = C.c_int
    lib.rt_set_traversal.argtypes = [vp, C.c_int]
    lib.rt_get_traversal.restype = C.c_int
    lib.rt_get_traversal.argtypes = [vp, C.POINTER(C.c_int)]
    lib.rt_set_light_sampling.restype = C.c_int
    lib.rt_set_light_sampling.argtypes = [vp, C.c_int]
    lib.rt_get_light_sampling.restype = C.c_int
    lib.rt_get_light_sampling.argtypes = [vp, C.POINTER(C.c_int)]
    lib.rt_debug_env_sample.restype = C.c_int
    lib.rt_debug_env_sample.argtypes = [vp, C.c_int, vp, C.c_int64, vp, vp]
    lib.rt_debug_alias.restype = C.c_int
    lib.rt_debug_alias.argtypes = [vp, C.c_int, vp]
    lib.rt_cancel.restype = C.c_int
    lib.rt_cancel.argtypes = [vp]
    lib.rt_render_particles.restype = C.c_int
    lib.rt_render_particles.argtypes = [vp, C.POINTER(RenderParams), C.c_int64, C.c_int64, vp]
    lib.rt_render_particles_device.restype = C.c_int
    lib.rt_render_particles_device.argtypes = [vp, C.POINTER(RenderParams), C.c_int64, C.c_int64, vp, vp]
    lib.rt_debug_particle_splats.restype = C.c_int
    lib.rt_debug_particle_splats.argtypes = [vp, C.POINTER(RenderParams), C.c_int64, C.c_int64, C.c_int, vp, vp, vp]
    return lib


def load_library(path: str | None = None):
    """Loads the CUDA library; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"radiantium_gb300: CUDA library {p} is missing; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = _declare(C.CDLL(p, mode=C.RTLD_GLOBAL))
    if lib.rt_abi_version() != ABI_VERSION:
        raise RuntimeError("radiantium_gb300: ABI version mismatch between radiantium.h and the built library")
    if path is None:
        _lib = lib
    return lib


class RTError(RuntimeError):
    """A negative status returned by the library (the C# shim maps it to InvalidOperationException)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"radiantium_gb300 error {code}: {msg}")
        self.code = code
