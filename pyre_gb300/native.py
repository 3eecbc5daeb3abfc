"""ctypes binding of libpyre_cuda.so (declarations mirror include/pyre_cuda.h).

The library is the only compute path: importing this module never falls back
to anything else, and every call raises ``PyreError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "libpyre_cuda.so"

PYRE_OK = 0
PYRE_ERR_INVALID = -1
PYRE_ERR_CUDA = -2
PYRE_ERR_OOM = -3
PYRE_ERR_UNSUPPORTED = -4
PYRE_ERR_OVERFLOW = -5
PYRE_ERR_TIMEOUT = -6
PYRE_MEM_HOST = 0
PYRE_MEM_DEVICE = 1
PYRE_MAT_LAMBERTIAN = 0
PYRE_MAT_DISNEY = 1
PYRE_CAMERA_PINHOLE = 0
PYRE_CAMERA_THIN_LENS = 1
PYRE_ENV_ALIAS = 0
PYRE_ENV_CDF = 1
PYRE_BVH_BUILDER_HOST, PYRE_BVH_BUILDER_DEVICE = 0, 1

F3 = C.c_float * 3
P_f = C.POINTER(C.c_float)
P_u32 = C.POINTER(C.c_uint32)
P_i32 = C.POINTER(C.c_int32)
P_u8 = C.POINTER(C.c_uint8)


class Bvh2Node(C.Structure):
    _fields_ = [("bounds_min", F3), ("bounds_max", F3), ("offset", C.c_uint32),
                ("n_primitives", C.c_uint16), ("axis", C.c_uint8), ("pad", C.c_uint8)]


BVH2_DTYPE = np.dtype([("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3), ("offset", "<u4"),
                       ("n_primitives", "<u2"), ("axis", "u1"), ("pad", "u1")])
assert BVH2_DTYPE.itemsize == C.sizeof(Bvh2Node) == 32


class MeshDesc(C.Structure):
    _fields_ = [("positions", P_f), ("n_vertices", C.c_uint32), ("indices", P_u32), ("n_triangles", C.c_uint32),
                ("normals", P_f), ("bvh_nodes", C.POINTER(Bvh2Node)), ("n_bvh_nodes", C.c_uint32),
                ("bvh_prim_indices", P_u32)]


class InstanceDesc(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("material", C.c_uint32), ("has_motion", C.c_uint32),
                ("offset_t0", F3), ("offset_t1", F3)]


class MaterialDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("base_color", F3), ("metallic", C.c_float), ("roughness", C.c_float),
                ("specular", C.c_float)]


class QuadLightDesc(C.Structure):
    _fields_ = [("p0", F3), ("edge_u", F3), ("edge_v", F3), ("emission", F3)]


class EnvDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgb", P_f), ("intensity", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("meshes", C.POINTER(MeshDesc)), ("n_meshes", C.c_uint32),
                ("instances", C.POINTER(InstanceDesc)), ("n_instances", C.c_uint32),
                ("materials", C.POINTER(MaterialDesc)), ("n_materials", C.c_uint32),
                ("lights", C.POINTER(QuadLightDesc)), ("n_lights", C.c_uint32),
                ("env", C.POINTER(EnvDesc))]


class Rays(C.Structure):
    _fields_ = [("origin", P_f), ("direction", P_f), ("t_min", P_f), ("t_max", P_f), ("time", P_f)]


class Hits(C.Structure):
    _fields_ = [("kind", P_i32), ("instance", P_i32), ("triangle", P_i32), ("t", P_f), ("u", P_f), ("v", P_f)]


class CameraDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("origin", F3), ("target", F3), ("up", F3), ("vfov_deg", C.c_float),
                ("aspect", C.c_float), ("aperture_radius", C.c_float), ("focus_distance", C.c_float)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("spp_begin", C.c_uint32), ("spp_end", C.c_uint32),
                ("max_depth", C.c_uint32), ("min_rr_depth", C.c_uint32), ("crop", C.c_uint32 * 4),
                ("env_sampling", C.c_uint32), ("wave_paths", C.c_uint32), ("block_size", C.c_uint32),
                ("sort_by_material", C.c_uint32), ("use_graph", C.c_uint32), ("refill_lanes", C.c_uint32),
                ("bvh_width", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class Film(C.Structure):
    _fields_ = [("radiance", P_f), ("albedo", P_f), ("normal", P_f), ("depth", P_f), ("mem", C.c_int)]


class BatchJob(C.Structure):
    _fields_ = [("part", C.c_uint32), ("camera", CameraDesc), ("width", C.c_uint32), ("height", C.c_uint32),
                ("spp_begin", C.c_uint32), ("spp_end", C.c_uint32), ("max_depth", C.c_uint32),
                ("min_rr_depth", C.c_uint32), ("film", Film)]


class Gradients(C.Structure):
    _fields_ = [("materials", C.POINTER(C.c_double)), ("env", P_f), ("mem", C.c_int)]


class SceneInfo(C.Structure):
    _fields_ = [("n_triangles", C.c_uint64), ("n_nodes", C.c_uint64), ("n_instances", C.c_uint64),
                ("triangle_bytes", C.c_uint64), ("node_bytes", C.c_uint64), ("device_bytes", C.c_uint64)]


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("waves", C.c_uint32), ("kernel_launches", C.c_uint32), ("ms_total", C.c_float),
                ("ms_extend", C.c_float), ("ms_shade", C.c_float), ("ms_shadow", C.c_float),
                ("ms_other", C.c_float)]


# Every entry point declared in include/pyre_cuda.h: name -> (restype, argtypes)
SIGNATURES = {
    "pyre_version": (C.c_int, []),
    "pyre_bvh_build": (C.c_int, [P_f, C.c_uint32, P_u32, C.c_uint32, C.POINTER(Bvh2Node), P_u32, P_u32]),
    "pyre_set_bvh_builder": (C.c_int, [C.c_void_p, C.c_int]),
    "pyre_inject_alloc_failure": (C.c_int, [C.c_void_p, C.c_int]),
    "pyre_distribution2d_query": (C.c_int, [C.c_void_p, P_f, C.c_uint32, C.c_uint32, C.c_int, C.c_uint32, P_f, P_f,
                                            C.c_uint32, P_f, P_f]),
    "pyre_bsdf_query": (C.c_int, [C.c_void_p, C.POINTER(MaterialDesc), C.c_uint32, P_f, P_f, P_f]),
    "pyre_bvh_build_device": (C.c_int, [C.c_void_p, P_f, C.c_uint32, P_u32, C.c_uint32, C.POINTER(Bvh2Node), P_u32,
                                        P_u32]),
    "pyre_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "pyre_ctx_destroy": (C.c_int, [C.c_void_p]),
    "pyre_last_error": (C.c_char_p, [C.c_void_p]),
    "pyre_scene_upload": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]),
    "pyre_scene_destroy": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pyre_scene_get_info": (C.c_int, [C.c_void_p, C.POINTER(SceneInfo)]),
    "pyre_scene_set_bvh_width": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "pyre_intersect_closest": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Rays), C.c_uint64, C.POINTER(Hits), C.c_int]),
    "pyre_intersect_any": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Rays), C.c_uint64, P_u8, C.c_int]),
    "pyre_render": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CameraDesc), C.POINTER(RenderParams), C.POINTER(Film)]),
    "pyre_render_progressive": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CameraDesc), C.POINTER(RenderParams),
                                          C.c_void_p, C.c_int]),
    "pyre_get_render_stats": (C.c_int, [C.c_void_p, C.POINTER(RenderStats)]),
    "pyre_render_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CameraDesc), C.POINTER(RenderParams),
                                      C.POINTER(Film)]),
    "pyre_set_stage_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "pyre_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CameraDesc), C.POINTER(RenderParams), C.POINTER(Film)]),
    "pyre_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CameraDesc), C.POINTER(RenderParams), P_f,
                                C.c_int, C.POINTER(Gradients)]),
    "pyre_scene_set_materials": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(MaterialDesc), C.c_uint32]),
    "pyre_scene_set_env": (C.c_int, [C.c_void_p, C.c_void_p, P_f, C.c_float]),
    "pyre_scene_upload_batch": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.c_uint32, C.POINTER(C.c_void_p)]),
    "pyre_render_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(BatchJob), C.c_uint32,
                                    C.POINTER(RenderParams)]),
}


class PyreError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"pyre error {code}: {message}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads the CUDA library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(the CUDA extension is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int, ctx=None) -> None:
    if rc != PYRE_OK:
        msg = load().pyre_last_error(ctx)
        raise PyreError(rc, msg.decode() if msg else "")


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(P_f)


def u32ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(P_u32)


def i32ptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(P_i32)


def dptr(t, ctype=C.c_float):
    """Device pointer of a CUDA torch tensor as a ctypes pointer."""
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ctype))
