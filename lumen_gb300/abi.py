"""ctypes mirror of include/lgb.h and the loader of the in-tree liblgb.so.

The CUDA library is the only implementation of the ray-tracing path: if it has not been built, every
call here raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblgb.so")

LGB_OK = 0
LGB_NO_HIT = 0xFFFFFFFF
STATUS_NAMES = {
    0: "LGB_OK",
    1: "LGB_ERR_INVALID_ARGUMENT",
    2: "LGB_ERR_CUDA",
    3: "LGB_ERR_OUT_OF_MEMORY",
    4: "LGB_ERR_NOT_READY",
    5: "LGB_ERR_DEVICE_STATUS",
    6: "LGB_ERR_UNSUPPORTED",
}

BSDF_DIFFUSE, BSDF_MIRROR, BSDF_GLASS, BSDF_DIELECTRIC, BSDF_CONDUCTOR, BSDF_PRINCIPLED = (1 << i for i in range(6))
FLAG_DIFFUSE, FLAG_SPECULAR, FLAG_GLOSSY, FLAG_REFLECTION, FLAG_TRANSMISSION = (1 << i for i in range(5))
LIGHT_SPOT, LIGHT_AREA, LIGHT_DIRECTIONAL = 1, 2, 3
LIGHT_FINITE, LIGHT_DELTA = 1 << 4, 1 << 5


class Ray(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("ox", "oy", "oz", "tmin", "dx", "dy", "dz", "tmax")]


class Hit(C.Structure):
    _fields_ = [("prim", C.c_uint32), ("t", C.c_float), ("u", C.c_float), ("v", C.c_float)]


class Material(C.Structure):
    _fields_ = [
        ("albedo", C.c_float * 3), ("ior", C.c_float), ("emissive_factor", C.c_float * 3),
        ("bsdf_type", C.c_uint32), ("bsdf_props", C.c_uint32), ("k", C.c_float * 3), ("texture_id", C.c_int32),
        ("roughness", C.c_float), ("diffuse_trans", C.c_float), ("spec_trans", C.c_float), ("metallic", C.c_float),
        ("specular_tint", C.c_float), ("sheen_tint", C.c_float), ("clearcoat", C.c_float),
        ("clearcoat_gloss", C.c_float), ("sheen", C.c_float), ("subsurface", C.c_float), ("flatness", C.c_float),
        ("anisotropy", C.c_float), ("thin", C.c_uint32),
    ]


class Light(C.Structure):
    _fields_ = [
        ("world_matrix", C.c_float * 16), ("pos", C.c_float * 3), ("prim_mesh_idx", C.c_uint32),
        ("to", C.c_float * 3), ("num_triangles", C.c_uint32), ("L", C.c_float * 3), ("light_flags", C.c_uint32),
        ("world_center", C.c_float * 3), ("world_radius", C.c_float),
    ]


class Mesh(C.Structure):
    _fields_ = [("index_offset", C.c_uint32), ("vertex_offset", C.c_uint32), ("material_index", C.c_uint32),
                ("tri_count", C.c_uint32)]


class Texture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba", C.POINTER(C.c_float))]


class SceneDesc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
        ("num_vertices", C.c_uint32), ("indices", C.POINTER(C.c_uint32)), ("num_indices", C.c_uint32),
        ("meshes", C.POINTER(Mesh)), ("num_meshes", C.c_uint32), ("materials", C.POINTER(Material)),
        ("num_materials", C.c_uint32), ("lights", C.POINTER(Light)), ("num_lights", C.c_uint32),
        ("textures", C.POINTER(Texture)), ("num_textures", C.c_uint32),
    ]


class BuildOpts(C.Structure):
    _fields_ = [("leaf_max", C.c_uint32), ("treelet_rounds", C.c_uint32), ("reserved", C.c_uint32 * 6)]


class BuildStats(C.Structure):
    _fields_ = [
        ("build_ms", C.c_float), ("num_tris", C.c_uint32), ("num_nodes", C.c_uint32), ("max_depth", C.c_uint32),
        ("node_bytes", C.c_uint64), ("tri_bytes", C.c_uint64), ("sah_cost", C.c_float), ("reserved", C.c_uint32 * 5),
    ]


class Camera(C.Structure):
    _fields_ = [("inv_view", C.c_float * 16), ("inv_projection", C.c_float * 16), ("width", C.c_uint32),
                ("height", C.c_uint32)]


class PathParams(C.Structure):
    _fields_ = [
        ("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
        ("light_triangle_count", C.c_int32), ("dir_light_idx", C.c_uint32), ("direct_lighting", C.c_uint32),
        ("film_mode", C.c_uint32), ("reserved", C.c_uint32 * 3),
    ]


DIFF_SAMPLE_PARAMS = 1


class DiffParams(C.Structure):
    _fields_ = [("texture_id", C.c_int32), ("flags", C.c_uint32), ("texels", C.c_void_p), ("roughness", C.c_void_p),
                ("emission", C.c_void_p)]


class DiffGrads(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("roughness", C.c_void_p), ("emission", C.c_void_p)]


class BatchJob(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("frame0", C.c_uint32), ("spp", C.c_uint32), ("reserved", C.c_uint32),
                ("camera", Camera), ("params", PathParams), ("d_film", C.c_void_p)]


class BatchOpts(C.Structure):
    _fields_ = [("path_capacity", C.c_uint32), ("work_blocks_per_sm", C.c_uint32),
                ("trace_blocks_per_sm", C.c_uint32), ("stack_placement", C.c_uint32),
                ("from_cache", C.c_uint32), ("chunk_paths", C.c_uint32), ("traversal", C.c_uint32),
                ("reserved", C.c_uint32 * 1)]


STACK_LOCAL, STACK_SHARED = 0, 1  # lgb_batch_opts.stack_placement
TRAVERSAL_AUTO, TRAVERSAL_COHERENT, TRAVERSAL_INCOHERENT = 0, 1, 2  # lgb_batch_opts.traversal
VCM_ACCUMULATE = 1
RESTIR_SPATIAL_COUNT_FIX = 1


class VcmParams(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
                ("light_triangle_count", C.c_int32), ("dir_light_idx", C.c_uint32), ("radius", C.c_float),
                ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3), ("use_vm", C.c_int32),
                ("use_vc", C.c_int32), ("light_seed", C.c_uint32), ("eye_seed", C.c_uint32),
                ("frame_num", C.c_uint32), ("flags", C.c_uint32), ("spot_angle", C.c_float),
                ("reserved", C.c_uint32)]


class VcmState(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("path_counts", C.c_void_p), ("table_count", C.c_void_p),
                ("table_rep", C.c_void_p), ("screen", C.c_uint32), ("per_path", C.c_uint32),
                ("table_size", C.c_uint32), ("grid_res", C.c_int32 * 3), ("radius", C.c_float),
                ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3), ("reserved", C.c_uint32)]


class SppmParams(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
                ("light_triangle_count", C.c_int32), ("dir_light_idx", C.c_uint32), ("base_radius", C.c_float),
                ("seed", C.c_uint32), ("frame_num", C.c_uint32), ("spot_angle", C.c_float),
                ("reserved", C.c_uint32 * 5)]


class BdptParams(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
                ("light_triangle_count", C.c_int32), ("dir_light_idx", C.c_uint32), ("seed", C.c_uint32),
                ("frame_num", C.c_uint32), ("spot_angle", C.c_float), ("reserved", C.c_uint32 * 6)]


class RestirParams(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
                ("light_triangle_count", C.c_int32), ("dir_light_idx", C.c_uint32), ("seed", C.c_uint32),
                ("frame_num", C.c_uint32), ("do_spatiotemporal", C.c_uint32), ("enable_accumulation", C.c_uint32),
                ("spot_angle", C.c_float), ("flags", C.c_uint32), ("reserved", C.c_uint32 * 3)]


# Every exported symbol with its argument and result types (the declarations of include/lgb.h).
SIGNATURES = {
    "lgb_abi_version": ([], C.c_uint32),
    "lgb_create": ([C.POINTER(C.c_void_p), C.c_int, C.c_char_p], C.c_int32),
    "lgb_destroy": ([C.c_void_p], None),
    "lgb_last_error": ([C.c_void_p], C.c_char_p),
    "lgb_scene_create": ([C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_void_p)], C.c_int32),
    "lgb_scene_destroy": ([C.c_void_p], None),
    "lgb_bvh_build": ([C.c_void_p, C.POINTER(BuildOpts), C.POINTER(BuildStats)], C.c_int32),
    "lgb_scene_set_visit_limit": ([C.c_void_p, C.c_uint32], C.c_int32),
    "lgb_trace_closest": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p], C.c_int32),
    "lgb_trace_any": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p], C.c_int32),
    "lgb_trace_closest_counted": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_trace_closest_host": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p], C.c_int32),
    "lgb_trace_any_host": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p], C.c_int32),
    "lgb_camera_lookat": ([C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_uint32, C.c_uint32,
                           C.POINTER(Camera)], C.c_int32),
    "lgb_camera_from_matrix": ([C.POINTER(C.c_float), C.c_float, C.c_uint32, C.c_uint32, C.POINTER(Camera)],
                               C.c_int32),
    "lgb_render_path": ([C.c_void_p, C.POINTER(Camera), C.POINTER(PathParams), C.c_uint32, C.c_uint32, C.c_void_p,
                         C.c_void_p], C.c_int32),
    "lgb_render_path_noalloc": ([C.c_void_p, C.POINTER(Camera), C.POINTER(PathParams), C.c_uint32, C.c_uint32,
                                 C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_diff_render": ([C.c_void_p, C.POINTER(Camera), C.POINTER(PathParams), C.POINTER(DiffParams), C.c_uint32,
                         C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_adjoint_path": ([C.c_void_p, C.POINTER(Camera), C.POINTER(PathParams), C.POINTER(DiffParams), C.c_uint32,
                          C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(DiffGrads), C.c_void_p], C.c_int32),
    "lgb_sync": ([C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_vcm_radius": ([C.c_float, C.c_float, C.c_uint32, C.c_float], C.c_float),
    "lgb_vcm_iteration": ([C.c_void_p, C.POINTER(Camera), C.POINTER(VcmParams), C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_sppm_iteration": ([C.c_void_p, C.POINTER(Camera), C.POINTER(SppmParams), C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_bdpt_iteration": ([C.c_void_p, C.POINTER(Camera), C.POINTER(BdptParams), C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_restir_di_iteration": ([C.c_void_p, C.POINTER(Camera), C.POINTER(Camera), C.POINTER(RestirParams),
                                 C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_vcm_grid": ([C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                      C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_vcm_state_get": ([C.c_void_p, C.POINTER(VcmState)], C.c_int32),
    "lgb_camera_forward": ([C.POINTER(Camera), C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int32),
    "lgb_batch_create": ([C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, C.POINTER(C.c_void_p)], C.c_int32),
    "lgb_batch_destroy": ([C.c_void_p], None),
    "lgb_batch_render": ([C.c_void_p, C.POINTER(BatchJob), C.c_uint32, C.POINTER(BatchOpts), C.c_void_p], C.c_int32),
    "lgb_batch_tune": ([C.c_void_p, C.POINTER(BatchJob), C.c_uint32, C.POINTER(BatchOpts), C.c_void_p], C.c_int32),
    "lgb_batch_sync": ([C.c_void_p, C.c_void_p], C.c_int32),
    "lgb_film_rmse": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_double), C.c_void_p],
                      C.c_int32),
    "lgb_measure_l2_read_gbs": ([C.c_int, C.c_uint64, C.c_uint32, C.POINTER(C.c_double)], C.c_int32),
}

_lib = None


def load() -> C.CDLL:
    """Loads liblgb.so (built in-tree by __graft_entry__.build()); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"liblgb.so is not built ({LIB_PATH}); run __graft_entry__.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


class LgbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
