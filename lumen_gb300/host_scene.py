"""ctypes face of liblgb_host.so (include/lgb_host.h): Lumen JSON/OBJ scene loading and headless rendering."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .scene import LIGHT_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, SceneArrays

HOST_LIB = os.path.join(os.path.dirname(abi.LIB_PATH), "liblgb_host.so")


class SceneInfo(C.Structure):
    _fields_ = [("cam_pos", C.c_float * 3), ("cam_dir", C.c_float * 3), ("fov", C.c_float),
                ("path_length", C.c_int32), ("sky_col", C.c_float * 3), ("light_triangle_count", C.c_uint32),
                ("dir_light_idx", C.c_uint32), ("total_light_area", C.c_float), ("bbox_min", C.c_float * 3),
                ("bbox_max", C.c_float * 3), ("radius", C.c_float), ("base_radius", C.c_float),
                ("radius_factor", C.c_float), ("enable_vm", C.c_int32), ("cam_use_matrix", C.c_int32),
                ("cam_matrix", C.c_float * 16)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError(f"liblgb_host.so is not built ({HOST_LIB}); run __graft_entry__.build()")
        lib = C.CDLL(HOST_LIB)
        lib.lgbh_scene_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        lib.lgbh_scene_load.restype = C.c_int32
        lib.lgbh_scene_free.argtypes = [C.c_void_p]
        lib.lgbh_scene_desc.argtypes = [C.c_void_p, C.POINTER(abi.SceneDesc)]
        lib.lgbh_scene_desc.restype = C.c_int32
        lib.lgbh_scene_get_info.argtypes = [C.c_void_p, C.POINTER(SceneInfo)]
        lib.lgbh_scene_get_info.restype = C.c_int32
        lib.lgbh_render_path.argtypes = [C.c_char_p, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_char_p,
                                         C.c_void_p, C.c_char_p, C.c_size_t]
        lib.lgbh_render_path.restype = C.c_int32
        lib.lgbh_write_image.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_char_p, C.c_size_t]
        lib.lgbh_write_image.restype = C.c_int32
        _lib = lib
    return _lib


def load_scene(json_path: str):
    """Loads a Lumen JSON scene (or a Mitsuba XML scene, by extension) with the C++ loader; returns
    (SceneArrays, SceneInfo)."""
    lib = load()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    st = lib.lgbh_scene_load(json_path.encode(), C.byref(h), err, 512)
    if st != abi.LGB_OK:
        raise abi.LgbError(st, err.value.decode())
    try:
        d = abi.SceneDesc()
        lib.lgbh_scene_desc(h, C.byref(d))
        info = SceneInfo()
        lib.lgbh_scene_get_info(h, C.byref(info))

        def arr(ptr, count, dtype):
            if count == 0:
                return np.zeros(0, dtype)
            buf = C.cast(ptr, C.POINTER(C.c_uint8 * (count * np.dtype(dtype).itemsize))).contents
            return np.frombuffer(bytes(buf), dtype=dtype).copy()

        nv = d.num_vertices
        arrays = SceneArrays(
            positions=arr(d.positions, 3 * nv, np.float32).reshape(-1, 3),
            normals=arr(d.normals, 3 * nv, np.float32).reshape(-1, 3),
            uvs=arr(d.uvs, 2 * nv, np.float32).reshape(-1, 2),
            indices=arr(d.indices, d.num_indices, np.uint32),
            meshes=arr(d.meshes, d.num_meshes, MESH_DTYPE),
            materials=arr(d.materials, d.num_materials, MATERIAL_DTYPE),
            lights=arr(d.lights, d.num_lights, LIGHT_DTYPE),
            light_triangle_count=int(info.light_triangle_count),
            camera_pos=tuple(info.cam_pos), camera_dir=tuple(info.cam_dir), fov=float(info.fov),
        )
        return arrays, info
    finally:
        lib.lgbh_scene_free(h)


def write_image(path: str, film: np.ndarray, width: int, height: int):
    """lgbh_write_image: an (H*W, 4) float32 film as OpenEXR (path ending in .exr) or PFM."""
    lib = load()
    film = np.ascontiguousarray(film, np.float32)
    assert film.size == width * height * 4
    err = C.create_string_buffer(512)
    st = lib.lgbh_write_image(path.encode(), film.ctypes.data, width, height, err, 512)
    if st != abi.LGB_OK:
        raise abi.LgbError(st, err.value.decode())


def render_path(json_path: str, width: int, height: int, spp: int, out_pfm: str | None = None, device: int = 0):
    """Headless render through the C++ Integrator mirror; returns the RGBA32F film as an (H*W, 4) array. The scene is
    a Lumen JSON or a Mitsuba XML file."""
    lib = load()
    film = np.zeros((width * height, 4), np.float32)
    err = C.create_string_buffer(512)
    st = lib.lgbh_render_path(json_path.encode(), device, width, height, spp,
                              out_pfm.encode() if out_pfm else None, film.ctypes.data, err, 512)
    if st != abi.LGB_OK:
        raise abi.LgbError(st, err.value.decode())
    return film
