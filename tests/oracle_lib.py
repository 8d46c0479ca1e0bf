"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so) for the test suite.

Test infrastructure only: the oracle is the checker the CUDA path is compared against.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])


class _Mesh(C.Structure):
    _fields_ = [("index_offset", C.c_uint32), ("vertex_offset", C.c_uint32), ("material_index", C.c_uint32),
                ("tri_count", C.c_uint32)]


class _Tex(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba", C.POINTER(C.c_float))]


class _Desc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
        ("num_vertices", C.c_uint32), ("indices", C.POINTER(C.c_uint32)), ("num_indices", C.c_uint32),
        ("meshes", C.POINTER(_Mesh)), ("num_meshes", C.c_uint32), ("materials", C.c_void_p),
        ("num_materials", C.c_uint32), ("lights", C.c_void_p), ("num_lights", C.c_uint32),
        ("textures", C.POINTER(_Tex)), ("num_textures", C.c_uint32),
    ]


class _Params(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("frame_num", C.c_uint32), ("size_x", C.c_uint32),
                ("size_y", C.c_uint32), ("num_lights", C.c_int32), ("max_depth", C.c_int32),
                ("light_triangle_count", C.c_int32), ("dir_light_idx", C.c_uint32), ("direct_lighting", C.c_uint32)]


class VcmParams(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
                ("light_triangle_count", C.c_int32), ("radius", C.c_float), ("use_vm", C.c_int32),
                ("use_vc", C.c_int32), ("light_seed", C.c_uint32), ("eye_seed", C.c_uint32),
                ("frame_num", C.c_uint32), ("scene_min", C.c_float * 3), ("scene_max", C.c_float * 3),
                ("flags", C.c_uint32), ("spot_angle", C.c_float)]


class SppmParams(C.Structure):
    _fields_ = [("sky_col", C.c_float * 3), ("max_depth", C.c_int32), ("num_lights", C.c_int32),
                ("light_triangle_count", C.c_int32), ("base_radius", C.c_float), ("seed", C.c_uint32),
                ("frame_num", C.c_uint32), ("spot_angle", C.c_float)]


class RestirParams(C.Structure):
    _fields_ = [("num_lights", C.c_int32), ("light_triangle_count", C.c_int32), ("seed", C.c_uint32),
                ("frame_num", C.c_uint32), ("do_spatiotemporal", C.c_uint32), ("enable_accumulation", C.c_uint32),
                ("spot_angle", C.c_float), ("flags", C.c_uint32)]


class BdptParams(C.Structure):
    _fields_ = [("max_depth", C.c_int32), ("num_lights", C.c_int32), ("light_triangle_count", C.c_int32),
                ("seed", C.c_uint32), ("frame_num", C.c_uint32), ("spot_angle", C.c_float),
                ("check_flags", C.c_uint32), ("check_len", C.c_int32), ("check_s", C.c_int32)]


VCM_VERTEX_BYTES = 104


def ensure_built() -> str:
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return LIB


def _p(a, ct=C.c_float):
    return a.ctypes.data_as(C.POINTER(ct))


class Oracle:
    def __init__(self):
        self.lib = C.CDLL(ensure_built())
        L = self.lib
        L.orc_bvh_build.restype = C.c_void_p
        L.orc_bvh_build.argtypes = [C.POINTER(C.c_float), C.c_uint32]
        L.orc_bvh_free.argtypes = [C.c_void_p]
        L.orc_bvh_num_nodes.restype = C.c_uint32
        L.orc_bvh_num_nodes.argtypes = [C.c_void_p]
        L.orc_trace_closest.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int]
        L.orc_trace_any.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int]
        L.orc_brute_closest.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32]
        L.orc_brute_any.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32]
        L.orc_intersect_tri.restype = C.c_int
        L.orc_intersect_tri.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_camera_matrices.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_uint32,
                                          C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_scene_create.restype = C.c_void_p
        L.orc_scene_create.argtypes = [C.POINTER(_Desc)]
        L.orc_scene_free.argtypes = [C.c_void_p]
        L.orc_render_samples.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(_Params),
                                         C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_float),
                                         C.POINTER(C.c_uint8), C.c_int, C.c_int]
        L.orc_render_film.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(_Params),
                                      C.c_uint32, C.c_uint32, C.POINTER(C.c_float), C.c_int, C.c_int]
        L.orc_render_diff.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(_Params),
                                      C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                      C.POINTER(C.c_double), C.c_int, C.c_int]
        L.orc_vcm_grid_res.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_int32)]
        L.orc_vcm_grid.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.c_float, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_vcm_iteration.argtypes = [C.c_void_p] + [C.POINTER(C.c_float)] * 4 + [
            C.c_uint32, C.c_uint32, C.POINTER(VcmParams), C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_float),
            C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_float), C.c_int]
        L.orc_render_mean_f64.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_void_p,
                                          C.c_uint32, C.c_uint32, C.POINTER(C.c_double), C.c_int]
        L.orc_vcm_render_f64.argtypes = [C.c_void_p] + [C.POINTER(C.c_float)] * 4 + [
            C.c_uint32, C.c_uint32, C.POINTER(VcmParams), C.c_uint32, C.POINTER(C.c_double), C.c_int]
        L.orc_sppm_iteration.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32,
                                         C.c_uint32, C.POINTER(SppmParams), C.POINTER(C.c_float),
                                         C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                         C.POINTER(C.c_float), C.c_int]
        L.orc_restir_di_iteration.argtypes = [C.c_void_p] + [C.POINTER(C.c_float)] * 4 + [
            C.c_uint32, C.c_uint32, C.POINTER(RestirParams)] + [C.POINTER(C.c_float)] * 5 + [C.c_int]
        L.orc_bdpt_iteration.argtypes = [C.c_void_p] + [C.POINTER(C.c_float)] * 4 + [
            C.c_uint32, C.c_uint32, C.POINTER(BdptParams)] + [C.POINTER(C.c_float)] * 2 + [C.c_int]
        L.orc_pcg4d.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32]
        L.orc_offset_ray.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32]

    def bvh(self, tri_verts: np.ndarray) -> "OracleBvh":
        return OracleBvh(self, tri_verts)

    def scene(self, arrays) -> "OracleScene":
        return OracleScene(self, arrays)

    def camera(self, pos, direction, fov, width, height):
        iv = np.zeros(16, np.float32)
        ip = np.zeros(16, np.float32)
        p = np.asarray(pos, np.float32)
        d = np.asarray(direction, np.float32)
        self.lib.orc_camera_matrices(_p(p), _p(d), float(fov), width, height, _p(iv), _p(ip))
        return iv, ip

    def pcg4d(self, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, np.uint32)
        out = np.zeros_like(v)
        self.lib.orc_pcg4d(_p(v, C.c_uint32), _p(out, C.c_uint32), len(v))
        return out

    def offset_ray(self, p, n):
        p = np.ascontiguousarray(p, np.float32)
        n = np.ascontiguousarray(n, np.float32)
        out = np.zeros_like(p)
        self.lib.orc_offset_ray(_p(p), _p(n), _p(out), len(p))
        return out

    def brute_closest(self, tri_verts, rays):
        tv = np.ascontiguousarray(tri_verts, np.float32)
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.zeros(len(rays), HIT_DTYPE)
        self.lib.orc_brute_closest(_p(tv), len(tv), rays.ctypes.data, hits.ctypes.data, len(rays))
        return hits

    def brute_any(self, tri_verts, rays):
        tv = np.ascontiguousarray(tri_verts, np.float32)
        rays = np.ascontiguousarray(rays, np.float32)
        occ = np.zeros(len(rays), np.uint8)
        self.lib.orc_brute_any(_p(tv), len(tv), rays.ctypes.data, occ.ctypes.data, len(rays))
        return occ


class OracleBvh:
    def __init__(self, ora: Oracle, tri_verts: np.ndarray):
        self.ora = ora
        self.tv = np.ascontiguousarray(tri_verts, np.float32)
        self.h = ora.lib.orc_bvh_build(_p(self.tv), len(self.tv))

    def __del__(self):
        try:
            self.ora.lib.orc_bvh_free(self.h)
        except Exception:
            pass

    def closest(self, rays: np.ndarray, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.zeros(len(rays), HIT_DTYPE)
        self.ora.lib.orc_trace_closest(self.h, rays.ctypes.data, hits.ctypes.data, len(rays),
                                       threads or (os.cpu_count() or 1))
        return hits

    def any(self, rays: np.ndarray, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        occ = np.zeros(len(rays), np.uint8)
        self.ora.lib.orc_trace_any(self.h, rays.ctypes.data, occ.ctypes.data, len(rays),
                                   threads or (os.cpu_count() or 1))
        return occ


class OracleScene:
    def __init__(self, ora: Oracle, arrays):
        self.ora = ora
        keep = []

        def arr(a, dt=None):
            a = np.ascontiguousarray(a if dt is None else a.astype(dt))
            keep.append(a)
            return a

        d = _Desc()
        d.positions = _p(arr(arrays.positions, np.float32))
        d.normals = _p(arr(arrays.normals, np.float32))
        d.uvs = _p(arr(arrays.uvs, np.float32))
        d.num_vertices = len(arrays.positions)
        d.indices = _p(arr(arrays.indices, np.uint32), C.c_uint32)
        d.num_indices = len(arrays.indices)
        meshes = arr(arrays.meshes)
        d.meshes = C.cast(meshes.ctypes.data, C.POINTER(_Mesh))
        d.num_meshes = len(meshes)
        mats = arr(arrays.materials)
        d.materials = mats.ctypes.data
        d.num_materials = len(mats)
        lights = arr(arrays.lights)
        d.lights = lights.ctypes.data if len(lights) else None
        d.num_lights = len(lights)
        if arrays.textures:
            tex = (_Tex * len(arrays.textures))()
            for i, t in enumerate(arrays.textures):
                t = arr(t, np.float32)
                tex[i].width = t.shape[1]
                tex[i].height = t.shape[0]
                tex[i].rgba = _p(t)
            keep.append(tex)
            d.textures = C.cast(tex, C.POINTER(_Tex))
        d.num_textures = len(arrays.textures)
        self.keep = keep
        self.arrays = arrays
        self.h = ora.lib.orc_scene_create(C.byref(d))

    def __del__(self):
        try:
            self.ora.lib.orc_scene_free(self.h)
        except Exception:
            pass

    def _params(self, max_depth, width, height, frame, sky=(0.0, 0.0, 0.0), direct_lighting=1):
        p = _Params()
        p.sky_col[:] = list(sky)
        p.frame_num = frame
        p.size_x, p.size_y = width, height
        p.num_lights = len(self.arrays.lights)
        p.max_depth = max_depth
        p.light_triangle_count = self.arrays.light_triangle_count
        p.dir_light_idx = 0xFFFFFFFF
        p.direct_lighting = direct_lighting
        return p

    def samples(self, cam, max_depth, width, height, frame, pixels=None, fp64=False, threads=0):
        """Per-sample radiance of frame `frame` for the listed pixels (all by default): (N, 3), nan flags."""
        iv = np.ascontiguousarray(np.array(cam.inv_view[:], np.float32))
        ip = np.ascontiguousarray(np.array(cam.inv_projection[:], np.float32))
        if pixels is None:
            pixels = np.arange(width * height, dtype=np.uint32)
        pixels = np.ascontiguousarray(pixels, np.uint32)
        out = np.zeros((len(pixels), 3), np.float32)
        nan = np.zeros(len(pixels), np.uint8)
        p = self._params(max_depth, width, height, frame)
        self.ora.lib.orc_render_samples(self.h, _p(iv), _p(ip), C.byref(p), _p(pixels, C.c_uint32), len(pixels),
                                        _p(out), _p(nan, C.c_uint8), int(fp64), threads or (os.cpu_count() or 1))
        return out, nan

    def film(self, cam, max_depth, width, height, frame0, spp, film=None, fp64=False, threads=0):
        iv = np.ascontiguousarray(np.array(cam.inv_view[:], np.float32))
        ip = np.ascontiguousarray(np.array(cam.inv_projection[:], np.float32))
        if film is None:
            film = np.zeros((width * height, 4), np.float32)
        p = self._params(max_depth, width, height, frame0)
        self.ora.lib.orc_render_film(self.h, _p(iv), _p(ip), C.byref(p), frame0, spp, _p(film), int(fp64),
                                     threads or (os.cpu_count() or 1))
        return film

    def mean_f64(self, cam, max_depth, width, height, frame0, spp, threads=0):
        """Plain FP64 mean (npix, 3) of the path samples of frames [frame0, frame0 + spp), NaN samples skipped."""
        iv = np.ascontiguousarray(np.array(cam.inv_view[:], np.float32))
        ip = np.ascontiguousarray(np.array(cam.inv_projection[:], np.float32))
        out = np.zeros((width * height, 3), np.float64)
        p = self._params(max_depth, width, height, frame0)
        self.ora.lib.orc_render_mean_f64(self.h, _p(iv), _p(ip), C.byref(p), frame0, spp,
                                         out.ctypes.data_as(C.POINTER(C.c_double)), threads or (os.cpu_count() or 1))
        return out

    def diff(self, cam, max_depth, width, height, frame0, spp, tex_id=-1, texels=None, rough=None, emis=None,
             fp64=True, threads=0):
        """Mean image (npix, 3) float64 of the detached differentiable estimator over frames [frame0, frame0+spp).
        texels (H, W, 4) replace texture tex_id, rough (per material) and emis (per material, RGB) replace the
        scene values in every BSDF value and emission, while sampling keeps the scene's materials."""
        iv = np.ascontiguousarray(np.array(cam.inv_view[:], np.float32))
        ip = np.ascontiguousarray(np.array(cam.inv_projection[:], np.float32))
        out = np.zeros((width * height, 3), np.float64)
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, np.float32)
            keep.append(a)
            return a.ctypes.data

        p = self._params(max_depth, width, height, frame0)
        self.ora.lib.orc_render_diff(self.h, _p(iv), _p(ip), C.byref(p), int(tex_id), ptr(texels), ptr(rough),
                                     ptr(emis), frame0, spp, _p(out, C.c_double), int(fp64),
                                     threads or (os.cpu_count() or 1))
        return out

    def vcm_state(self, width, height, max_depth):
        """Buffers that persist across VCM iterations (as the reference's do), zero-initialised."""
        screen = width * height
        return {"verts": np.zeros(screen * (max_depth + 1) * VCM_VERTEX_BYTES, np.uint8),
                "counts": np.zeros(screen, np.uint32), "splat": np.zeros(screen * 3, np.float32),
                "grid_count": np.zeros(10 * screen, np.uint32), "grid_rep": np.zeros(10 * screen, np.uint32),
                "film": np.zeros((screen, 4), np.float32), "width": width, "height": height}

    def vcm_iteration(self, cam, view, proj, params: "VcmParams", state, threads=0):
        """One VCM iteration into state['film'] (RGBA32F, row-major); view / proj are the camera's forward
        matrices (column-major 4x4 float32)."""
        f32 = lambda a: np.ascontiguousarray(np.array(a, np.float32).reshape(16))
        iv, ip, vw, pj = f32(cam.inv_view[:]), f32(cam.inv_projection[:]), f32(view), f32(proj)
        self.ora.lib.orc_vcm_iteration(self.h, _p(iv), _p(ip), _p(vw), _p(pj), state["width"], state["height"],
                                       C.byref(params), state["verts"].ctypes.data, _p(state["counts"], C.c_uint32),
                                       _p(state["splat"]), _p(state["grid_count"], C.c_uint32),
                                       _p(state["grid_rep"], C.c_uint32), _p(state["film"]),
                                       threads or (os.cpu_count() or 1))
        return state["film"]

    def vcm_render_f64(self, cam, view, proj, params_list, threads=0):
        """len(params_list) VCM iterations in FP64 (converged reference renders); returns the progressive film as
        (W*H, 4) float64."""
        f32 = lambda a: np.ascontiguousarray(np.array(a, np.float32).reshape(16))
        iv, ip, vw, pj = f32(cam.inv_view[:]), f32(cam.inv_projection[:]), f32(view), f32(proj)
        arr = (VcmParams * len(params_list))(*params_list)
        film = np.zeros((cam.width * cam.height, 4), np.float64)
        self.ora.lib.orc_vcm_render_f64(self.h, _p(iv), _p(ip), _p(vw), _p(pj), cam.width, cam.height, arr,
                                        len(params_list), film.ctypes.data_as(C.POINTER(C.c_double)),
                                        threads or (os.cpu_count() or 1))
        return film


def sppm_state(width, height, max_depth):
    """Buffers that persist across SPPM frames, zero-initialised (the reference clears them at frame 0)."""
    screen = width * height
    return {"vp": np.zeros(screen * 32, np.float32), "photons": np.zeros(screen * max_depth * 16, np.float32),
            "grid_count": np.zeros(10 * screen, np.uint32), "grid_rep": np.zeros(10 * screen, np.uint32),
            "film": np.zeros((screen, 4), np.float32), "width": width, "height": height}


def sppm_iteration(scene: "OracleScene", cam, params: SppmParams, state, threads=0):
    """One SPPM frame of the oracle into state['film']."""
    f32 = lambda a: np.ascontiguousarray(np.array(a, np.float32).reshape(16))
    iv, ip = f32(cam.inv_view[:]), f32(cam.inv_projection[:])
    scene.ora.lib.orc_sppm_iteration(scene.h, _p(iv), _p(ip), state["width"], state["height"], C.byref(params),
                                     _p(state["vp"]), _p(state["photons"]), _p(state["grid_count"], C.c_uint32),
                                     _p(state["grid_rep"], C.c_uint32), _p(state["film"]),
                                     threads or (os.cpu_count() or 1))
    return state["film"]


def restir_state(width, height):
    """G-buffer, reservoirs and film that persist across ReSTIR frames, zero-initialised."""
    screen = width * height
    return {"gbuf": np.zeros(screen * 12, np.float32), "pass": np.zeros(screen * 12, np.float32),
            "temporal": np.zeros(screen * 12, np.float32), "spatial": np.zeros(screen * 12, np.float32),
            "film": np.zeros((screen, 4), np.float32), "width": width, "height": height}


def restir_iteration(scene: "OracleScene", cam, prev_view, prev_proj, params: RestirParams, state, threads=0):
    """One ReSTIR DI frame of the oracle into state['film']."""
    f32 = lambda a: np.ascontiguousarray(np.array(a, np.float32).reshape(16))
    iv, ip, pv, pp = f32(cam.inv_view[:]), f32(cam.inv_projection[:]), f32(prev_view), f32(prev_proj)
    scene.ora.lib.orc_restir_di_iteration(scene.h, _p(iv), _p(ip), _p(pv), _p(pp), state["width"], state["height"],
                                          C.byref(params), _p(state["gbuf"]), _p(state["pass"]),
                                          _p(state["temporal"]), _p(state["spatial"]), _p(state["film"]),
                                          threads or (os.cpu_count() or 1))
    return state["film"]


def bdpt_state(width, height):
    """The progressive film (persists across BDPT frames) and the last frame's splat image, row-major."""
    screen = width * height
    return {"film": np.zeros((screen, 4), np.float32), "splat": np.zeros(screen * 3, np.float32),
            "width": width, "height": height}


def bdpt_iteration(scene: "OracleScene", cam, view, proj, params: BdptParams, state, threads=0):
    """One BDPT frame of the oracle into state['film']; view / proj are the camera's forward matrices."""
    f32 = lambda a: np.ascontiguousarray(np.array(a, np.float32).reshape(16))
    iv, ip, vw, pj = f32(cam.inv_view[:]), f32(cam.inv_projection[:]), f32(view), f32(proj)
    scene.ora.lib.orc_bdpt_iteration(scene.h, _p(iv), _p(ip), _p(vw), _p(pj), state["width"], state["height"],
                                     C.byref(params), _p(state["film"]), _p(state["splat"]),
                                     threads or (os.cpu_count() or 1))
    return state["film"]


def vcm_grid(ora: Oracle, pos4, scene_min, scene_max, radius, screen_size):
    """The sequential photon table: (count, representative) per slot, 10 * screen_size slots."""
    pos4 = np.ascontiguousarray(pos4, np.float32)
    count = np.zeros(10 * screen_size, np.uint32)
    rep = np.zeros(10 * screen_size, np.uint32)
    mn = np.ascontiguousarray(scene_min, np.float32)
    mx = np.ascontiguousarray(scene_max, np.float32)
    ora.lib.orc_vcm_grid(_p(pos4), len(pos4), _p(mn), _p(mx), radius, screen_size, _p(count, C.c_uint32),
                         _p(rep, C.c_uint32))
    return count, rep
