"""Host-side scene arrays and the Python face of the C ABI.

`SceneArrays` holds what Lumen's LumenScene::load_scene produces (src/RayTracer/LumenScene.cpp:52-229):
flattened vertex/index buffers, per-mesh records, materials, lights. `Context`/`GpuScene` wrap the
lgb_* entry points for callers working with torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

MATERIAL_DTYPE = np.dtype([
    ("albedo", "<f4", 3), ("ior", "<f4"), ("emissive_factor", "<f4", 3), ("bsdf_type", "<u4"),
    ("bsdf_props", "<u4"), ("k", "<f4", 3), ("texture_id", "<i4"), ("roughness", "<f4"), ("diffuse_trans", "<f4"),
    ("spec_trans", "<f4"), ("metallic", "<f4"), ("specular_tint", "<f4"), ("sheen_tint", "<f4"),
    ("clearcoat", "<f4"), ("clearcoat_gloss", "<f4"), ("sheen", "<f4"), ("subsurface", "<f4"), ("flatness", "<f4"),
    ("anisotropy", "<f4"), ("thin", "<u4"),
])
LIGHT_DTYPE = np.dtype([
    ("world_matrix", "<f4", 16), ("pos", "<f4", 3), ("prim_mesh_idx", "<u4"), ("to", "<f4", 3),
    ("num_triangles", "<u4"), ("L", "<f4", 3), ("light_flags", "<u4"), ("world_center", "<f4", 3),
    ("world_radius", "<f4"),
])
MESH_DTYPE = np.dtype([("index_offset", "<u4"), ("vertex_offset", "<u4"), ("material_index", "<u4"),
                       ("tri_count", "<u4")])
assert MATERIAL_DTYPE.itemsize == 104 and LIGHT_DTYPE.itemsize == 128 and MESH_DTYPE.itemsize == 16


def new_material(**kw) -> np.ndarray:
    """A material record with Lumen's loader defaults (albedo 1, texture -1, clearcoat_gloss 1)."""
    m = np.zeros(1, MATERIAL_DTYPE)
    m["albedo"] = 1.0
    m["texture_id"] = -1
    m["clearcoat_gloss"] = 1.0
    m["sheen_tint"] = 0.5
    for k, v in kw.items():
        m[k] = v
    return m


def diffuse(albedo, emissive=(0.0, 0.0, 0.0)) -> np.ndarray:
    """"type": "diffuse" as LumenScene.cpp:372-375 maps it."""
    return new_material(albedo=albedo, emissive_factor=emissive, bsdf_type=abi.BSDF_DIFFUSE,
                        bsdf_props=abi.FLAG_DIFFUSE | abi.FLAG_REFLECTION)


def conductor(reflectance, roughness) -> np.ndarray:
    """"type": "conductor" with "reflectance" (LumenScene.cpp:406-443, reflectance_to_conductor_eta_k :47-50)."""
    r = np.clip(np.asarray(reflectance, np.float32), 0.0, 0.9999).astype(np.float32)
    eta = np.ones(3, np.float32)
    k = (np.float32(2.0) * np.sqrt(r) / np.sqrt(np.maximum(np.float32(1.0) - r, np.float32(0.001)))).astype(np.float32)
    props = abi.FLAG_REFLECTION | (abi.FLAG_GLOSSY if roughness > 0.08 else abi.FLAG_SPECULAR)
    return new_material(albedo=eta, k=k, roughness=roughness, bsdf_type=abi.BSDF_CONDUCTOR, bsdf_props=props)


def dielectric(ior, roughness=0.0, albedo=(1.0, 1.0, 1.0), thin=0) -> np.ndarray:
    """"type": "dielectric" (LumenScene.cpp:385-405)."""
    props = abi.FLAG_TRANSMISSION | abi.FLAG_REFLECTION
    props |= abi.FLAG_GLOSSY if (ior != 1.0 and roughness > 0.08) else abi.FLAG_SPECULAR
    return new_material(albedo=albedo, ior=ior, roughness=roughness, bsdf_type=abi.BSDF_DIELECTRIC, bsdf_props=props,
                        thin=thin)


def glass(ior) -> np.ndarray:
    """"type": "glass" (LumenScene.cpp:380-384): smooth specular transmission only, no reflection lobe."""
    return new_material(ior=ior, bsdf_type=abi.BSDF_GLASS, bsdf_props=abi.FLAG_SPECULAR | abi.FLAG_TRANSMISSION)


def principled(albedo, roughness=0.5, metallic=0.0, ior=1.0, spec_trans=0.0, clearcoat=0.0, clearcoat_gloss=1.0,
               specular_tint=0.0, anisotropy=0.0, flatness=0.0) -> np.ndarray:
    """"type": "principled" (LumenScene.cpp:444-475)."""
    props = 0
    if roughness < 1.0:
        props |= abi.FLAG_REFLECTION
    if spec_trans > 0.0:
        props |= abi.FLAG_TRANSMISSION
    props |= abi.FLAG_GLOSSY if roughness > 0.08 else abi.FLAG_SPECULAR
    return new_material(albedo=albedo, roughness=roughness, metallic=metallic, ior=ior, spec_trans=spec_trans,
                        clearcoat=clearcoat, clearcoat_gloss=clearcoat_gloss, specular_tint=specular_tint,
                        anisotropy=anisotropy, flatness=flatness, bsdf_type=abi.BSDF_PRINCIPLED, bsdf_props=props)


@dataclass
class SceneArrays:
    positions: np.ndarray            # (V, 3) f32
    normals: np.ndarray              # (V, 3) f32
    uvs: np.ndarray                  # (V, 2) f32
    indices: np.ndarray              # (I,) u32
    meshes: np.ndarray               # MESH_DTYPE
    materials: np.ndarray            # MATERIAL_DTYPE
    lights: np.ndarray               # LIGHT_DTYPE
    textures: list = field(default_factory=list)  # list of (H, W, 4) f32
    light_triangle_count: int = 0
    camera_pos: tuple = (0.0, 0.0, 0.0)
    camera_dir: tuple = (0.0, 0.0, 1.0)
    fov: float = 45.0

    @property
    def num_tris(self) -> int:
        return int(self.meshes["tri_count"].sum())

    def bounds(self):
        """(min, max) of the vertex positions as float32 arrays, computed once per positions array (a reduction
        over every vertex takes milliseconds on the host, longer than a frame's kernels; assign a new positions
        array rather than editing it in place to change the geometry)."""
        key = (id(self.positions), self.positions.shape)
        cached = self.__dict__.get("_bounds")
        if cached is None or cached[0] != key:
            cached = (key, self.positions.min(0), self.positions.max(0))
            self.__dict__["_bounds"] = cached
        return cached[1], cached[2]

    def tri_verts(self) -> np.ndarray:
        """(T, 9) world-space vertices of every global triangle, meshes in order."""
        out = []
        for m in self.meshes:
            n = int(m["tri_count"])
            idx = self.indices[int(m["index_offset"]):int(m["index_offset"]) + 3 * n].astype(np.int64)
            idx = idx + int(m["vertex_offset"])
            out.append(self.positions[idx].reshape(n, 9))
        return np.ascontiguousarray(np.concatenate(out).astype(np.float32))

    def make_desc(self, desc_cls=abi.SceneDesc, mesh_cls=abi.Mesh, mat_cls=abi.Material, light_cls=abi.Light,
                  tex_cls=abi.Texture):
        """Builds a ctypes scene description; returns (desc, keepalive)."""
        keep = []

        def ptr(a, ct):
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ct))

        d = desc_cls()
        d.positions = ptr(self.positions.astype(np.float32), C.c_float)
        d.normals = ptr(self.normals.astype(np.float32), C.c_float)
        d.uvs = ptr(self.uvs.astype(np.float32), C.c_float)
        d.num_vertices = len(self.positions)
        d.indices = ptr(self.indices.astype(np.uint32), C.c_uint32)
        d.num_indices = len(self.indices)
        d.meshes = ptr(self.meshes, mesh_cls)
        d.num_meshes = len(self.meshes)
        d.materials = ptr(self.materials, mat_cls)
        d.num_materials = len(self.materials)
        d.lights = ptr(self.lights, light_cls) if len(self.lights) else None
        d.num_lights = len(self.lights)
        if self.textures:
            arr = (tex_cls * len(self.textures))()
            for i, t in enumerate(self.textures):
                t = np.ascontiguousarray(t, np.float32)
                keep.append(t)
                arr[i].width = t.shape[1]
                arr[i].height = t.shape[0]
                arr[i].rgba = t.ctypes.data_as(C.POINTER(C.c_float))
            keep.append(arr)
            d.textures = C.cast(arr, C.POINTER(tex_cls))
        d.num_textures = len(self.textures)
        keep.append(d)
        return d, keep


def _check(lib, ctx, st):
    if st != abi.LGB_OK:
        msg = lib.lgb_last_error(ctx)
        raise abi.LgbError(st, msg.decode() if msg else "")


def camera_lookat(pos, direction, fov, width, height) -> abi.Camera:
    lib = abi.load()
    cam = abi.Camera()
    p = (C.c_float * 3)(*pos)
    d = (C.c_float * 3)(*direction)
    st = lib.lgb_camera_lookat(p, d, float(fov), int(width), int(height), C.byref(cam))
    if st != abi.LGB_OK:
        raise abi.LgbError(st, "lgb_camera_lookat")
    return cam


def camera_from_matrix(camera_to_world, fov, width, height) -> abi.Camera:
    """lgb_camera_from_matrix: camera_to_world is 16 floats, column-major (as lgbh_scene_info.cam_matrix)."""
    lib = abi.load()
    cam = abi.Camera()
    m = (C.c_float * 16)(*[float(x) for x in camera_to_world])
    st = lib.lgb_camera_from_matrix(m, float(fov), int(width), int(height), C.byref(cam))
    if st != abi.LGB_OK:
        raise abi.LgbError(st, "lgb_camera_from_matrix")
    return cam


class Context:
    """An lgb_ctx on one CUDA device (the counterpart of Lumen's Vulkan context)."""

    def __init__(self, device: int = 0, tuning_cache: str | None = None):
        self.lib = abi.load()
        h = C.c_void_p()
        st = self.lib.lgb_create(C.byref(h), device, tuning_cache.encode() if tuning_cache else None)
        if st != abi.LGB_OK:
            raise abi.LgbError(st, f"lgb_create(device={device})")
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.lgb_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def camera_forward(cam: abi.Camera):
    """lgb_camera_forward: (view, projection) as two 16-float column-major numpy arrays."""
    lib = abi.load()
    view, proj = (C.c_float * 16)(), (C.c_float * 16)()
    st = lib.lgb_camera_forward(C.byref(cam), view, proj)
    if st != abi.LGB_OK:
        raise abi.LgbError(st, "lgb_camera_forward")
    return np.array(view[:], np.float32), np.array(proj[:], np.float32)


def vcm_radius(scene_radius: float, radius_factor: float, iteration: int, alpha: float = 2.0 / 3.0) -> float:
    return float(abi.load().lgb_vcm_radius(scene_radius, radius_factor, iteration, alpha))


def vcm_grid(ctx: Context, pos4, scene_min, scene_max, radius: float, screen_size: int, count, rep, stream=None):
    """lgb_vcm_grid on CUDA tensors: pos4 (n, 4) float32; count / rep (10 * screen_size,) int32."""
    mn = (C.c_float * 3)(*[float(v) for v in scene_min])
    mx = (C.c_float * 3)(*[float(v) for v in scene_max])
    _check(ctx.lib, ctx.handle,
           ctx.lib.lgb_vcm_grid(ctx.handle, C.c_void_p(pos4.data_ptr()), pos4.shape[0], mn, mx, radius, screen_size,
                                C.c_void_p(count.data_ptr()), C.c_void_p(rep.data_ptr()), C.c_void_p(stream)))


def film_rmse(ctx: Context, film, reference, mode: int = 0, stream=None) -> float:
    """lgb_film_rmse on two (N, 4) float32 CUDA tensors; mode 1 gives the value Lumen reports."""
    out = C.c_double(0.0)
    _check(ctx.lib, ctx.handle, ctx.lib.lgb_film_rmse(ctx.handle, C.c_void_p(film.data_ptr()),
                                                        C.c_void_p(reference.data_ptr()), film.shape[0], mode,
                                                        C.byref(out), C.c_void_p(stream)))
    return out.value


class GpuScene:
    """A scene uploaded with lgb_scene_create; owns its BVH (lgb_bvh_build)."""

    def __init__(self, ctx: Context, arrays: SceneArrays):
        self.ctx = ctx
        self.lib = ctx.lib
        self.arrays = arrays
        desc, keep = arrays.make_desc()
        h = C.c_void_p()
        _check(self.lib, ctx.handle, self.lib.lgb_scene_create(ctx.handle, C.byref(desc), C.byref(h)))
        self.handle = h
        self.stats = None

    def build(self, leaf_max: int = 0, treelet_rounds: int = 0) -> abi.BuildStats:
        opts = abi.BuildOpts()
        opts.leaf_max = leaf_max
        opts.treelet_rounds = treelet_rounds
        stats = abi.BuildStats()
        _check(self.lib, self.ctx.handle, self.lib.lgb_bvh_build(self.handle, C.byref(opts), C.byref(stats)))
        self.stats = stats
        return stats

    def set_visit_limit(self, max_visits: int):
        """lgb_scene_set_visit_limit: node visits one ray of the public queries may make (0 = default)."""
        _check(self.lib, self.ctx.handle, self.lib.lgb_scene_set_visit_limit(self.handle, max_visits))

    def trace_closest(self, rays, hits, n=None, stream=None):
        n = rays.shape[0] if n is None else n
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_trace_closest(self.handle, C.c_void_p(rays.data_ptr()), C.c_void_p(hits.data_ptr()), n,
                                          C.c_void_p(stream)))

    def trace_closest_counted(self, rays, hits, counters, stream=None):
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_trace_closest_counted(self.handle, C.c_void_p(rays.data_ptr()),
                                                  C.c_void_p(hits.data_ptr()), rays.shape[0],
                                                  C.c_void_p(counters.data_ptr()), C.c_void_p(stream)))

    def trace_closest_host(self, rays, hits, stream=None):
        """lgb_trace_closest_host on CPU tensors ((n, 8) float32 rays, (n, 4) int32 hits; pinned for overlap)."""
        assert rays.device.type == "cpu" and hits.device.type == "cpu"
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_trace_closest_host(self.handle, C.c_void_p(rays.data_ptr()), C.c_void_p(hits.data_ptr()),
                                               rays.shape[0], C.c_void_p(stream)))

    def trace_any_host(self, rays, bits, stream=None):
        """lgb_trace_any_host on CPU tensors ((n, 8) float32 rays, ((n + 31) // 32,) int32 occlusion bits)."""
        assert rays.device.type == "cpu" and bits.device.type == "cpu"
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_trace_any_host(self.handle, C.c_void_p(rays.data_ptr()), C.c_void_p(bits.data_ptr()),
                                           rays.shape[0], C.c_void_p(stream)))

    def trace_any(self, rays, bits, n=None, stream=None):
        n = rays.shape[0] if n is None else n
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_trace_any(self.handle, C.c_void_p(rays.data_ptr()), C.c_void_p(bits.data_ptr()), n,
                                      C.c_void_p(stream)))

    def render_path(self, cam: abi.Camera, params: abi.PathParams, frame0: int, spp: int, film, stream=None):
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_render_path(self.handle, C.byref(cam), C.byref(params), frame0, spp,
                                        C.c_void_p(film.data_ptr()), C.c_void_p(stream)))

    def sync(self, stream=None):
        _check(self.lib, self.ctx.handle, self.lib.lgb_sync(self.handle, C.c_void_p(stream)))

    def vcm_iteration(self, cam: abi.Camera, params: abi.VcmParams, film, stream=None):
        """lgb_vcm_iteration into film ((npix, 4) float32 CUDA)."""
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_vcm_iteration(self.handle, C.byref(cam), C.byref(params), C.c_void_p(film.data_ptr()),
                                          C.c_void_p(stream)))

    def vcm_state(self) -> abi.VcmState:
        """lgb_vcm_state_get: device pointers and grid of the VCM state kept in the scene."""
        out = abi.VcmState()
        _check(self.lib, self.ctx.handle, self.lib.lgb_vcm_state_get(self.handle, C.byref(out)))
        return out

    def restir_di_iteration(self, cam: abi.Camera, params: abi.RestirParams, film, prev_cam: abi.Camera = None,
                            stream=None):
        """lgb_restir_di_iteration: one ReSTIR DI frame into film ((npix, 4) float32 CUDA)."""
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_restir_di_iteration(self.handle, C.byref(cam),
                                                C.byref(prev_cam) if prev_cam is not None else None,
                                                C.byref(params), C.c_void_p(film.data_ptr()), C.c_void_p(stream)))

    def sppm_iteration(self, cam: abi.Camera, params: abi.SppmParams, film, stream=None):
        """lgb_sppm_iteration: one SPPM frame into film ((npix, 4) float32 CUDA)."""
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_sppm_iteration(self.handle, C.byref(cam), C.byref(params), C.c_void_p(film.data_ptr()),
                                           C.c_void_p(stream)))

    def bdpt_iteration(self, cam: abi.Camera, params: abi.BdptParams, film, stream=None):
        """lgb_bdpt_iteration: one BDPT frame into film ((npix, 4) float32 CUDA)."""
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_bdpt_iteration(self.handle, C.byref(cam), C.byref(params), C.c_void_p(film.data_ptr()),
                                           C.c_void_p(stream)))

    @staticmethod
    def _diff_params(texture_id, texels, roughness, emission, flags=0) -> abi.DiffParams:
        dp = abi.DiffParams()
        dp.texture_id = texture_id
        dp.flags = flags
        dp.texels = texels.data_ptr() if texels is not None else None
        dp.roughness = roughness.data_ptr() if roughness is not None else None
        dp.emission = emission.data_ptr() if emission is not None else None
        return dp

    def diff_render(self, cam: abi.Camera, params: abi.PathParams, frame0: int, spp: int, film, texture_id=-1,
                    texels=None, roughness=None, emission=None, samples=None, flags=0, stream=None):
        """lgb_diff_render: mean image of the differentiable estimator into film ((npix, 4) float32 CUDA).
        texels (H, W, 4), roughness (num_materials,) and emission (num_materials, 3) are float32 CUDA tensors
        or None (scene values); samples ((spp * npix, 4) float32 CUDA) optionally receives every sample;
        flags = abi.DIFF_SAMPLE_PARAMS samples with the parameter values."""
        dp = self._diff_params(texture_id, texels, roughness, emission, flags)
        sp = C.c_void_p(samples.data_ptr()) if samples is not None else None
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_diff_render(self.handle, C.byref(cam), C.byref(params), C.byref(dp), frame0, spp,
                                        C.c_void_p(film.data_ptr()), sp, C.c_void_p(stream)))

    def adjoint_path(self, cam: abi.Camera, params: abi.PathParams, frame0: int, spp: int, dimage, texture_id=-1,
                     texels=None, roughness=None, emission=None, g_texels=None, g_roughness=None, g_emission=None,
                     samples=None, flags=0, stream=None):
        """lgb_adjoint_path: adds d loss / d parameter into the g_* tensors given dimage = d loss / d image
        ((npix, 4) float32 CUDA) for the image diff_render makes with the same arguments; samples are the
        per-sample radiance diff_render wrote (one replay) or None (primal and replay)."""
        dp = self._diff_params(texture_id, texels, roughness, emission, flags)
        g = abi.DiffGrads()
        g.texels = g_texels.data_ptr() if g_texels is not None else None
        g.roughness = g_roughness.data_ptr() if g_roughness is not None else None
        g.emission = g_emission.data_ptr() if g_emission is not None else None
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_adjoint_path(self.handle, C.byref(cam), C.byref(params), C.byref(dp), frame0, spp,
                                         C.c_void_p(dimage.data_ptr()),
                                         C.c_void_p(samples.data_ptr()) if samples is not None else None,
                                         C.byref(g), C.c_void_p(stream)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.lgb_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """lgb_batch_*: several GpuScenes (BVHs built) rendered as one wavefront. The scenes are kept alive by the
    batch."""

    def __init__(self, ctx: Context, scenes):
        self.ctx = ctx
        self.lib = ctx.lib
        self.scenes = list(scenes)
        arr = (C.c_void_p * len(self.scenes))(*[sc.handle.value for sc in self.scenes])
        h = C.c_void_p()
        _check(self.lib, ctx.handle, self.lib.lgb_batch_create(ctx.handle, arr, len(self.scenes), C.byref(h)))
        self.handle = h

    @staticmethod
    def job(scene_index: int, cam: abi.Camera, params: abi.PathParams, frame0: int, spp: int, film) -> abi.BatchJob:
        j = abi.BatchJob()
        j.scene = scene_index
        j.frame0 = frame0
        j.spp = spp
        j.camera = cam
        j.params = params
        j.d_film = film.data_ptr()
        return j

    @staticmethod
    def _array(jobs):
        return (abi.BatchJob * len(jobs))(*jobs)

    def render(self, jobs, opts: abi.BatchOpts | None = None, stream=None):
        arr = self._array(jobs)
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_batch_render(self.handle, arr, len(jobs), C.byref(opts) if opts is not None else None,
                                         C.c_void_p(stream)))

    def tune(self, jobs, stream=None) -> abi.BatchOpts:
        best = abi.BatchOpts()
        _check(self.lib, self.ctx.handle,
               self.lib.lgb_batch_tune(self.handle, self._array(jobs), len(jobs), C.byref(best), C.c_void_p(stream)))
        return best

    def sync(self, stream=None):
        _check(self.lib, self.ctx.handle, self.lib.lgb_batch_sync(self.handle, C.c_void_p(stream)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.lgb_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def vcm_params(arrays: SceneArrays, max_depth: int, radius: float, light_seed: int, eye_seed: int, frame_num: int,
               use_vm: int = 1, use_vc: int = 1, sky=(0.0, 0.0, 0.0), flags: int = 0,
               spot_angle: float = 0.0) -> abi.VcmParams:
    """PCVCM as VCM::render fills it (src/RayTracer/VCM.cpp:131-147) with explicit seeds; the grid bounds are the
    scene's bounding box. spot_angle: spot cone half-angle in degrees (0: the reference's fixed 30)."""
    p = abi.VcmParams()
    p.sky_col[:] = list(sky)
    p.max_depth = max_depth
    p.num_lights = len(arrays.lights)
    p.light_triangle_count = arrays.light_triangle_count
    p.dir_light_idx = 0xFFFFFFFF
    p.radius = radius
    mn, mx = arrays.bounds()
    p.scene_min[:] = [float(v) for v in mn]
    p.scene_max[:] = [float(v) for v in mx]
    p.use_vm = use_vm
    p.use_vc = use_vc
    p.light_seed = light_seed
    p.eye_seed = eye_seed
    p.frame_num = frame_num
    p.flags = flags
    p.spot_angle = spot_angle
    return p


def sppm_params(arrays: SceneArrays, max_depth: int, base_radius: float, seed: int, frame_num: int,
                sky=(0.0, 0.0, 0.0), spot_angle: float = 0.0) -> abi.SppmParams:
    """PCSPPM as SPPM::render fills it (src/RayTracer/SPPM.cpp:78-96) with an explicit seed."""
    p = abi.SppmParams()
    p.sky_col[:] = list(sky)
    p.max_depth = max_depth
    p.num_lights = len(arrays.lights)
    p.light_triangle_count = arrays.light_triangle_count
    p.dir_light_idx = 0xFFFFFFFF
    p.base_radius = base_radius
    p.seed = seed
    p.frame_num = frame_num
    p.spot_angle = spot_angle
    return p


def bdpt_params(arrays: SceneArrays, max_depth: int, seed: int, frame_num: int, sky=(0.0, 0.0, 0.0),
                spot_angle: float = 0.0) -> abi.BdptParams:
    """PCBDPT as BDPT::render fills it (src/RayTracer/BDPT.cpp:55-64) with an explicit seed."""
    p = abi.BdptParams()
    p.sky_col[:] = list(sky)
    p.max_depth = max_depth
    p.num_lights = len(arrays.lights)
    p.light_triangle_count = arrays.light_triangle_count
    p.dir_light_idx = 0xFFFFFFFF
    p.seed = seed
    p.frame_num = frame_num
    p.spot_angle = spot_angle
    return p


def restir_params(arrays: SceneArrays, seed: int, frame_num: int, do_spatiotemporal: int = 1,
                  enable_accumulation: int = 1, spot_angle: float = 0.0, flags: int = 0) -> abi.RestirParams:
    """PCReSTIR as ReSTIR::render fills it (src/RayTracer/ReSTIR.cpp:74-86) with an explicit seed."""
    p = abi.RestirParams()
    p.max_depth = 6
    p.num_lights = len(arrays.lights)
    p.light_triangle_count = arrays.light_triangle_count
    p.dir_light_idx = 0xFFFFFFFF
    p.seed = seed
    p.frame_num = frame_num
    p.do_spatiotemporal = do_spatiotemporal
    p.enable_accumulation = enable_accumulation
    p.spot_angle = spot_angle
    p.flags = flags
    return p


def scene_radius(arrays: SceneArrays) -> float:
    """Half the diagonal of the scene's bounding box (LumenScene::m_dimensions.radius)."""
    mn, mx = arrays.bounds()
    return float(np.linalg.norm(mx.astype(np.float64) - mn.astype(np.float64)) / 2.0)


def path_params(arrays: SceneArrays, max_depth: int, sky=(0.0, 0.0, 0.0), direct_lighting: int = 1,
                film_mode: int = 0) -> abi.PathParams:
    """PCPath as Path::render fills it (src/RayTracer/Path.cpp:28-38)."""
    p = abi.PathParams()
    p.sky_col[:] = list(sky)
    p.max_depth = max_depth
    p.num_lights = len(arrays.lights)
    p.light_triangle_count = arrays.light_triangle_count
    p.dir_light_idx = 0xFFFFFFFF
    p.direct_lighting = direct_lighting
    p.film_mode = film_mode
    return p
