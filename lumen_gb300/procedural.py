"""Seeded procedural scenes and ray sets for the benchmark configurations.

Generation runs in float64 from numpy's PCG64 streams and is cast to float32 once at the end, so a seed
fixes the arrays; tests that need bit-identical inputs on every host read them from committed fixtures.

  cornell_box()        36 triangles: 5 walls (white 0.73 / red / green), two boxes rotated +-18 deg about y,
                       a 0.5 x 0.5 emitter (L = 17) just below the ceiling; camera on the +z axis
                       viewing the box along -z.
  cornell_diff()       the same box with a textured back wall and two GGX conductor boxes (differentiable
                       rendering).
  traversal_scene()    icosphere of frequency 200 (800 000 triangles) displaced by 3-octave value noise of
                       amplitude 0.1, plus 200 000 random small triangles in [-2, 2]^3.
  batch_scene()        displaced sphere + floor + boxes + 1-8 quad lights with principled / dielectric
                       materials (batched rendering); batch_config() draws the 32 scenes' sizes.
  vcm_scene()          dielectric torus on a diffuse plane lit by a spot light (VCM caustics).
  primary_rays()       one ray per pixel centre of a pinhole camera.
  incoherent_rays()    origins area-uniform on the surfaces, cosine-distributed about a random side.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .scene import MESH_DTYPE, LIGHT_DTYPE, SceneArrays, conductor, diffuse

WHITE = (0.73, 0.73, 0.73)
RED = (0.63, 0.065, 0.05)
GREEN = (0.14, 0.45, 0.09)


class _Builder:
    """Accumulates unwelded triangle meshes the way Lumen's OBJ loader lays them out (LumenScene.cpp:302-324)."""

    def __init__(self):
        self.pos, self.nrm, self.uv, self.idx, self.meshes = [], [], [], [], []
        self.nv = 0
        self.ni = 0

    def add(self, tris: np.ndarray, normals: np.ndarray | None, material: int, uvs: np.ndarray | None = None):
        """tris: (T, 3, 3) float64 vertices; normals: (T, 3, 3) or None (flat geometric normals)."""
        t = len(tris)
        if normals is None:
            e0 = tris[:, 2] - tris[:, 0]
            e1 = tris[:, 1] - tris[:, 0]
            n = np.cross(e0, e1)
            n = n / np.sqrt((n * n).sum(-1, keepdims=True))
            normals = np.repeat(n[:, None, :], 3, axis=1)
        if uvs is None:
            uvs = np.tile(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]), (t, 1, 1))
        self.pos.append(tris.reshape(-1, 3))
        self.nrm.append(normals.reshape(-1, 3))
        self.uv.append(uvs.reshape(-1, 2))
        m = np.zeros(1, MESH_DTYPE)
        m["index_offset"] = self.ni
        m["vertex_offset"] = self.nv
        m["material_index"] = material
        m["tri_count"] = t
        self.idx.append(np.arange(3 * t, dtype=np.uint32))
        self.meshes.append(m)
        self.nv += 3 * t
        self.ni += 3 * t
        return len(self.meshes) - 1

    def arrays(self, materials, lights, light_tri_count, cam_pos, cam_dir, fov):
        return SceneArrays(
            positions=np.concatenate(self.pos).astype(np.float32),
            normals=np.concatenate(self.nrm).astype(np.float32),
            uvs=np.concatenate(self.uv).astype(np.float32),
            indices=np.concatenate(self.idx).astype(np.uint32),
            meshes=np.concatenate(self.meshes),
            materials=np.concatenate(materials),
            lights=lights,
            light_triangle_count=light_tri_count,
            camera_pos=cam_pos,
            camera_dir=cam_dir,
            fov=fov,
        )


def _quad(p0, p1, p2, p3, inward):
    """Two triangles (p0, p1, p2), (p0, p2, p3) oriented so that the geometric normal of ray.rchit
    (cross(v2 - v0, v1 - v0)) points along `inward`."""
    q = np.array([p0, p1, p2, p3], np.float64)
    t = np.array([[q[0], q[1], q[2]], [q[0], q[2], q[3]]])
    n = np.cross(t[0, 2] - t[0, 0], t[0, 1] - t[0, 0])
    if np.dot(n, inward) < 0:
        t = t[:, [0, 2, 1]]
    nn = np.array(inward, np.float64) / np.linalg.norm(inward)
    return t, np.tile(nn, (2, 3, 1))


def _box(center, size, angle_deg):
    """Closed axis-aligned box rotated about y; outward flat normals. Returns (12, 3, 3), (12, 3, 3)."""
    hx, hy, hz = (s / 2.0 for s in size)
    c, s = math.cos(math.radians(angle_deg)), math.sin(math.radians(angle_deg))
    rot = np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])
    faces = []
    normals = []
    # (axis, sign)
    for axis in range(3):
        for sign in (-1.0, 1.0):
            u, v = [a for a in range(3) if a != axis]
            corners = []
            for du, dv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                p = np.zeros(3)
                p[axis] = sign
                p[u] = du
                p[v] = dv
                corners.append(p * np.array([hx, hy, hz]))
            outward = np.zeros(3)
            outward[axis] = sign
            t, n = _quad(*corners, inward=outward)
            faces.append(t)
            normals.append(n)
    tris = np.concatenate(faces) @ rot.T + np.array(center)
    nrms = np.concatenate(normals) @ rot.T
    return tris, nrms


def cornell_box() -> SceneArrays:
    """The 36-triangle Cornell box of the path-tracer configuration (256^2, 16 spp, depth 8)."""
    b = _Builder()
    mats = [diffuse(WHITE), diffuse(RED), diffuse(GREEN), diffuse((1.0, 1.0, 1.0), emissive=(17.0, 17.0, 17.0))]
    W, R, G, E = 0, 1, 2, 3
    # walls of [-1, 1]^3, open towards +z where the camera is
    t, n = _quad((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), inward=(0, 1, 0))
    b.add(t, n, W)  # floor
    t, n = _quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), inward=(0, -1, 0))
    b.add(t, n, W)  # ceiling
    t, n = _quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), inward=(0, 0, 1))
    b.add(t, n, W)  # back wall
    t, n = _quad((-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1), inward=(1, 0, 0))
    b.add(t, n, R)  # left wall (x = -1, left in the image)
    t, n = _quad((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1), inward=(-1, 0, 0))
    b.add(t, n, G)  # right wall
    t, n = _box((0.35, -0.7, -0.25), (0.6, 0.6, 0.6), -18.0)
    b.add(t, n, W)  # short box
    t, n = _box((-0.33, -0.4, -0.45), (0.6, 1.2, 0.6), 18.0)
    b.add(t, n, W)  # tall box
    y = 0.999
    t, n = _quad((-0.25, y, -0.25), (0.25, y, -0.25), (0.25, y, 0.25), (-0.25, y, 0.25), inward=(0, -1, 0))
    light_mesh = b.add(t, n, E)
    lights = np.zeros(1, LIGHT_DTYPE)
    lights["world_matrix"] = np.eye(4, dtype=np.float32).reshape(16)
    lights["prim_mesh_idx"] = light_mesh
    lights["num_triangles"] = 2
    lights["L"] = 17.0
    lights["light_flags"] = abi.LIGHT_AREA | abi.LIGHT_FINITE
    # Lumen's camera "dir" is the look-at direction of a left-handed view combined with a right-handed
    # projection (Camera.h:74,111-115), so the rendered view looks along -dir: here towards -z.
    return b.arrays(mats, lights, 2, (0.0, 0.0, 3.5), (0.0, 0.0, 1.0), 45.0)


def albedo_texture(seed: int, size: int = 64) -> np.ndarray:
    """(size, size, 4) float32 RGBA texture with RGB uniform in [0.1, 0.9] from PCG64(seed), alpha 1."""
    rng = np.random.default_rng(seed)
    tex = np.ones((size, size, 4), np.float32)
    tex[..., :3] = rng.uniform(0.1, 0.9, (size, size, 3))
    return tex


def cornell_diff(texture_seed: int = 5, roughness=(0.35, 0.2)) -> SceneArrays:
    """The Cornell box of the differentiable-rendering configuration: the back wall has its own white material
    (albedo 1) modulated by a 64 x 64 RGB texture (albedo_texture(texture_seed)), mapped once over the wall
    (u along +x, v along +y); the short and tall boxes are GGX conductors (reflectance 0.9, 0.6, 0.3 and
    0.8, 0.8, 0.8) with one roughness per box. Materials: 0 white, 1 red, 2 green, 3 emitter, 4 back wall,
    5 short box, 6 tall box."""
    b = _Builder()
    mats = [diffuse(WHITE), diffuse(RED), diffuse(GREEN), diffuse((1.0, 1.0, 1.0), emissive=(17.0, 17.0, 17.0)),
            diffuse((1.0, 1.0, 1.0)), conductor((0.9, 0.6, 0.3), roughness[0]), conductor((0.8, 0.8, 0.8), roughness[1])]
    mats[4]["texture_id"] = 0
    W, R, G, E, BACK, SHORT, TALL = range(7)
    t, n = _quad((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1), inward=(0, 1, 0))
    b.add(t, n, W)
    t, n = _quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), inward=(0, -1, 0))
    b.add(t, n, W)
    t, n = _quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), inward=(0, 0, 1))
    uv = (t[..., :2] + 1.0) * 0.5  # back wall at z = -1: (x, y) in [-1, 1]^2 -> [0, 1]^2
    b.add(t, n, BACK, uv)
    t, n = _quad((-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1), inward=(1, 0, 0))
    b.add(t, n, R)
    t, n = _quad((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1), inward=(-1, 0, 0))
    b.add(t, n, G)
    t, n = _box((0.35, -0.7, -0.25), (0.6, 0.6, 0.6), -18.0)
    b.add(t, n, SHORT)
    t, n = _box((-0.33, -0.4, -0.45), (0.6, 1.2, 0.6), 18.0)
    b.add(t, n, TALL)
    y = 0.999
    t, n = _quad((-0.25, y, -0.25), (0.25, y, -0.25), (0.25, y, 0.25), (-0.25, y, 0.25), inward=(0, -1, 0))
    light_mesh = b.add(t, n, E)
    lights = np.zeros(1, LIGHT_DTYPE)
    lights["world_matrix"] = np.eye(4, dtype=np.float32).reshape(16)
    lights["prim_mesh_idx"] = light_mesh
    lights["num_triangles"] = 2
    lights["L"] = 17.0
    lights["light_flags"] = abi.LIGHT_AREA | abi.LIGHT_FINITE
    arrays = b.arrays(mats, lights, 2, (0.0, 0.0, 3.5), (0.0, 0.0, 1.0), 45.0)
    arrays.textures = [albedo_texture(texture_seed)]
    return arrays


# ---------------------------------------------------------------------------------------------------
# traversal scene

_ICO_V = None


def _icosahedron():
    p = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], np.float64)
    v /= np.sqrt((v * v).sum(-1, keepdims=True))
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    return v, f


def _lattice_hash(ix, iy, iz, seed):
    """Integer lattice hash -> value in [-1, 1]."""
    h = (ix.astype(np.uint64) * np.uint64(73856093)) ^ (iy.astype(np.uint64) * np.uint64(19349663)) ^ \
        (iz.astype(np.uint64) * np.uint64(83492791)) ^ np.uint64(seed * 2654435761 & 0xFFFFFFFF)
    h = h & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(16)
    h = (h * np.uint64(0x7feb352d)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x846ca68b)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(16)
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise(p: np.ndarray, freq: float, seed: int) -> np.ndarray:
    """Trilinear value noise with smoothstep weights on an integer lattice scaled by freq."""
    q = p * freq
    i = np.floor(q)
    f = q - i
    w = f * f * (3.0 - 2.0 * f)
    i = i.astype(np.int64) + 1024  # keep lattice coordinates positive
    out = np.zeros(len(p))
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1.0 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += wx * wy * wz * _lattice_hash(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
    return out


def displaced_icosphere(freq: int = 200, amplitude: float = 0.1, seed: int = 1, radius: float = 1.0,
                        center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Class-I geodesic sphere (20 * freq^2 triangles), displaced along the normal by 3-octave value noise
    (octaves 4, 8, 16; gains 1, 1/2, 1/4; normalised to `amplitude`). Returns (T, 3, 3) float64."""
    v, f = _icosahedron()
    n = freq
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = ii + jj <= n
    ii, jj = ii[keep], jj[keep]
    # index of grid point (i, j) in the per-face point list
    lut = -np.ones((n + 1, n + 1), np.int64)
    lut[ii, jj] = np.arange(len(ii))
    # triangles of the per-face grid
    a_i, a_j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    up = a_i + a_j <= n - 1
    ui, uj = a_i[up], a_j[up]
    tri_up = np.stack([lut[ui, uj], lut[ui + 1, uj], lut[ui, uj + 1]], -1)
    dn = a_i + a_j <= n - 2
    di, dj = a_i[dn], a_j[dn]
    tri_dn = np.stack([lut[di + 1, dj], lut[di + 1, dj + 1], lut[di, dj + 1]], -1)
    local = np.concatenate([tri_up, tri_dn])
    tris = []
    for face in f:
        A, B, Cc = v[face[0]], v[face[1]], v[face[2]]
        pts = A + (B - A) * (ii[:, None] / n) + (Cc - A) * (jj[:, None] / n)
        pts /= np.sqrt((pts * pts).sum(-1, keepdims=True))
        tris.append(pts[local])
    tris = np.concatenate(tris)  # (20 n^2, 3, 3) on the unit sphere
    flat = tris.reshape(-1, 3)
    disp = (value_noise(flat, 4.0, seed) + 0.5 * value_noise(flat, 8.0, seed + 1) +
            0.25 * value_noise(flat, 16.0, seed + 2)) / 1.75
    flat = flat * (radius * (1.0 + amplitude * disp))[:, None] + np.asarray(center)
    return flat.reshape(-1, 3, 3)


def _random_rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.sqrt((q * q).sum(-1, keepdims=True))
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def random_triangles(n: int = 200_000, seed: int = 2, lo=-2.0, hi=2.0, edge=(0.01, 0.05)) -> np.ndarray:
    """Equilateral triangles with centres U[lo, hi]^3, edge length U[edge] and uniformly random orientation."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(lo, hi, (n, 3))
    e = rng.uniform(edge[0], edge[1], n)
    R = _random_rotations(rng, n)
    h = math.sqrt(3.0) / 2.0
    base = np.array([[1.0, 0.0, 0.0], [-0.5, h, 0.0], [-0.5, -h, 0.0]]) / math.sqrt(3.0)  # unit edge
    return c[:, None, :] + e[:, None, None] * np.einsum("nij,kj->nki", R, base)


def traversal_scene(sphere_freq: int = 200, n_random: int = 200_000, seed: int = 1) -> SceneArrays:
    """The 1M-triangle traversal benchmark scene (two meshes, one diffuse material, no lights)."""
    b = _Builder()
    sph = displaced_icosphere(sphere_freq, 0.1, seed)
    b.add(sph, None, 0)
    if n_random:
        b.add(random_triangles(n_random, seed + 1), None, 0)
    return b.arrays([diffuse(WHITE)], np.zeros(0, LIGHT_DTYPE), 0, (0.0, 0.0, -4.0), (0.0, 0.0, 1.0), 45.0)


def batch_scene(seed: int, n_tris: int) -> SceneArrays:
    """One scene of the batched-rendering configuration: a displaced icosphere of about n_tris triangles
    (frequency round(sqrt(n_tris / 20))) on a floor, three boxes and 1-8 quad lights (L = 12) overhead. Every
    surface material is drawn from PCG64(seed): with probability 0.2 a smooth dielectric of IOR 1.5, else
    Disney principled with baseColor U[0,1]^3, roughness U[0.05,1], metallic Bernoulli(0.3) and specular 0.5
    (IOR 1.5, F0 = 0.04). Camera on +z looking at the sphere."""
    rng = np.random.default_rng(seed)
    from .scene import dielectric, principled

    def material():
        if rng.uniform() < 0.2:
            return dielectric(1.5, 0.0)
        return principled(tuple(rng.uniform(0.0, 1.0, 3)), roughness=float(rng.uniform(0.05, 1.0)),
                          metallic=float(rng.uniform() < 0.3), ior=1.5)

    b = _Builder()
    mats = []
    freq = max(2, int(round(math.sqrt(n_tris / 20.0))))
    mats.append(material())
    b.add(displaced_icosphere(freq, 0.1, seed * 7 + 1), None, len(mats) - 1)
    mats.append(material())
    t, n = _quad((-4, -1.2, -4), (4, -1.2, -4), (4, -1.2, 4), (-4, -1.2, 4), inward=(0, 1, 0))
    b.add(t, n, len(mats) - 1)
    for k in range(3):
        mats.append(material())
        c = (float(rng.uniform(-2.5, 2.5)), -1.2 + 0.3, float(rng.uniform(-2.5, 0.5)))
        t, n = _box(c, (0.6, 0.6, 0.6), float(rng.uniform(-45, 45)))
        b.add(t, n, len(mats) - 1)
    n_lights = int(rng.integers(1, 9))
    emitter = diffuse((1.0, 1.0, 1.0), emissive=(12.0, 12.0, 12.0))
    mats.append(emitter)
    lights = np.zeros(n_lights, LIGHT_DTYPE)
    for k in range(n_lights):
        cx, cz = (float(v) for v in rng.uniform(-2.0, 2.0, 2))
        y = 2.5
        t, n = _quad((cx - 0.25, y, cz - 0.25), (cx + 0.25, y, cz - 0.25), (cx + 0.25, y, cz + 0.25),
                     (cx - 0.25, y, cz + 0.25), inward=(0, -1, 0))
        mesh = b.add(t, n, len(mats) - 1)
        lights[k]["world_matrix"] = np.eye(4, dtype=np.float32).reshape(16)
        lights[k]["prim_mesh_idx"] = mesh
        lights[k]["num_triangles"] = 2
        lights[k]["L"] = 12.0
        lights[k]["light_flags"] = abi.LIGHT_AREA | abi.LIGHT_FINITE
    return b.arrays(mats, lights, 2 * n_lights, (0.0, 0.5, 4.5), (0.0, 0.5 / 4.5, 1.0), 45.0)


def batch_config(seed: int = 0, n_scenes: int = 32, min_tris: int = 10_000, max_tris: int = 2_000_000,
                 min_res: int = 128, max_res: int = 1024, min_spp: int = 8, max_spp: int = 64):
    """The batched-rendering configuration: n_scenes (seed, triangles, width, height, spp) with triangle counts,
    square resolutions (multiples of 32) and spp log-uniform in their ranges, drawn from PCG64(seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        tris = int(round(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))))
        res = int(round(math.exp(rng.uniform(math.log(min_res), math.log(max_res))) / 32.0)) * 32
        res = min(max(res, min_res), max_res)
        spp = int(round(math.exp(rng.uniform(math.log(min_spp), math.log(max_spp)))))
        out.append((1000 + i, tris, res, res, spp))
    return out


def torus(R: float = 1.0, r: float = 0.35, n_major: int = 500, n_minor: int = 200, center=(0.0, 0.35, 0.0)):
    """Torus around the y axis with smooth analytic normals: 2 * n_major * n_minor triangles, (T, 3, 3) vertices
    and normals."""
    u = np.arange(n_major + 1) * (2.0 * math.pi / n_major)
    v = np.arange(n_minor + 1) * (2.0 * math.pi / n_minor)
    U, V = np.meshgrid(u, v, indexing="ij")
    cu, su, cv, sv = np.cos(U), np.sin(U), np.cos(V), np.sin(V)
    pos = np.stack([(R + r * cv) * cu, r * sv, (R + r * cv) * su], -1) + np.asarray(center)
    nrm = np.stack([cv * cu, sv, cv * su], -1)
    i, j = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    i, j = i.ravel(), j.ravel()
    a, b, c, d = (i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1)
    tri_idx = [(a, c, b), (a, d, c)]
    tris = np.concatenate([np.stack([pos[p0], pos[p1], pos[p2]], 1) for p0, p1, p2 in tri_idx])
    nrms = np.concatenate([np.stack([nrm[p0], nrm[p1], nrm[p2]], 1) for p0, p1, p2 in tri_idx])
    return tris, nrms


def vcm_scene(n_major: int = 500, n_minor: int = 200) -> SceneArrays:
    """The VCM caustics configuration: a smooth dielectric torus (IOR 1.5, R = 1, r = 0.35, 2 * n_major * n_minor
    triangles, 200 000 by default) resting on a 10 x 10 diffuse plane (albedo 0.8), lit by a spot light of
    intensity 100 at (0, 4, 1) aimed at the torus. Lumen's spot light has a fixed 30 degree cone with a 25 degree
    falloff start (commons.glsl:264-265, 344-345): its Light record has no cone angle. Camera at (0, 3, 5)."""
    from .scene import dielectric
    b = _Builder()
    mats = [diffuse((0.8, 0.8, 0.8)), dielectric(1.5, 0.0)]
    t, n = _quad((-5, 0, -5), (5, 0, -5), (5, 0, 5), (-5, 0, 5), inward=(0, 1, 0))
    b.add(t, n, 0)
    t, n = torus(1.0, 0.35, n_major, n_minor)
    b.add(t, n, 1)
    lights = np.zeros(1, LIGHT_DTYPE)
    lights["world_matrix"] = np.eye(4, dtype=np.float32).reshape(16)
    lights["pos"] = (0.0, 4.0, 1.0)
    lights["to"] = (0.0, 0.0, 0.0)
    lights["L"] = 100.0
    lights["light_flags"] = abi.LIGHT_SPOT | abi.LIGHT_FINITE | abi.LIGHT_DELTA
    cam_pos = np.array([0.0, 3.0, 5.0])
    cam_dir = cam_pos - np.array([0.0, 0.2, 0.0])  # Lumen's view looks along -dir
    cam_dir /= np.linalg.norm(cam_dir)
    # a non-area light counts as one light triangle (LumenScene.cpp:106)
    return b.arrays(mats, lights, 1, tuple(cam_pos), tuple(cam_dir), 45.0)


def primary_rays(width: int, height: int, pos=(0.0, 0.0, -4.0), fov: float = 45.0, tmax: float = 10000.0) -> np.ndarray:
    """(W*H, 8) float32 rays through pixel centres of a pinhole camera looking along +z (row 0 at +y)."""
    t = math.tan(math.radians(fov) / 2.0)
    aspect = width / height
    x = (np.arange(width) + 0.5) / width * 2.0 - 1.0
    y = (np.arange(height) + 0.5) / height * 2.0 - 1.0
    X, Y = np.meshgrid(x, y)
    d = np.stack([X * t * aspect, -Y * t, np.ones_like(X)], -1).reshape(-1, 3)
    d /= np.sqrt((d * d).sum(-1, keepdims=True))
    rays = np.zeros((len(d), 8), np.float32)
    rays[:, 0:3] = pos
    rays[:, 3] = 0.0
    rays[:, 4:7] = d
    rays[:, 7] = tmax
    return rays


def offset_ray(p: np.ndarray, n: np.ndarray) -> np.ndarray:
    """Integer-ULP ray origin offset of utils.glsl:73-84 on float32 arrays."""
    p = p.astype(np.float32)
    n = n.astype(np.float32)
    of = (np.float32(256.0) * n).astype(np.int32)  # truncation as GLSL int()
    pi = p.view(np.int32)
    moved = (pi + np.where(p < 0, -of, of)).astype(np.int32).view(np.float32)
    small = np.abs(p) < np.float32(1.0 / 32.0)
    return np.where(small, p + np.float32(1.0 / 65536.0) * n, moved).astype(np.float32)


def incoherent_rays(arrays: SceneArrays, n: int, seed: int = 3, tmax: float = 10000.0) -> np.ndarray:
    """(n, 8) float32 rays: a triangle picked with probability proportional to its area, a uniform point on it,
    a random side of its geometric normal, origin pushed off the surface with offset_ray, and a
    cosine-distributed direction about that side's normal."""
    rng = np.random.default_rng(seed)
    tv = arrays.tri_verts().astype(np.float64).reshape(-1, 3, 3)
    e1 = tv[:, 1] - tv[:, 0]
    e2 = tv[:, 2] - tv[:, 0]
    cr = np.cross(e1, e2)
    area = 0.5 * np.sqrt((cr * cr).sum(-1))
    cdf = np.cumsum(area)
    cdf /= cdf[-1]
    tri = np.minimum(np.searchsorted(cdf, rng.random(n)), len(tv) - 1)
    r1 = rng.random(n)
    r2 = rng.random(n)
    s = np.sqrt(r1)
    b0, b1, b2 = 1.0 - s, s * (1.0 - r2), s * r2
    p = tv[tri, 0] * b0[:, None] + tv[tri, 1] * b1[:, None] + tv[tri, 2] * b2[:, None]
    ng = cr[tri] / np.sqrt((cr[tri] ** 2).sum(-1, keepdims=True))
    side = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    ng = ng * side[:, None]
    # cosine-weighted direction: uniform point in the unit disk (rejection), lifted to the hemisphere
    xy = np.zeros((n, 2))
    todo = np.arange(n)
    while len(todo):
        cand = rng.uniform(-1.0, 1.0, (len(todo), 2))
        ok = (cand * cand).sum(-1) < 1.0
        xy[todo[ok]] = cand[ok]
        todo = todo[~ok]
    z = np.sqrt(np.maximum(0.0, 1.0 - (xy * xy).sum(-1)))
    sgn = np.where(ng[:, 2] >= 0.0, 1.0, -1.0)
    a = -1.0 / (sgn + ng[:, 2])
    bb = ng[:, 0] * ng[:, 1] * a
    t1 = np.stack([1.0 + sgn * ng[:, 0] ** 2 * a, sgn * bb, -sgn * ng[:, 0]], -1)
    t2 = np.stack([bb, sgn + ng[:, 1] ** 2 * a, -ng[:, 1]], -1)
    d = xy[:, 0:1] * t1 + xy[:, 1:2] * t2 + z[:, None] * ng
    d /= np.sqrt((d * d).sum(-1, keepdims=True))
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = offset_ray(p.astype(np.float32), ng.astype(np.float32))
    rays[:, 3] = 0.0
    rays[:, 4:7] = d
    rays[:, 7] = tmax
    return rays
