"""CPU tests of the C++ host layer (liblgb_host.so): Lumen JSON/OBJ scene loading onto the C ABI arrays,
checked against the mapping rules of LumenScene.cpp restated here in numpy."""
import os

import numpy as np
import pytest

from lumen_gb300 import abi, build

HERE = os.path.dirname(os.path.abspath(__file__))
SCENE = os.path.join(HERE, "golden", "scenes", "mixed.json")


@pytest.fixture(scope="module")
def loaded():
    from lumen_gb300 import host_scene
    if not os.path.exists(host_scene.HOST_LIB):
        build.build_library()
    return host_scene.load_scene(SCENE)


def test_meshes_and_material_refs(loaded):
    arrays, info = loaded
    assert list(arrays.meshes["tri_count"]) == [2, 2, 12, 4, 2, 2, 2]
    assert list(arrays.meshes["material_index"]) == [0, 0, 1, 2, 3, 4, 5]
    assert list(arrays.meshes["index_offset"]) == [0, 6, 12, 48, 60, 66, 72]
    assert list(arrays.meshes["vertex_offset"]) == [0, 6, 12, 48, 60, 66, 72]
    # indices are per-mesh local, one fresh vertex per face corner (LumenScene.cpp:302-324)
    assert np.array_equal(arrays.indices[:6], np.arange(6))
    assert len(arrays.positions) == 78
    # fan triangulation of the first quad: corners (1, 2, 3) and (1, 3, 4)
    np.testing.assert_array_equal(arrays.positions[:6], [[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, -2], [2, 0, 2], [-2, 0, 2]])
    np.testing.assert_array_equal(arrays.uvs[:3], [[0, 0], [1, 0], [1, 1]])
    np.testing.assert_array_equal(arrays.normals[:6], np.tile([0, 1, 0], (6, 1)))


def test_missing_normals_get_geometric_normal(loaded):
    arrays, _ = loaded
    p = arrays.positions[12:15].astype(np.float64)  # first triangle of "block" (no vn in the file)
    n = np.cross(p[2] - p[0], p[1] - p[0])
    n /= np.linalg.norm(n)
    np.testing.assert_allclose(arrays.normals[12:15], np.tile(n, (3, 1)), atol=1e-6)
    assert (arrays.uvs[12:15] == 0).all()


def test_material_mapping(loaded):
    arrays, _ = loaded
    m = arrays.materials
    assert m[0]["bsdf_type"] == abi.BSDF_DIFFUSE and m[0]["bsdf_props"] == abi.FLAG_DIFFUSE | abi.FLAG_REFLECTION
    np.testing.assert_allclose(m[0]["albedo"], 0.7, rtol=1e-7)
    # conductor with reflectance: eta = 1, k = 2 sqrt(r) / sqrt(max(1 - r, 0.001)) (LumenScene.cpp:47-50)
    r = np.array([0.9, 0.7, 0.3], np.float32)
    k = np.float32(2.0) * np.sqrt(r) / np.sqrt(np.maximum(np.float32(1.0) - r, np.float32(0.001)))
    assert m[1]["bsdf_type"] == abi.BSDF_CONDUCTOR
    np.testing.assert_allclose(m[1]["albedo"], 1.0)
    np.testing.assert_allclose(m[1]["k"], k, rtol=1e-6)
    assert m[1]["bsdf_props"] == abi.FLAG_REFLECTION | abi.FLAG_GLOSSY
    # dielectric: both lobes by default, specular below roughness 0.08
    assert m[2]["bsdf_type"] == abi.BSDF_DIELECTRIC and m[2]["ior"] == np.float32(1.5)
    assert m[2]["bsdf_props"] == abi.FLAG_TRANSMISSION | abi.FLAG_REFLECTION | abi.FLAG_SPECULAR
    # principled defaults (LumenScene.cpp:444-475)
    p = m[3]
    assert p["bsdf_type"] == abi.BSDF_PRINCIPLED and p["bsdf_props"] == abi.FLAG_REFLECTION | abi.FLAG_GLOSSY
    assert p["sheen_tint"] == np.float32(0.5) and p["clearcoat_gloss"] == 1.0 and p["clearcoat"] == np.float32(0.5)
    assert p["ior"] == np.float32(1.45) and p["metallic"] == 0.0
    # conductor with edge tint and reflectivity (Gulbrandsen mapping, LumenScene.cpp:425-435)
    g = np.array([0.9, 0.8, 0.7], np.float64)
    rr = np.array([0.6, 0.5, 0.4], np.float64)
    n = g * (1 - rr) / (1 + rr) + (1 - g) * (1 + np.sqrt(rr)) / (1 - np.sqrt(rr))
    kk = np.sqrt(1 / (1 - rr) * ((rr * (n + 1)) ** 2 - (n - 1) ** 2))
    np.testing.assert_allclose(m[4]["albedo"], n, rtol=1e-5)
    np.testing.assert_allclose(m[4]["k"], kk, rtol=1e-5)
    assert m[4]["bsdf_props"] == abi.FLAG_REFLECTION | abi.FLAG_SPECULAR
    np.testing.assert_allclose(m[5]["emissive_factor"], [10, 9, 8])
    assert (m["texture_id"] == -1).all()


def test_lights_camera_and_config(loaded):
    arrays, info = loaded
    L = arrays.lights
    assert len(L) == 2
    assert L[0]["light_flags"] == abi.LIGHT_AREA | abi.LIGHT_FINITE and L[0]["prim_mesh_idx"] == 6
    assert L[0]["num_triangles"] == 2
    np.testing.assert_allclose(L[0]["L"], [10, 9, 8])
    np.testing.assert_allclose(L[0]["world_matrix"], np.eye(4).reshape(16))
    assert L[1]["light_flags"] == abi.LIGHT_SPOT | abi.LIGHT_FINITE | abi.LIGHT_DELTA
    np.testing.assert_allclose(L[1]["pos"], [0, 1.8, 1])
    radius = 0.5 * np.sqrt(4 ** 2 + 2.5 ** 2 + 4 ** 2)
    np.testing.assert_allclose(L[1]["world_radius"], radius, rtol=1e-6)
    np.testing.assert_allclose(L[1]["world_center"], [0, 1.25, 0])
    assert info.light_triangle_count == 3 and arrays.light_triangle_count == 3
    assert info.path_length == 5 and info.dir_light_idx == 0xFFFFFFFF
    np.testing.assert_allclose(list(info.sky_col), [0.05, 0.06, 0.07], rtol=1e-6)
    np.testing.assert_allclose(list(info.cam_pos), [0, 0.6, 4])
    assert info.fov == 40.0
    np.testing.assert_allclose(info.total_light_area, 0.64, rtol=1e-6)


def test_load_errors(tmp_path):
    from lumen_gb300 import host_scene
    with pytest.raises(abi.LgbError, match="cannot open"):
        host_scene.load_scene(str(tmp_path / "missing.json"))
    unknown = tmp_path / "unknown.json"
    unknown.write_text('{"bsdfs": [{"type": "velvet", "albedo": [0.5, 0.5, 0.5], "emissive_factor": [1, 2, 3], '
                       '"refs": ["a"]}], "mesh_file": "x.obj", "camera": {"fov": 40, "position": [0, 0, 5], '
                       '"dir": [0, 0, -1]}, "lights": []}')
    (tmp_path / "x.obj").write_text("o a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    arrays, _ = host_scene.load_scene(str(unknown))  # as Lumen's loader: no lobes, emission kept
    assert arrays.materials[0]["bsdf_type"] == 0 and arrays.materials[0]["bsdf_props"] == 0
    np.testing.assert_allclose(arrays.materials[0]["emissive_factor"], [1, 2, 3])
    broken = tmp_path / "broken.json"
    broken.write_text('{"mesh_file": "x.obj", ')
    with pytest.raises(abi.LgbError, match="JSON parse error"):
        host_scene.load_scene(str(broken))


def _read_exr(path):
    """Reader for single-part, uncompressed scanline OpenEXR with FLOAT channels (the subset the host layer
    writes), from the published file layout: returns {channel: (H, W) float32}."""
    import struct
    data = open(path, "rb").read()
    assert data[:4] == b"\x76\x2f\x31\x01" and struct.unpack_from("<I", data, 4)[0] & 0xff == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        tend = data.index(b"\0", end + 1)
        size = struct.unpack_from("<I", data, tend + 1)[0]
        attrs[name] = data[tend + 5:tend + 5 + size]
        pos = tend + 5 + size
    pos += 1
    chans, p = [], 0
    cl = attrs["channels"]
    while cl[p] != 0:
        e = cl.index(b"\0", p)
        chans.append((cl[p:e].decode(), struct.unpack_from("<i", cl, e + 1)[0]))
        p = e + 1 + 16
    assert attrs["compression"] == b"\0" and all(t == 2 for _, t in chans)
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack_from(f"<{h}Q", data, pos)
    out = {c: np.zeros((h, w), np.float32) for c, _ in chans}
    for off in offsets:
        y, size = struct.unpack_from("<iI", data, off)
        assert size == 4 * w * len(chans)
        row = np.frombuffer(data, np.float32, w * len(chans), off + 8).reshape(len(chans), w)
        for k, (c, _) in enumerate(chans):
            out[c][y - y0] = row[k]
    return out


def test_film_writers_exr_and_pfm(tmp_path):
    from lumen_gb300 import host_scene
    rng = np.random.default_rng(3)
    w, h = 37, 23
    film = rng.uniform(0, 5, (w * h, 4)).astype(np.float32)
    film[5, :3] = [np.inf, 0.0, 1e-30]
    host_scene.write_image(str(tmp_path / "f.exr"), film, w, h)
    img = _read_exr(str(tmp_path / "f.exr"))
    assert sorted(img) == ["B", "G", "R"]
    for k, c in enumerate("RGB"):
        np.testing.assert_array_equal(img[c], film[:, k].reshape(h, w))
    host_scene.write_image(str(tmp_path / "f.pfm"), film, w, h)
    raw = open(tmp_path / "f.pfm", "rb").read()
    header_end = [i for i, b in enumerate(raw) if b == 0x0a][2] + 1
    assert raw[:3] == b"PF\n"
    pfm = np.frombuffer(raw[header_end:], "<f4").reshape(h, w, 3)[::-1]  # PFM rows run bottom-up
    np.testing.assert_array_equal(pfm, film[:, :3].reshape(h, w, 3))
    with pytest.raises(abi.LgbError):
        host_scene.write_image(str(tmp_path / "no" / "such" / "dir.exr"), film, w, h)


def test_integrator_blocks():
    """The integrator block's own fields (LumenScene.cpp:237-253): base_radius for SPPM; radius_factor and
    enable_vm for VCM; each read only for its own integrator type."""
    from lumen_gb300 import host_scene
    scenes = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scenes")
    _, sppm = host_scene.load_scene(os.path.join(scenes, "mixed_sppm.json"))
    assert sppm.path_length == 5 and abs(sppm.base_radius - 0.05) < 1e-7
    _, vcm = host_scene.load_scene(os.path.join(scenes, "mixed_vcm.json"))
    assert vcm.enable_vm == 1 and abs(vcm.radius_factor - 1.0) < 1e-7 and abs(vcm.base_radius - 0.03) < 1e-7
