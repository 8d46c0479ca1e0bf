"""CPU tests of the Mitsuba XML reader of the host layer (LumenScene::load_mitsuba_scene semantics,
LumenScene.cpp:514-690 over MitsubaParser.cpp:5-147): version-0 camelCase names, BSDF mappings, shape
transforms, the sensor's camera with Lumen's Euler-angle round trip, the sun-sky emitter, and load errors."""
import math
import os

import numpy as np
import pytest

from lumen_gb300 import abi, build

HERE = os.path.dirname(os.path.abspath(__file__))
MTS = os.path.join(HERE, "golden", "scenes", "mitsuba")


@pytest.fixture(scope="module")
def host():
    from lumen_gb300 import host_scene
    if not os.path.exists(host_scene.HOST_LIB):
        build.build_library()
    return host_scene


@pytest.fixture(scope="module")
def loaded(host):
    return host.load_scene(os.path.join(MTS, "scene.xml"))


def _obj_corners(name):
    """Vertices of an OBJ file in face-corner order, fans split as the loader splits them."""
    v, out = [], []
    for line in open(os.path.join(MTS, name)):
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            v.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            idx = [int(c.split("/")[0]) - 1 for c in t[1:]]
            for k in range(2, len(idx)):
                out += [v[idx[0]], v[idx[k - 1]], v[idx[k]]]
    return np.array(out, np.float64)


def _rot(axis, deg):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    t = math.radians(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(4)
    R[:3, :3] = np.eye(3) + math.sin(t) * K + (1 - math.cos(t)) * K @ K
    return R


def _scale(x, y, z):
    return np.diag([x, y, z, 1.0])


def _translate(x, y, z):
    T = np.eye(4)
    T[:3, 3] = [x, y, z]
    return T


def test_meshes_and_transforms(loaded):
    arrays, info = loaded
    assert len(arrays.meshes) == 6
    assert list(arrays.meshes["tri_count"]) == [2, 2, 12, 12, 12, 2]  # the cube's two OBJ groups are one mesh
    xforms = [_scale(2, 2, 2),
              _translate(0, 1.5, -2) @ _rot((1, 0, 0), 90) @ _scale(2, 1, 1.5),
              _translate(-0.6, 0.3, -0.5) @ _rot((0, 1, 0), 30) @ _scale(0.6, 0.6, 0.6),
              np.array([[0.5, 0, 0, 0.6], [0, 0.5, 0, 0.25], [0, 0, 0.5, -0.1], [0, 0, 0, 1]]),
              _translate(0.1, 0.1, 0.6) @ _scale(0.3, 0.2, 0.3),
              _translate(0, 1.9, -0.4) @ _rot((1, 0, 0), 180) @ _scale(0.35, 0.35, 0.35)]
    files = ["quad.obj", "quad.obj", "cube.obj", "cube.obj", "cube.obj", "quad.obj"]
    for m, X, f in zip(arrays.meshes, xforms, files):
        raw = _obj_corners(f)
        want = (X @ np.concatenate([raw, np.ones((len(raw), 1))], 1).T).T[:, :3]
        got = arrays.positions[m["vertex_offset"]:m["vertex_offset"] + 3 * m["tri_count"]]
        np.testing.assert_allclose(got, want, atol=2e-6)
        idx = arrays.indices[m["index_offset"]:m["index_offset"] + 3 * m["tri_count"]]
        assert list(idx) == list(range(3 * m["tri_count"]))
    # normals follow the inverse transpose: the lamp quad faces down after its 180 degree turn
    lamp = arrays.meshes[5]
    np.testing.assert_allclose(arrays.normals[lamp["vertex_offset"]], [0, -1, 0], atol=1e-6)
    n = arrays.normals[arrays.meshes[1]["vertex_offset"]]  # the back wall, quad normal +y turned to +z
    np.testing.assert_allclose(n, [0, 0, 1], atol=1e-6)


def test_bsdf_mappings(loaded):
    arrays, _ = loaded
    m = arrays.materials
    assert list(m["bsdf_type"][:6]) == [abi.BSDF_DIFFUSE, abi.BSDF_PRINCIPLED, abi.BSDF_CONDUCTOR,
                                        abi.BSDF_PRINCIPLED, abi.BSDF_GLASS, abi.BSDF_DIFFUSE]
    np.testing.assert_allclose(m["albedo"][0], [0.7, 0.7, 0.7])  # unwrapped from the twosided BSDF
    # roughplastic: diffuseReflectance is the albedo, roughness sqrt(alpha), the plastic principled parameters
    np.testing.assert_allclose(m["albedo"][1], [0.2, 0.5, 0.8])
    np.testing.assert_allclose(m["roughness"][1], 0.3, rtol=1e-6)
    np.testing.assert_allclose(m["ior"][1], 1.45, rtol=1e-6)
    assert m["metallic"][1] == 1.0 and m["spec_trans"][1] == 0.5 and m["thin"][1] == 1
    np.testing.assert_allclose(m["subsurface"][1], 0.1, rtol=1e-6)
    assert m["bsdf_props"][1] == (abi.FLAG_DIFFUSE | abi.FLAG_REFLECTION | abi.FLAG_TRANSMISSION | abi.FLAG_GLOSSY)
    # roughconductor: specularReflectance through reflectance_to_conductor_eta_k, roughness sqrt(0.04)
    r = np.array([0.9, 0.7, 0.3], np.float32)
    np.testing.assert_allclose(m["k"][2], 2 * np.sqrt(r) / np.sqrt(np.maximum(1 - r, 0.001)), rtol=1e-6)
    np.testing.assert_allclose(m["albedo"][2], [1, 1, 1])
    np.testing.assert_allclose(m["roughness"][2], 0.2, rtol=1e-6)
    assert m["bsdf_props"][2] == abi.FLAG_REFLECTION | abi.FLAG_GLOSSY
    # dielectric -> principled with full specular transmission; glass keeps its own type
    assert m["spec_trans"][3] == 1.0 and m["metallic"][3] == 0.0
    assert m["bsdf_props"][3] == (abi.FLAG_DIFFUSE | abi.FLAG_REFLECTION | abi.FLAG_TRANSMISSION | abi.FLAG_SPECULAR)
    np.testing.assert_allclose(m["ior"][4], 1.33, rtol=1e-6)
    assert m["bsdf_props"][4] == abi.FLAG_SPECULAR | abi.FLAG_TRANSMISSION
    # make_default_principled: clearcoat_gloss and sheen_tint are zero, not the JSON defaults
    assert (m["clearcoat_gloss"][:6] == 0).all() and (m["sheen_tint"][:6] == 0).all()


def test_area_emitter_and_lights(loaded):
    arrays, info = loaded
    # the lamp shape's nested area emitter: an emissive copy of its material, one area light of 2 triangles
    assert len(arrays.materials) == 7 and arrays.meshes["material_index"][5] == 6
    np.testing.assert_allclose(arrays.materials["emissive_factor"][6], [12, 11, 10])
    np.testing.assert_allclose(arrays.materials["albedo"][6], [0.8, 0.8, 0.8])
    assert len(arrays.lights) == 1 and arrays.lights["light_flags"][0] == abi.LIGHT_AREA | abi.LIGHT_FINITE
    assert arrays.lights["prim_mesh_idx"][0] == 5 and info.light_triangle_count == 2
    assert info.dir_light_idx == 0xFFFFFFFF and info.path_length == 5


def _euler_round_trip(R):
    """The camera rotation Lumen renders with: R = Rx(a) Ry(b) Rz(c) decomposed, then Ry(b) Rx(a) Rz(c)."""
    a = math.atan2(-R[1, 2], R[2, 2])
    b = math.asin(max(-1.0, min(1.0, R[0, 2])))
    c = math.atan2(-R[0, 1], R[0, 0])
    return _rot((0, 1, 0), math.degrees(b))[:3, :3] @ _rot((1, 0, 0), math.degrees(a))[:3, :3] @ \
        _rot((0, 0, 1), math.degrees(c))[:3, :3]


def _lookat(origin, target, up):
    o, t, u = (np.asarray(x, np.float64) for x in (origin, target, up))
    f = (t - o) / np.linalg.norm(t - o)
    left = np.cross(u, f)
    left /= np.linalg.norm(left)
    nu = np.cross(f, left)
    return np.stack([left, nu / np.linalg.norm(nu), f], 1)


def test_sensor_camera(loaded):
    arrays, info = loaded
    assert info.cam_use_matrix == 1
    np.testing.assert_allclose(info.fov, 40.0)  # Lumen halves the sensor's fov (LumenScene.cpp:530)
    C = np.array(info.cam_matrix, np.float64).reshape(4, 4).T  # column-major
    np.testing.assert_allclose(C[:3, 3], [0, 1, 3], atol=1e-6)
    np.testing.assert_allclose(C[3], [0, 0, 0, 1])
    R = _lookat((0, 1, 3), (0.3, 1.2, 6), (0, 1, 0))
    np.testing.assert_allclose(C[:3, :3], _euler_round_trip(R), atol=1e-6)
    np.testing.assert_allclose(C[:3, :3] @ C[:3, :3].T, np.eye(3), atol=1e-6)
    # the round trip reorders the rotations: with both pitch and yaw it is not the sensor's own rotation
    assert np.abs(C[:3, :3] - R).max() > 1e-3


def test_round_trip_is_exact_for_a_single_axis(host, tmp_path):
    for target in ("0, 1, 6", "2, 1, 6", "0, 3, 6"):  # straight, yaw only, pitch only
        (tmp_path / "quad.obj").write_text(open(os.path.join(MTS, "quad.obj")).read())
        (tmp_path / "s.xml").write_text(f"""<scene version="0.5.0"><sensor type="perspective">
            <float name="fov" value="60"/><transform name="toWorld">
            <lookat origin="0, 1, 3" target="{target}" up="0, 1, 0"/></transform></sensor>
            <bsdf type="diffuse" id="w"/><shape type="obj"><string name="filename" value="quad.obj"/>
            <ref id="w"/></shape></scene>""")
        _, info = host.load_scene(str(tmp_path / "s.xml"))
        C = np.array(info.cam_matrix, np.float64).reshape(4, 4).T
        t = np.array([float(x) for x in target.split(",")])
        np.testing.assert_allclose(C[:3, :3], _lookat((0, 1, 3), t, (0, 1, 0)), atol=1e-6)


def test_sunsky_loads_as_directional_light(host):
    arrays, info = host.load_scene(os.path.join(MTS, "sunsky.xml"))
    assert len(arrays.lights) == 1
    assert arrays.lights["light_flags"][0] == abi.LIGHT_DIRECTIONAL | abi.LIGHT_DELTA
    np.testing.assert_allclose(arrays.lights["pos"][0], [0.3, 1, 0.2])
    np.testing.assert_allclose(arrays.lights["L"][0], 100 * 0.01 * np.array([0.98, 0.82, 0.30]), rtol=1e-6)
    np.testing.assert_allclose(list(info.sky_col), [0.053, 0.08, 0.092], rtol=1e-6)
    assert info.dir_light_idx == 0 and info.light_triangle_count == 1
    np.testing.assert_allclose(arrays.materials["albedo"][0], [1, 1, 1])  # no reflectance: Lumen's default


@pytest.mark.parametrize("body,msg", [
    ('<bsdf type="diffuse" id="w"/><shape type="obj"><string name="filename" value="quad.obj"/>'
     '<ref id="missing"/></shape>', "names no object"),
    ('<shape type="obj"><string name="filename" value="quad.obj"/></shape>', "names no BSDF"),
    ('<bsdf type="diffuse" id="w"/><shape type="sphere"><ref id="w"/><string name="filename" value="x.obj"/>'
     '</shape>', "OBJ only"),
    ('<emitter type="point"><point name="position" x="0" y="1" z="0"/></emitter>', "emitter type 'point'"),
    ('<bsdf type="diffuse" id="w"><rgb name="reflectance" value="1 2"/></bsdf>', "1 or 3 values"),
    ('<bsdf type="diffuse" id="w">', "</scene> closes <bsdf>"),
    ('<bsdf type="diffuse" id="w"></bsdfx>', "</bsdfx> closes <bsdf>"),
    ('<include filename="other.xml"/>', "unsupported element"),
])
def test_load_errors(host, tmp_path, body, msg):
    (tmp_path / "quad.obj").write_text(open(os.path.join(MTS, "quad.obj")).read())
    (tmp_path / "bad.xml").write_text(f'<?xml version="1.0"?><scene version="0.5.0">{body}</scene>')
    with pytest.raises(abi.LgbError) as e:
        host.load_scene(str(tmp_path / "bad.xml"))
    assert msg in str(e.value)


def test_version_2_keeps_names(host, tmp_path):
    """From version 2 on, Mitsuba names are snake_case already and are not converted: a camelCase name is then
    a different property, as tinyparser-mitsuba reads it (the conversion applies to version-0 files only)."""
    (tmp_path / "quad.obj").write_text(open(os.path.join(MTS, "quad.obj")).read())
    (tmp_path / "v2.xml").write_text('<scene version="2.0.0"><integrator type="path">'
                                     '<integer name="max_depth" value="3"/></integrator>'
                                     '<bsdf type="roughconductor" id="m"><float name="alpha" value="0.25"/>'
                                     '<float name="intIOR" value="9"/></bsdf>'
                                     '<shape type="obj"><string name="filename" value="quad.obj"/>'
                                     '<ref id="m"/></shape></scene>')
    arrays, info = host.load_scene(str(tmp_path / "v2.xml"))
    assert info.path_length == 3
    np.testing.assert_allclose(arrays.materials["roughness"][0], 0.5)
    assert arrays.materials["ior"][0] == 0.0  # conductors do not take an IOR; intIOR is not int_ior in version 2
