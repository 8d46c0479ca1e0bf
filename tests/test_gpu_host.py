"""GPU tests of the C++ host layer: a Lumen JSON scene loaded by liblgb_host.so and rendered headless by
the Integrator mirror (init, create_accel, render/update per frame) against the oracle, and the lgb_render
command line writing the same film to a PFM file."""
import os
import subprocess

import numpy as np
import pytest

from lumen_gb300 import abi, build

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
SCENE = os.path.join(HERE, "golden", "scenes", "mixed.json")


def read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return data[::-1].reshape(-1, 3)  # rows bottom-up in the file


@pytest.fixture(scope="module")
def host():
    from lumen_gb300 import host_scene
    if not os.path.exists(host_scene.HOST_LIB):
        build.build_library()
    return host_scene


def test_headless_render_matches_oracle(host, oracle):
    from lumen_gb300.scene import camera_lookat
    w, h, spp = 40, 30, 3
    film = host.render_path(SCENE, w, h, spp)
    arrays, info = host.load_scene(SCENE)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    osc = oracle.scene(arrays)
    osc._params_sky = tuple(info.sky_col)
    want = np.zeros((w * h, 4), np.float32)
    import ctypes as C
    import oracle_lib
    p = osc._params(int(info.path_length), w, h, 0, sky=tuple(info.sky_col))
    iv = np.ascontiguousarray(np.array(cam.inv_view[:], np.float32))
    ip = np.ascontiguousarray(np.array(cam.inv_projection[:], np.float32))
    osc.ora.lib.orc_render_film(osc.h, oracle_lib._p(iv), oracle_lib._p(ip), C.byref(p), 0, spp, oracle_lib._p(want),
                                0, os.cpu_count() or 1)
    ok = np.abs(film[:, :3] - want[:, :3]) <= 1e-4 * np.maximum(np.abs(want[:, :3]), 1e-6) + 1e-7
    frac = ok.all(axis=1).mean()
    assert frac >= 0.97, f"only {frac:.3f} of pixels agree"
    assert film[:, :3].mean() > 0.01


def test_cli_writes_the_same_film(host, tmp_path):
    out = tmp_path / "frame.pfm"
    exe = os.path.join(os.path.dirname(abi.LIB_PATH), "lgb_render")
    r = subprocess.run([exe, SCENE, "40", "30", "3", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    img = read_pfm(str(out))
    film = host.render_path(SCENE, 40, 30, 3)
    np.testing.assert_array_equal(img, film[:, :3])
    bad = subprocess.run([exe, str(tmp_path / "none.json"), "8", "8", "1", str(out)], capture_output=True, text=True)
    assert bad.returncode == 1 and "cannot open" in bad.stderr


def _hash32(x):
    x &= 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def test_headless_vcm_matches_direct_iterations(host):
    """A scene whose integrator is "vcm" renders through the GpuVCM mirror (radius schedule, bounds, seeds) exactly
    as direct lgb_vcm_iteration calls with the same parameters; splats are float atomics, so pixels agree to
    rounding."""
    from lumen_gb300.scene import Context, GpuScene, camera_lookat, vcm_params, vcm_radius
    scene = os.path.join(HERE, "golden", "scenes", "mixed_vcm.json")
    w, h, n = 40, 30, 4
    film = host.render_path(scene, w, h, n)
    arrays, info = host.load_scene(scene)
    ctx = Context(0)
    sc = GpuScene(ctx, arrays)
    sc.build()
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    direct = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    for f in range(n):
        ls, es = _hash32(2 * f + 1), _hash32(2 * f + 2)
        p = vcm_params(arrays, int(info.path_length), vcm_radius(float(info.radius), 1.0, f), ls, es, f,
                       sky=tuple(info.sky_col))
        p.scene_min[:] = list(info.bbox_min)
        p.scene_max[:] = list(info.bbox_max)
        sc.vcm_iteration(cam, p, direct)
    sc.sync()
    got = direct.cpu().numpy()
    ok = np.abs(film[:, :3] - got[:, :3]) <= 1e-4 * np.maximum(np.abs(got[:, :3]), 1e-6) + 1e-6
    assert ok.all(axis=1).mean() >= 0.99
    assert film[:, :3].mean() > 0.01


def test_headless_sppm_matches_direct_iterations(host):
    """A scene whose integrator is "sppm" renders through the GpuSPPM mirror (base radius, seeds) as direct
    lgb_sppm_iteration calls with the same parameters; the host layer sets its camera up through its own
    Integrator::init, so pixels agree to rounding."""
    from lumen_gb300.scene import Context, GpuScene, camera_lookat, sppm_params
    scene = os.path.join(HERE, "golden", "scenes", "mixed_sppm.json")
    w, h, n = 40, 30, 4
    film = host.render_path(scene, w, h, n)
    arrays, info = host.load_scene(scene)
    ctx = Context(0)
    sc = GpuScene(ctx, arrays)
    sc.build()
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    direct = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    for f in range(n):
        sc.sppm_iteration(cam, sppm_params(arrays, int(info.path_length), float(info.base_radius),
                                           _hash32(2 * f + 1), f, sky=tuple(info.sky_col)), direct)
    sc.sync()
    got = direct.cpu().numpy()
    ok = np.abs(film[:, :3] - got[:, :3]) <= 1e-4 * np.maximum(np.abs(got[:, :3]), 1e-6) + 1e-6
    assert ok.all(axis=1).mean() >= 0.99, (ok.all(axis=1).mean(), np.abs(film - got).max())
    np.testing.assert_allclose(film[:, :3].mean(0), got[:, :3].mean(0), rtol=1e-3)
    assert film[:, :3].mean() > 0.01


def test_headless_restir_matches_direct_iterations(host):
    """A scene whose integrator is "restir" renders through the GpuReSTIR mirror (reuse off for the first frame, on
    afterwards, the previous camera, seeds) as direct lgb_restir_di_iteration calls with the same parameters."""
    from lumen_gb300.scene import Context, GpuScene, camera_lookat, restir_params
    scene = os.path.join(HERE, "golden", "scenes", "mixed_restir.json")
    w, h, n = 40, 30, 4
    film = host.render_path(scene, w, h, n)
    arrays, info = host.load_scene(scene)
    assert len(arrays.lights) == 1
    ctx = Context(0)
    sc = GpuScene(ctx, arrays)
    sc.build()
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    direct = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    for f in range(n):
        sc.restir_di_iteration(cam, restir_params(arrays, _hash32(2 * f + 1), f, 1 if f > 0 else 0), direct,
                               prev_cam=cam)
    sc.sync()
    got = direct.cpu().numpy()
    ok = np.abs(film[:, :3] - got[:, :3]) <= 1e-4 * np.maximum(np.abs(got[:, :3]), 1e-6) + 1e-6
    assert ok.all(axis=1).mean() >= 0.97, (ok.all(axis=1).mean(), np.abs(film - got).max())
    assert film[:, :3].mean() > 0.0


def test_headless_bdpt_matches_direct_iterations(host):
    """A scene whose integrator is "bdpt" renders through the GpuBDPT mirror (path length, seeds, frame numbers)
    as direct lgb_bdpt_iteration calls with the same parameters (splat atomics aside, pixels agree to rounding)."""
    from lumen_gb300.scene import Context, GpuScene, bdpt_params, camera_lookat
    scene = os.path.join(HERE, "golden", "scenes", "mixed_bdpt.json")
    w, h, n = 40, 30, 4
    film = host.render_path(scene, w, h, n)
    arrays, info = host.load_scene(scene)
    ctx = Context(0)
    sc = GpuScene(ctx, arrays)
    sc.build()
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    direct = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    for f in range(n):
        sc.bdpt_iteration(cam, bdpt_params(arrays, int(info.path_length), _hash32(2 * f + 1), f,
                                           sky=tuple(info.sky_col)), direct)
    sc.sync()
    got = direct.cpu().numpy()
    ok = np.abs(film[:, :3] - got[:, :3]) <= 1e-4 * np.maximum(np.abs(got[:, :3]), 1e-6) + 1e-6
    assert ok.all(axis=1).mean() >= 0.97, (ok.all(axis=1).mean(), np.abs(film - got).max())
    np.testing.assert_allclose(film[:, :3].mean(0), got[:, :3].mean(0), rtol=1e-3)
    assert film[:, :3].mean() > 0.0


MTS_SCENE = os.path.join(HERE, "golden", "scenes", "mitsuba", "scene.xml")


def test_mitsuba_scene_renders_like_the_oracle(host, oracle):
    """A Mitsuba XML scene (every BSDF mapping, transformed OBJ shapes, a lookat sensor, a nested area emitter)
    loaded by the host layer and rendered headless, against the oracle on the loaded arrays and camera."""
    import ctypes as C
    import oracle_lib
    from lumen_gb300.scene import camera_from_matrix
    w, h, spp = 48, 36, 2
    film = host.render_path(MTS_SCENE, w, h, spp)
    arrays, info = host.load_scene(MTS_SCENE)
    assert info.cam_use_matrix == 1
    cam = camera_from_matrix(list(info.cam_matrix), info.fov, w, h)
    osc = oracle.scene(arrays)
    want = np.zeros((w * h, 4), np.float32)
    p = osc._params(int(info.path_length), w, h, 0, sky=tuple(info.sky_col))
    iv = np.ascontiguousarray(np.array(cam.inv_view[:], np.float32))
    ip = np.ascontiguousarray(np.array(cam.inv_projection[:], np.float32))
    osc.ora.lib.orc_render_film(osc.h, oracle_lib._p(iv), oracle_lib._p(ip), C.byref(p), 0, spp, oracle_lib._p(want),
                                0, os.cpu_count() or 1)
    ok = np.abs(film[:, :3] - want[:, :3]) <= 1e-4 * np.maximum(np.abs(want[:, :3]), 1e-6) + 1e-7
    frac = ok.all(axis=1).mean()
    assert frac >= 0.97, f"only {frac:.3f} of pixels agree"
    assert film[:, :3].mean() > 0.01


def test_mitsuba_sunsky_scene_is_refused(host):
    with pytest.raises(abi.LgbError) as e:
        host.render_path(os.path.join(HERE, "golden", "scenes", "mitsuba", "sunsky.xml"), 16, 16, 1)
    assert e.value.status == 6  # LGB_ERR_UNSUPPORTED: the directional sun needs the atmosphere model
