"""GPU tests of BDPT (lgb_bdpt_iteration) against the CPU oracle's restatement of Lumen's BDPT integrator.

Subpaths, strategies, MIS weights and the film are deterministic; only the light-tracing (t = 1) splats are summed
with float atomics on the GPU (in pixel order on the CPU), so films agree with the oracle pixel by pixel to
rounding, and a rare branch flip (CUDA's and glibc's sinf / cosf differ by an ulp) changes a few pixels.
Scenes: the Cornell box (diffuse, area light), the caustics scene (dielectric torus, spot light: a delta light),
and a mixed scene with every BSDF type (conductor, dielectric, principled) under a spot light.
"""
import os

import numpy as np
import pytest

import parity_log

import oracle_lib
from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene, bdpt_params, camera_forward, camera_lookat

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ctx():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return Context(0)


def close_fraction(a, b, rtol=1e-4, atol=1e-7):
    ok = np.abs(a - b) <= rtol * np.maximum(np.abs(b), 1e-6) + atol
    frac = ok.all(axis=1).mean()
    parity_log.record(frac, rtol)
    return frac


def _run_both(ctx, oracle, arrays, w, h, frames, depth, spot_angle=0.0, seed=4242):
    sc = GpuScene(ctx, arrays)
    sc.build()
    osc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    st = oracle_lib.bdpt_state(w, h)
    for f in range(frames):
        p = bdpt_params(arrays, depth, seed, f, spot_angle=spot_angle)
        sc.bdpt_iteration(cam, p, film)
        op = oracle_lib.BdptParams()
        for name in ("max_depth", "num_lights", "light_triangle_count", "seed", "frame_num", "spot_angle"):
            setattr(op, name, getattr(p, name))
        oracle_lib.bdpt_iteration(osc, cam, view, proj, op, st)
    sc.sync()
    got = film.cpu().numpy()
    sc.close()
    return got, st["film"]


def test_bdpt_matches_oracle_cornell(ctx, oracle):
    cb = procedural.cornell_box()
    got, want = _run_both(ctx, oracle, cb, 48, 40, 1, 6)
    assert (got[:, 3] == 1.0).all() and not np.isnan(got).any()
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.005)
    got4, want4 = _run_both(ctx, oracle, cb, 48, 40, 4, 6)
    assert close_fraction(got4[:, :3], want4[:, :3]) >= 0.99
    np.testing.assert_allclose(got4[:, :3].mean(0), want4[:, :3].mean(0), rtol=0.005)


@pytest.mark.parametrize("depth", [1, 2, 3, 10])
def test_bdpt_path_lengths_match_oracle(ctx, oracle, depth):
    """max_depth 1 leaves only (s, t) = (0, 2) (the emitter seen directly); 2 and 3 add the first strategies
    of each kind; 10 runs long subpaths (64 strategies per pixel)."""
    cb = procedural.cornell_box()
    got, want = _run_both(ctx, oracle, cb, 32, 32, 2, depth)
    assert not np.isnan(got).any()
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.01)


def test_bdpt_caustics_scene_matches_oracle(ctx, oracle):
    """A spot light is a delta light: its vertex 0 has pdf_fwd = 0 and is skipped by the MIS sums."""
    arrays = procedural.vcm_scene(100, 40)
    got, want = _run_both(ctx, oracle, arrays, 64, 64, 2, 8, spot_angle=20.0)
    assert not np.isnan(got).any() and got[:, :3].mean() > 0.0
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.02)


def test_bdpt_mixed_materials_match_oracle(ctx, oracle):
    from lumen_gb300 import host_scene
    if not os.path.exists(host_scene.HOST_LIB):
        build.build_library()
    arrays, _ = host_scene.load_scene(os.path.join(HERE, "golden", "scenes", "mixed_sppm.json"))
    got, want = _run_both(ctx, oracle, arrays, 40, 30, 2, 5)
    assert not np.isnan(got).any() and got[:, :3].mean() > 0.0
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.02)


def test_bdpt_frame_zero_restarts_and_is_deterministic(ctx):
    """Frame 0 writes the film outright; the same seed and frame give the same film up to the atomics' order."""
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    sc.build()
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 32, 32)
    a = torch.zeros((32 * 32, 4), dtype=torch.float32, device="cuda")
    b = torch.full_like(a, 7.0)
    sc.bdpt_iteration(cam, bdpt_params(cb, 6, 9, 0), a)
    for f in range(1, 3):
        sc.bdpt_iteration(cam, bdpt_params(cb, 6, 9, f), b)
    sc.bdpt_iteration(cam, bdpt_params(cb, 6, 9, 0), b)
    sc.sync()
    np.testing.assert_allclose(a.cpu().numpy(), b.cpu().numpy(), rtol=1e-5, atol=1e-6)
    sc.close()


def test_bdpt_error_paths(ctx):
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 16, 16)
    film = torch.zeros((256, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(abi.LgbError):
        sc.bdpt_iteration(cam, bdpt_params(cb, 6, 1, 0), film)  # no BVH
    sc.build()
    for bad in (dict(max_depth=0), dict(max_depth=33), dict(num_lights=0), dict(light_triangle_count=0),
                dict(spot_angle=95.0), dict(dir_light_idx=0)):
        p = bdpt_params(cb, 6, 1, 0)
        for k, v in bad.items():
            setattr(p, k, v)
        with pytest.raises(abi.LgbError):
            sc.bdpt_iteration(cam, p, film)
    sc.bdpt_iteration(cam, bdpt_params(cb, 6, 1, 0), film)
    sc.sync()
    assert not torch.isnan(film).any()
    sc.close()
