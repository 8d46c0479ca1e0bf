"""GPU tests of SPPM (lgb_sppm_iteration) against the CPU oracle's restatement of Lumen's SPPM integrator.

The eye pass, grid bounds, light pass, photon table, gather and composite are all deterministic (the table is
built by sort and scan; nothing is summed with atomics), so films agree with the oracle pixel by pixel to
rounding; a rare branch flip (CUDA's and glibc's sinf / cosf differ by an ulp) changes a few pixels.
"""
import os

import numpy as np
import pytest

import parity_log

import oracle_lib
from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene, camera_lookat, sppm_params

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


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


def _run_both(ctx, oracle, arrays, w, h, frames, depth, base_radius=0.03, spot_angle=0.0, sky=(0.0, 0.0, 0.0)):
    sc = GpuScene(ctx, arrays)
    sc.build()
    osc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    st = oracle_lib.sppm_state(w, h, depth)
    for f in range(frames):
        p = sppm_params(arrays, depth, base_radius, 4242, f, sky=sky, spot_angle=spot_angle)
        sc.sppm_iteration(cam, p, film)
        op = oracle_lib.SppmParams()
        for name in ("max_depth", "num_lights", "light_triangle_count", "base_radius", "seed", "frame_num",
                     "spot_angle"):
            setattr(op, name, getattr(p, name))
        op.sky_col[:] = list(p.sky_col)
        oracle_lib.sppm_iteration(osc, cam, op, st)
    sc.sync()
    got = film.cpu().numpy()
    sc.close()
    return got, st["film"]


def test_sppm_matches_oracle_cornell(ctx, oracle):
    cb = procedural.cornell_box()
    got, want = _run_both(ctx, oracle, cb, 48, 48, 1, 6)
    assert (got[:, 3] == 1.0).all() and not np.isnan(got).any()
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    got8, want8 = _run_both(ctx, oracle, cb, 48, 48, 8, 6, sky=(0.2, 0.3, 0.4))
    assert close_fraction(got8[:, :3], want8[:, :3]) >= 0.99
    np.testing.assert_allclose(got8[:, :3].mean(0), want8[:, :3].mean(0), rtol=0.01)


def test_sppm_caustics_scene_matches_oracle(ctx, oracle):
    arrays = procedural.vcm_scene(100, 40)
    got, want = _run_both(ctx, oracle, arrays, 64, 64, 4, 10, base_radius=0.05, spot_angle=20.0)
    assert not np.isnan(got).any() and got[:, :3].mean() > 0.0
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.02)


def test_sppm_restarts_at_frame_zero(ctx):
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    sc.build()
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 32, 32)
    a = torch.zeros((32 * 32, 4), dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 9, 0), a)
    for f in range(1, 4):
        sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 9, f), b)
    sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 9, 0), b)  # frame 0 clears the per-pixel state
    sc.sync()
    assert torch.equal(a, b)
    sc.close()


def test_sppm_error_paths(ctx):
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 16, 16)
    film = torch.zeros((256, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(abi.LgbError):
        sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 1, 0), film)  # no BVH
    sc.build()
    for bad in (dict(max_depth=0), dict(num_lights=0), dict(base_radius=float("nan")), dict(spot_angle=95.0),
                dict(dir_light_idx=0)):
        p = sppm_params(cb, 6, 0.03, 1, 0)
        for k, v in bad.items():
            setattr(p, k, v)
        with pytest.raises(abi.LgbError):
            sc.sppm_iteration(cam, p, film)
    sc.sppm_iteration(cam, sppm_params(cb, 6, 0.03, 1, 0), film)
    sc.sync()
    sc.close()
