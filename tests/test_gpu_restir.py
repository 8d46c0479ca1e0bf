"""GPU tests of ReSTIR DI (lgb_restir_di_iteration) against the CPU oracle's restatement of Lumen's ReSTIR DI.

Every pass is per pixel and deterministic (no atomics), so films agree with the oracle pixel by pixel to rounding;
a rare branch flip (sinf / cosf of the neighbour offsets, or a visibility test on an edge) changes a few pixels,
and later frames inherit such a difference through the temporal reservoirs.
"""
import os

import numpy as np
import pytest

import parity_log

import oracle_lib
from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene, camera_forward, camera_lookat, restir_params

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


def _run_both(ctx, oracle, arrays, w, h, frames, flags=0, spot_angle=0.0, accumulate=1):
    sc = GpuScene(ctx, arrays)
    sc.build()
    osc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    st = oracle_lib.restir_state(w, h)
    for f in range(frames):
        p = restir_params(arrays, 31, f, 1 if f > 0 else 0, accumulate, spot_angle=spot_angle, flags=flags)
        sc.restir_di_iteration(cam, p, film, prev_cam=cam)
        op = oracle_lib.RestirParams()
        for name in ("num_lights", "light_triangle_count", "seed", "frame_num", "do_spatiotemporal",
                     "enable_accumulation", "spot_angle", "flags"):
            setattr(op, name, getattr(p, name))
        oracle_lib.restir_iteration(osc, cam, view, proj, op, st)
    sc.sync()
    got = film.cpu().numpy()
    sc.close()
    return got, st["film"]


@pytest.mark.parametrize("flags", [0, abi.RESTIR_SPATIAL_COUNT_FIX])
def test_restir_matches_oracle_cornell(ctx, oracle, flags):
    cb = procedural.cornell_box()
    got, want = _run_both(ctx, oracle, cb, 48, 48, 1, flags)
    assert (got[:, 3] == 1.0).all() and not np.isnan(got).any()
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    got6, want6 = _run_both(ctx, oracle, cb, 48, 48, 6, flags)
    assert close_fraction(got6[:, :3], want6[:, :3]) >= 0.99
    np.testing.assert_allclose(got6[:, :3].mean(0), want6[:, :3].mean(0), rtol=0.03)


def test_restir_spot_light_matches_oracle(ctx, oracle):
    arrays = procedural.vcm_scene(100, 40)
    got, want = _run_both(ctx, oracle, arrays, 48, 48, 3, abi.RESTIR_SPATIAL_COUNT_FIX, spot_angle=20.0)
    assert got[:, :3].mean() > 0.0
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.03)


def test_restir_error_paths(ctx):
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 16, 16)
    film = torch.zeros((256, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(abi.LgbError):
        sc.restir_di_iteration(cam, restir_params(cb, 1, 0, 0), film)  # no BVH
    sc.build()
    other = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 8, 8)
    with pytest.raises(abi.LgbError):
        sc.restir_di_iteration(cam, restir_params(cb, 1, 0, 0), film, prev_cam=other)  # size mismatch
    for bad in (dict(num_lights=0), dict(light_triangle_count=0), dict(spot_angle=-3.0), dict(dir_light_idx=1)):
        p = restir_params(cb, 1, 0, 0)
        for k, v in bad.items():
            setattr(p, k, v)
        with pytest.raises(abi.LgbError):
            sc.restir_di_iteration(cam, p, film)
    sc.restir_di_iteration(cam, restir_params(cb, 1, 0, 0), film)
    sc.sync()
    sc.close()
