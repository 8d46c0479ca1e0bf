"""GPU tests of VCM (lgb_vcm_iteration, lgb_vcm_grid) against the CPU oracle's restatement.

  * the photon table built by radix sort and scan equals the oracle's sequentially written table bit for bit
    (same positions in, same counts and representatives out);
  * VCM iterations equal the oracle's pixel by pixel (same seeds); the light subpaths' camera splats are summed
    with float atomics on the GPU and in path order on the CPU, so pixels agree to rounding, and a rare branch
    flip (CUDA's and glibc's sinf/cosf differ by an ULP) changes a few pixels;
  * the caustics configuration (dielectric torus, spot light) with merging; the accumulate option; error paths.
"""
import os

import numpy as np
import pytest

import parity_log

from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import (Context, GpuScene, camera_forward, camera_lookat, scene_radius, vcm_grid, vcm_params,
                               vcm_radius)

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return Context(0)


def close_fraction(a, b, rtol=1e-3, atol=1e-5):
    ok = np.abs(a - b) <= rtol * np.maximum(np.abs(b), 1e-6) + atol
    frac = ok.all(axis=1).mean()
    parity_log.record(frac, rtol)
    if rtol != 1e-4:  # also the per-sample tolerance of the path tracer, for the record only
        parity_log.record((np.abs(a - b) <= 1e-4 * np.maximum(np.abs(b), 1e-6) + 1e-7).all(axis=1).mean(), 1e-4)
    return frac


def test_photon_table_is_bit_exact(ctx, oracle):
    from oracle_lib import vcm_grid as oracle_grid
    rng = np.random.default_rng(8)
    n, screen = 200_000, 128 * 128
    pos4 = np.concatenate([rng.uniform(-2.1, 2.1, (n, 3)), np.where(rng.uniform(size=(n, 1)) < 0.2, -1.0, 1.0)], 1)
    pos4[:1000, :3] = pos4[1000:2000, :3]
    pos4 = pos4.astype(np.float32)
    mn, mx, radius = (-2.0, -2.0, -2.0), (2.0, 2.0, 2.0), 0.03
    count = torch.zeros(10 * screen, dtype=torch.int32, device="cuda")
    rep = torch.zeros(10 * screen, dtype=torch.int32, device="cuda")
    vcm_grid(ctx, torch.from_numpy(pos4).cuda(), mn, mx, radius, screen, count, rep)
    want_c, want_r = oracle_grid(oracle, pos4, mn, mx, radius, screen)
    assert np.array_equal(count.cpu().numpy().view(np.uint32), want_c)
    assert np.array_equal(rep.cpu().numpy().view(np.uint32), want_r)
    assert (want_c > 1).sum() > 1000
    # an empty input gives an empty table
    vcm_grid(ctx, torch.zeros((0, 4), device="cuda"), mn, mx, radius, screen, count, rep)
    assert int(count.abs().sum()) == 0


class _DeviceArray:
    """A device buffer owned by the library, seen by torch through the CUDA array interface (no copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2}


def test_photon_table_is_bit_exact_on_caustics_light_vertices(ctx, oracle):
    """The table of one iteration of the caustics configuration (1024^2 light subpaths on the 200k-triangle
    torus, depth 10, radius 0.01 x scene radius): the oracle's sequential table built from the GPU's own light
    vertices equals the GPU's sort-and-scan table bit for bit."""
    from oracle_lib import vcm_grid as oracle_grid
    arrays = procedural.vcm_scene()
    sc = GpuScene(ctx, arrays)
    sc.build()
    w = h = 1024
    depth = 10
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    r = vcm_radius(scene_radius(arrays), 1.0, 0, 0.75)
    sc.vcm_iteration(cam, vcm_params(arrays, depth, r, 11, 12, 0, spot_angle=20.0), film)
    sc.sync()
    st = sc.vcm_state()
    assert st.screen == w * h and st.per_path == depth + 1 and st.table_size == 10 * w * h
    nv = st.screen * st.per_path
    verts = torch.as_tensor(_DeviceArray(st.vertices, (nv, 6, 4), "<f4"), device="cuda")
    counts = torch.as_tensor(_DeviceArray(st.path_counts, (st.screen,), "<i4"), device="cuda").cpu().numpy()
    pos4 = verts[:, 0, :].cpu().numpy().copy()
    used = (np.arange(nv) % st.per_path) < np.repeat(counts, st.per_path)
    pos4[:, 3] = np.where(used, 1.0, -1.0)
    got_c = torch.as_tensor(_DeviceArray(st.table_count, (st.table_size,), "<i4"), device="cuda").cpu().numpy()
    got_r = torch.as_tensor(_DeviceArray(st.table_rep, (st.table_size,), "<i4"), device="cuda").cpu().numpy()
    want_c, want_r = oracle_grid(oracle, pos4, list(st.scene_min), list(st.scene_max), st.radius, st.screen)
    assert used.sum() > 1_000_000, "the light pass stored too few vertices to exercise the table"
    assert int(want_c.sum()) == int(used.sum())
    assert np.array_equal(got_c.view(np.uint32), want_c)
    occupied = want_c > 0
    assert np.array_equal(got_r.view(np.uint32)[occupied], want_r[occupied])
    assert (want_c > 1).sum() > 1_000
    sc.close()


def _run_both(ctx, oracle, arrays, w, h, iters, depth, flags=0, use_vm=1, alpha=2.0 / 3.0, factor=1.0, spot_angle=0.0):
    from oracle_lib import VcmParams
    sc = GpuScene(ctx, arrays)
    sc.build()
    osc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    st = osc.vcm_state(w, h, depth)
    R = scene_radius(arrays)
    for it in range(iters):
        r = vcm_radius(R, factor, it, alpha)
        p = vcm_params(arrays, depth, r, 1000 + it, 5000 + it, it, use_vm=use_vm, flags=flags, spot_angle=spot_angle)
        sc.vcm_iteration(cam, p, film)
        op = VcmParams()
        for name in ("max_depth", "num_lights", "light_triangle_count", "radius", "use_vm", "use_vc", "light_seed",
                     "eye_seed", "frame_num", "flags", "spot_angle"):
            setattr(op, name, getattr(p, name))
        op.sky_col[:] = list(p.sky_col)
        op.scene_min[:] = list(p.scene_min)
        op.scene_max[:] = list(p.scene_max)
        osc.vcm_iteration(cam, view, proj, op, st)
    sc.sync()
    got = film.cpu().numpy()
    sc.close()
    return got, st["film"]


def test_iteration_matches_oracle_cornell(ctx, oracle):
    cb = procedural.cornell_box()
    got, want = _run_both(ctx, oracle, cb, 48, 48, 1, 8)
    frac = close_fraction(got[:, :3], want[:, :3])
    assert frac >= 0.99, f"only {frac:.4f} of pixels agree"
    # at the path tracer's per-sample tolerance too: only the order of the float splat sums differs
    assert close_fraction(got[:, :3], want[:, :3], rtol=1e-4, atol=1e-7) >= 0.99
    assert (got[:, 3] == 1.0).all()
    got8, want8 = _run_both(ctx, oracle, cb, 48, 48, 8, 8)
    np.testing.assert_allclose(got8[:, :3].mean(0), want8[:, :3].mean(0), rtol=0.01)
    assert close_fraction(got8[:, :3], want8[:, :3]) >= 0.99


@pytest.mark.parametrize("spot_angle", [0.0, 20.0])
def test_caustics_scene_with_merging_matches_oracle(ctx, oracle, spot_angle):
    arrays = procedural.vcm_scene(100, 40)
    got, want = _run_both(ctx, oracle, arrays, 64, 64, 4, 10, alpha=0.75, spot_angle=spot_angle)
    assert not np.isnan(got).any()
    frac = close_fraction(got[:, :3], want[:, :3])
    assert frac >= 0.99, f"only {frac:.4f} of pixels agree"
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.02)
    assert got[:, :3].mean() > 0.0


def test_caustics_configuration_matches_oracle(ctx, oracle):
    """The caustics configuration itself (200k-triangle dielectric torus, 20 degree spot, depth 10, alpha 0.75)
    at 96^2: pixel by pixel against the oracle over four iterations with merging."""
    arrays = procedural.vcm_scene()
    got, want = _run_both(ctx, oracle, arrays, 96, 96, 4, 10, alpha=0.75, spot_angle=20.0)
    assert not np.isnan(got).any()
    frac = close_fraction(got[:, :3], want[:, :3])
    assert frac >= 0.99, f"only {frac:.4f} of pixels agree"
    assert close_fraction(got[:, :3], want[:, :3], rtol=1e-4, atol=1e-7) >= 0.95
    np.testing.assert_allclose(got[:, :3].mean(0), want[:, :3].mean(0), rtol=0.02)


def test_spot_cone_narrows_the_lit_area(ctx, oracle):
    arrays = procedural.vcm_scene(100, 40)
    wide, _ = _run_both(ctx, oracle, arrays, 48, 48, 1, 4, alpha=0.75)
    narrow, want = _run_both(ctx, oracle, arrays, 48, 48, 1, 4, alpha=0.75, spot_angle=10.0)
    assert close_fraction(narrow[:, :3], want[:, :3]) >= 0.99
    lit = lambda img: int((img[:, :3].sum(1) > 1e-4).sum())
    assert 0 < lit(narrow) < lit(wide)


def test_accumulate_option_matches_oracle(ctx, oracle):
    cb = procedural.cornell_box()
    got, want = _run_both(ctx, oracle, cb, 32, 32, 2, 8, flags=abi.VCM_ACCUMULATE)
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.99
    base, _ = _run_both(ctx, oracle, cb, 32, 32, 2, 8)
    assert got[:, :3].mean() >= base[:, :3].mean()


def test_vcm_error_paths(ctx):
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    sc.build()
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 16, 16)
    film = torch.zeros((256, 4), dtype=torch.float32, device="cuda")
    for bad in (dict(max_depth=0), dict(radius=0.0), dict(num_lights=0), dict(spot_angle=90.0),
                dict(spot_angle=-1.0), dict(spot_angle=float("nan"))):
        p = vcm_params(cb, 8, 0.01, 1, 2, 0)
        for k, v in bad.items():
            setattr(p, k, v)
        with pytest.raises(abi.LgbError):
            sc.vcm_iteration(cam, p, film)
    p = vcm_params(cb, 8, 0.01, 1, 2, 0)
    p.scene_max[1] = p.scene_min[1]
    with pytest.raises(abi.LgbError):
        sc.vcm_iteration(cam, p, film)
    sc.vcm_iteration(cam, vcm_params(cb, 8, 0.01, 1, 2, 0), film)
    sc.sync()
    sc.close()


def test_converged_rmse_against_oracle_reference(ctx, oracle):
    """64 iterations of the caustics configuration at 256^2 against the committed 2048-iteration FP64 oracle
    render (independent seeds): the GPU image and the oracle's own 64 FP32 iterations have the same error against
    it."""
    from lumen_gb300.scene import film_rmse
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vcm_torus_256_fp64_ref.npy"))
    ref = ref.reshape(-1, 3)
    arrays = procedural.vcm_scene()
    got, want = _run_both(ctx, oracle, arrays, 256, 256, 64, 10, alpha=0.75, spot_angle=20.0)
    ref4 = torch.from_numpy(np.concatenate([ref, np.ones((len(ref), 1), np.float32)], 1)).cuda()
    rmse_gpu = film_rmse(ctx, torch.from_numpy(got).cuda(), ref4, 0)
    rmse_cpu = float(np.sqrt(((want[:, :3].astype(np.float64) - ref) ** 2).mean()))
    assert 0.0 < rmse_gpu < 1.0
    np.testing.assert_allclose(rmse_gpu, rmse_cpu, rtol=0.05)
