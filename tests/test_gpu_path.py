"""GPU parity tests of the wavefront path integrator against the CPU oracle (same per-pixel RNG seeding).

Contract: per-sample radiance within 1e-4 relative. CUDA's sinf/cosf/powf may differ from the host C
library by a few ULP, which can flip a rare branch (Russian roulette, lobe choice) and send a sample down
another path; such flips are counted and must stay rare, and the image means must agree."""
import os

import numpy as np
import pytest

import parity_log

from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene, camera_lookat, path_params

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return Context(0)


@pytest.fixture(scope="module")
def cornell(ctx, oracle):
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    sc.build()
    return cb, sc, oracle.scene(cb)


def gpu_samples(sc, cb, w, h, frame, depth=8):
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    sc.render_path(cam, path_params(cb, depth, film_mode=1), frame, 1, film)
    sc.sync()
    return cam, film.cpu().numpy()[:, :3]


def close_fraction(a, b):
    ok = np.abs(a - b) <= RTOL * np.maximum(np.abs(b), 1e-6) + 1e-7
    frac = ok.all(axis=1).mean()
    parity_log.record(frac, RTOL)
    return frac


@pytest.mark.parametrize("frame", [0, 5])
def test_per_sample_radiance_matches_oracle(cornell, frame):
    cb, sc, osc = cornell
    cam, got = gpu_samples(sc, cb, 64, 64, frame)
    want, nan = osc.samples(cam, 8, 64, 64, frame)
    frac = close_fraction(got, want)
    assert frac >= 0.99, f"only {frac:.4f} of samples within {RTOL} relative"
    np.testing.assert_allclose(got.mean(0), want.mean(0), rtol=2e-2)


def test_progressive_film_matches_oracle(cornell):
    cb, sc, osc = cornell
    w = h = 48
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    sc.render_path(cam, path_params(cb, 8), 0, 3, film)   # frames 0..2 in one launch sequence
    sc.render_path(cam, path_params(cb, 8), 3, 2, film)   # frames 3..4 continue the running mean
    sc.sync()
    got = film.cpu().numpy()
    want = osc.film(cam, 8, w, h, 0, 5)
    assert (got[:, 3] == 1.0).all()
    assert close_fraction(got[:, :3], want[:, :3]) >= 0.97


def test_depth_limits_and_determinism(cornell):
    cb, sc, osc = cornell
    for depth in (1, 2, 3):
        cam, got = gpu_samples(sc, cb, 32, 32, 1, depth=depth)
        want, _ = osc.samples(cam, depth, 32, 32, 1)
        assert close_fraction(got, want) >= 0.99
    _, a = gpu_samples(sc, cb, 32, 32, 2)
    _, b = gpu_samples(sc, cb, 32, 32, 2)
    assert np.array_equal(a, b)


def _material_scene(kind):
    """The Cornell box with the two inner boxes switched to another BSDF."""
    from lumen_gb300 import scene as S
    cb = procedural.cornell_box()
    mats = list(cb.materials)
    if kind == "conductor":
        extra = S.conductor((0.9, 0.6, 0.3), 0.3)
    elif kind == "dielectric":
        extra = S.dielectric(1.5, 0.0)
    elif kind == "rough_dielectric":
        extra = S.dielectric(1.5, 0.3)
    elif kind == "principled":
        extra = S.principled((0.8, 0.3, 0.2), roughness=0.4, metallic=0.3, ior=1.5, clearcoat=0.5)
    elif kind == "principled_glass":
        extra = S.principled((0.9, 0.9, 0.9), roughness=0.2, ior=1.5, spec_trans=0.8)
    elif kind == "glass":
        extra = S.glass(1.5)
    elif kind == "mirror":
        extra = S.new_material(bsdf_type=abi.BSDF_MIRROR, bsdf_props=abi.FLAG_SPECULAR | abi.FLAG_REFLECTION)
    else:
        raise ValueError(kind)
    mats = np.concatenate([cb.materials, extra])
    meshes = cb.meshes.copy()
    meshes["material_index"][5:7] = len(mats) - 1
    cb.materials = mats
    cb.meshes = meshes
    return cb


@pytest.mark.parametrize("kind", ["conductor", "dielectric", "rough_dielectric", "principled", "principled_glass",
                                  "mirror", "glass"])
def test_materials_match_oracle(ctx, oracle, kind):
    cb = _material_scene(kind)
    sc = GpuScene(ctx, cb)
    sc.build()
    cam, got = gpu_samples(sc, cb, 48, 48, 3)
    want, _ = oracle.scene(cb).samples(cam, 8, 48, 48, 3)
    frac = close_fraction(got, want)
    assert frac >= 0.98, f"{kind}: only {frac:.4f} of samples within {RTOL}"


def test_textured_albedo_matches_oracle(ctx, oracle):
    cb = procedural.cornell_box()
    rng = np.random.default_rng(5)
    tex = np.ones((64, 64, 4), np.float32)
    tex[..., :3] = rng.uniform(0.1, 0.9, (64, 64, 3))
    cb.textures = [tex]
    mats = cb.materials.copy()
    mats["texture_id"][0] = 0
    cb.materials = mats
    sc = GpuScene(ctx, cb)
    sc.build()
    cam, got = gpu_samples(sc, cb, 48, 48, 0)
    want, _ = oracle.scene(cb).samples(cam, 8, 48, 48, 0)
    assert close_fraction(got, want) >= 0.99


def test_converged_rmse_against_fp64_reference(cornell, oracle):
    """16 spp at 256^2 against the committed 2048-spp FP64 oracle render: the GPU image and the FP32 oracle image
    of the same samples have the same error against the converged reference."""
    from lumen_gb300.scene import film_rmse
    cb, sc, osc = cornell
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cornell_256_fp64_ref.npy"))
    ref = ref.reshape(-1, 3)
    w = h = 256
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    film = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    sc.render_path(cam, path_params(cb, 8), 0, 16, film)
    sc.sync()
    ref4 = torch.from_numpy(np.concatenate([ref, np.ones((len(ref), 1), np.float32)], 1)).cuda()
    rmse_gpu = film_rmse(sc.ctx, film, ref4, 0)
    cpu = osc.film(cam, 8, w, h, 0, 16)
    rmse_cpu = float(np.sqrt(((cpu[:, :3].astype(np.float64) - ref) ** 2).mean()))
    assert 0.0 < rmse_gpu < 0.5
    np.testing.assert_allclose(rmse_gpu, rmse_cpu, rtol=0.02)
