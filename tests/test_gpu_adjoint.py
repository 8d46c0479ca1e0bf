"""GPU tests of the differentiable path estimator (lgb_diff_render) and its adjoint path replay
(lgb_adjoint_path) on the differentiable Cornell box (textured back wall, two GGX conductor boxes).

  * the primal equals the ordinary path estimator at the scene's own parameter values, and the oracle's
    detached estimator (same per-pixel RNG seeding);
  * adjoint gradients of a fixed linear image loss match FP64 central finite differences of the oracle's
    detached estimator (h = 1e-3, common random numbers: the same frames on both sides) within 1 %;
  * a torch.autograd.Function wrapper, defined here in the tests only, drives Adam to recover texture,
    roughness and emission of a target rendered with other seeded parameters.
"""
import os

import numpy as np
import pytest

import parity_log

from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene, camera_lookat, path_params

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

DEPTH = 6
TEX_ID = 0
EMITTER, SHORT, TALL = 3, 5, 6
FD_H = 1e-3


@pytest.fixture(scope="module")
def ctx():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return Context(0)


@pytest.fixture(scope="module")
def diff_scene(ctx, oracle):
    arrays = procedural.cornell_diff()
    sc = GpuScene(ctx, arrays)
    sc.build()
    return arrays, sc, oracle.scene(arrays)


def scene_params(arrays):
    """The scene's own values as parameter tensors: texels (64, 64, 4), roughness (M,), emission (M, 3)."""
    tex = torch.from_numpy(np.ascontiguousarray(arrays.textures[TEX_ID])).cuda()
    rough = torch.from_numpy(arrays.materials["roughness"].astype(np.float32)).cuda()
    emis = torch.from_numpy(arrays.materials["emissive_factor"].astype(np.float32)).cuda()
    return tex, rough, emis


def render(sc, arrays, w, h, frame0, spp, tex=None, rough=None, emis=None, samples=None, flags=0):
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    film = torch.empty((w * h, 4), dtype=torch.float32, device="cuda")
    sc.diff_render(cam, path_params(arrays, DEPTH), frame0, spp, film, TEX_ID, tex, rough, emis, samples=samples,
                   flags=flags)
    return cam, film


def adjoint(sc, arrays, w, h, frame0, spp, dimage, tex, rough, emis, samples=None, flags=0):
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    gt, gr, ge = torch.zeros_like(tex), torch.zeros_like(rough), torch.zeros_like(emis)
    sc.adjoint_path(cam, path_params(arrays, DEPTH), frame0, spp, dimage, TEX_ID, tex, rough, emis, gt, gr, ge,
                    samples=samples, flags=flags)
    sc.sync()
    return gt, gr, ge


def close_fraction(a, b, rtol=1e-4):
    ok = np.abs(a - b) <= rtol * np.maximum(np.abs(b), 1e-6) + 1e-7
    frac = ok.all(axis=1).mean()
    parity_log.record(frac, rtol)
    return frac


def test_primal_matches_path_estimator_and_oracle(diff_scene):
    arrays, sc, osc = diff_scene
    w = h = 64
    tex, rough, emis = scene_params(arrays)
    cam, film = render(sc, arrays, w, h, 3, 1, tex, rough, emis)
    raw = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    sc.render_path(cam, path_params(arrays, DEPTH, film_mode=1), 3, 1, raw)
    sc.sync()
    got = film.cpu().numpy()[:, :3]
    assert close_fraction(got, raw.cpu().numpy()[:, :3]) >= 0.99
    want = osc.diff(cam, DEPTH, w, h, 3, 1, tex_id=TEX_ID, texels=arrays.textures[TEX_ID],
                    rough=arrays.materials["roughness"], emis=arrays.materials["emissive_factor"], fp64=False)
    frac = close_fraction(got, want.astype(np.float32))
    assert frac >= 0.99, f"only {frac:.4f} of samples within 1e-4 of the oracle"
    # null parameter pointers keep the scene's values
    _, film0 = render(sc, arrays, w, h, 3, 1)
    sc.sync()
    assert np.array_equal(film0.cpu().numpy(), film.cpu().numpy())


def test_sampling_with_parameters_equals_scene_with_those_values(ctx, diff_scene):
    """With LGB_DIFF_SAMPLE_PARAMS the estimator at parameters p is the path estimator of the scene whose
    materials and texture hold p."""
    arrays, sc, _ = diff_scene
    w = h = 64
    tex = torch.from_numpy(procedural.albedo_texture(9)).cuda()
    _, rough, emis = scene_params(arrays)
    rough[SHORT], rough[TALL] = 0.5, 0.12
    emis[EMITTER] = torch.tensor([12.0, 15.0, 9.0])
    _, film = render(sc, arrays, w, h, 2, 1, tex, rough, emis, flags=abi.DIFF_SAMPLE_PARAMS)
    other = procedural.cornell_diff(texture_seed=9, roughness=(0.5, 0.12))
    mats = other.materials.copy()
    mats["emissive_factor"][EMITTER] = (12.0, 15.0, 9.0)
    other.materials = mats
    sc2 = GpuScene(ctx, other)
    sc2.build()
    raw = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    cam = camera_lookat(other.camera_pos, other.camera_dir, other.fov, w, h)
    sc2.render_path(cam, path_params(other, DEPTH, film_mode=1), 2, 1, raw)
    sc2.sync()
    frac = close_fraction(film.cpu().numpy()[:, :3], raw.cpu().numpy()[:, :3])
    assert frac >= 0.99, f"only {frac:.4f} of samples agree"
    sc2.close()


def test_samples_buffer_and_replay_modes_agree(diff_scene):
    arrays, sc, _ = diff_scene
    w = h = 48
    spp = 4
    tex, rough, emis = scene_params(arrays)
    samples = torch.empty((spp * w * h, 4), dtype=torch.float32, device="cuda")
    _, film = render(sc, arrays, w, h, 0, spp, tex, rough, emis, samples=samples)
    sc.sync()
    np.testing.assert_allclose(film.cpu().numpy()[:, :3],
                               samples.view(spp, w * h, 4).mean(0).cpu().numpy()[:, :3], rtol=1e-5, atol=1e-6)
    dimage = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, (w * h, 4)).astype(np.float32)).cuda()
    a = adjoint(sc, arrays, w, h, 0, spp, dimage, tex, rough, emis, samples=samples)
    b = adjoint(sc, arrays, w, h, 0, spp, dimage, tex, rough, emis)
    for x, y in zip(a, b):
        x, y = x.cpu().numpy(), y.cpu().numpy()
        assert np.abs(x).max() > 0
        # stored-total replay subtracts, the two-pass replay sums suffixes: equal up to rounding
        np.testing.assert_allclose(x, y, rtol=1e-3, atol=1e-4 * np.abs(y).max())


def test_error_paths(diff_scene):
    arrays, sc, _ = diff_scene
    tex, rough, emis = scene_params(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, 16, 16)
    film = torch.empty((256, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(abi.LgbError):
        sc.diff_render(cam, path_params(arrays, 17), 0, 1, film, TEX_ID, tex, rough, emis)  # depth above 16
    with pytest.raises(abi.LgbError):
        sc.diff_render(cam, path_params(arrays, DEPTH), 0, 1, film, 3, tex, rough, emis)  # no texture 3
    with pytest.raises(abi.LgbError):
        sc.diff_render(cam, path_params(arrays, DEPTH), 0, 0, film, TEX_ID, tex, rough, emis)  # zero spp
    with pytest.raises(abi.LgbError):  # a parameter set without its gradient buffer
        sc.adjoint_path(cam, path_params(arrays, DEPTH), 0, 1, film, TEX_ID, tex, rough, emis, None,
                        torch.zeros_like(rough), torch.zeros_like(emis))


@pytest.mark.parametrize("w,spp,single_texels", [(128, 8, True), (512, 32, False)])
def test_adjoint_matches_fp64_central_differences(diff_scene, w, spp, single_texels):
    """d loss / d parameter for loss = sum(W * image), W fixed and seeded, against FP64 central differences of
    the oracle's detached estimator over the same frames (h = 1e-3): every emission channel of the emitter,
    both box roughnesses, a directional derivative over all texels and (at 128^2) the eight largest texel
    gradients. Run at 128^2 x 8 spp and at the configuration's own 512^2 x 32 spp."""
    arrays, sc, osc = diff_scene
    h = w
    tex, rough, emis = scene_params(arrays)
    W = np.random.default_rng(11).uniform(-1.0, 1.0, (w * h, 3))
    dimage = torch.zeros((w * h, 4), dtype=torch.float32)
    dimage[:, :3] = torch.from_numpy(W.astype(np.float32))
    dimage = dimage.cuda()
    samples = torch.empty((spp * w * h, 4), dtype=torch.float32, device="cuda")
    cam, _ = render(sc, arrays, w, h, 0, spp, tex, rough, emis, samples=samples)
    gt, gr, ge = (g.cpu().numpy().astype(np.float64)
                  for g in adjoint(sc, arrays, w, h, 0, spp, dimage, tex, rough, emis, samples=samples))
    W = dimage.cpu().numpy()[:, :3].astype(np.float64)
    p0 = {"tex_id": TEX_ID, "texels": arrays.textures[TEX_ID].copy(),
          "rough": arrays.materials["roughness"].astype(np.float32), "emis": arrays.materials["emissive_factor"].astype(np.float32)}

    def loss(p):
        return float((osc.diff(cam, DEPTH, w, h, 0, spp, fp64=True, **p) * W).sum())

    def check(name, key, direction, grad):
        """direction: float64 array shaped like p0[key]; grad: the adjoint gradient of that parameter set."""
        plus, minus = dict(p0), dict(p0)
        plus[key] = (p0[key] + FD_H * direction).astype(np.float32)
        minus[key] = (p0[key] - FD_H * direction).astype(np.float32)
        step = plus[key].astype(np.float64) - minus[key].astype(np.float64)  # the step actually taken
        fd = loss(plus) - loss(minus)
        pred = float((grad * step).sum())
        report.append((name, fd / (2 * FD_H), pred / (2 * FD_H)))
        assert abs(fd) > 0, name
        assert abs(pred - fd) <= 0.01 * abs(fd), f"{name}: adjoint {pred / (2 * FD_H):.6g} vs FD {fd / (2 * FD_H):.6g}"

    report = []
    for c in range(3):
        d = np.zeros((len(arrays.materials), 3))
        d[EMITTER, c] = 1.0
        check(f"emission[{c}]", "emis", d, ge)
    for m in (SHORT, TALL):
        d = np.zeros(len(arrays.materials))
        d[m] = 1.0
        check(f"roughness[{m}]", "rough", d, gr)
    v = np.random.default_rng(12).choice([-1.0, 1.0], gt.shape)
    v[..., 3] = 0.0
    check("texels . v", "texels", v, gt)
    flat = np.argsort(-np.abs(gt[..., :3]).ravel())[:8] if single_texels else []
    for i in flat:
        y, x, c = np.unravel_index(i, gt[..., :3].shape)
        d = np.zeros(gt.shape)
        d[y, x, c] = 1.0
        check(f"texel[{y},{x},{c}]", "texels", d, gt)
    for name, fd, adj in report:
        print(f"{name:16s} FD {fd: .6e}  adjoint {adj: .6e}  rel {abs(adj - fd) / abs(fd):.2e}")


class DiffRender(torch.autograd.Function):
    """Test-harness autograd wrapper: forward = lgb_diff_render over frames [frame0, frame0 + spp); backward =
    lgb_adjoint_path over `adjoint_frame0` instead, both sampling with the current parameter values. For a loss that is not linear in the image (L2), replaying
    the same frames that produced the residual gives the gradient of E[loss] plus Cov(image, d image / d param),
    which biases albedos towards zero; independent frames in the backward pass remove that term. With
    adjoint_frame0 == frame0 the backward replays the forward's stored samples."""

    @staticmethod
    def forward(ctx, tex, rough, emis, sc, arrays, w, h, frame0, spp, adjoint_frame0):
        same = adjoint_frame0 == frame0
        samples = torch.empty((spp * w * h, 4), dtype=torch.float32, device="cuda") if same else None
        _, film = render(sc, arrays, w, h, frame0, spp, tex.detach(), rough.detach(), emis.detach(), samples=samples,
                         flags=abi.DIFF_SAMPLE_PARAMS)
        ctx.save_for_backward(tex.detach(), rough.detach(), emis.detach())
        ctx.samples = samples
        ctx.setup = (sc, arrays, w, h, adjoint_frame0, spp)
        return film

    @staticmethod
    def backward(ctx, gfilm):
        tex, rough, emis = ctx.saved_tensors
        sc, arrays, w, h, frame0, spp = ctx.setup
        gt, gr, ge = adjoint(sc, arrays, w, h, frame0, spp, gfilm.contiguous(), tex, rough, emis,
                             samples=ctx.samples, flags=abi.DIFF_SAMPLE_PARAMS)
        return gt, gr, ge, None, None, None, None, None, None, None


def test_autograd_adam_recovers_target(diff_scene):
    """200 Adam steps from the scene's values towards a target rendered with another seeded texture, other
    roughnesses and another emission; every step uses fresh frames, and the adjoint replays frames independent
    of the forward's. 256^2 puts about two pixels across each of the 64 x 64 texels; texel recovery is measured
    on the texels the camera sees best (primary hits)."""
    arrays, sc, _ = diff_scene
    w = h = 256
    spp = 16
    steps = 200
    tex_t = torch.from_numpy(procedural.albedo_texture(6)).cuda()
    rough_t = torch.from_numpy(arrays.materials["roughness"].astype(np.float32)).cuda()
    rough_t[SHORT], rough_t[TALL] = 0.2, 0.3
    emis_t = torch.from_numpy(arrays.materials["emissive_factor"].astype(np.float32)).cuda()
    emis_t[EMITTER] = torch.tensor([14.0, 12.5, 11.0])
    _, target = render(sc, arrays, w, h, 1 << 20, 256, tex_t, rough_t, emis_t)
    target = target[:, :3].clone()

    tex0, rough0, emis0 = scene_params(arrays)
    # texels seen by primary rays: the texel gradient of the image sum at depth 2 (primary hit + direct light)
    ones = torch.ones((w * h, 4), dtype=torch.float32, device="cuda")
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    vis = torch.zeros_like(tex0)
    sc.adjoint_path(cam, path_params(arrays, 2), 0, 16, ones, TEX_ID, tex0, rough0, emis0, vis,
                    torch.zeros_like(rough0), torch.zeros_like(emis0))
    sc.sync()
    vis = vis[..., :3].abs().sum(-1)
    mask = vis > torch.quantile(vis[vis > 0], 0.5)
    assert mask.float().mean() > 0.25

    tex = tex0.clone().requires_grad_(True)
    rough = rough0.clone().requires_grad_(True)
    emis = emis0.clone().requires_grad_(True)
    opt = torch.optim.Adam([{"params": [tex], "lr": 0.05}, {"params": [rough], "lr": 0.01},
                            {"params": [emis], "lr": 0.2}])

    def errors():
        return ((tex - tex_t)[..., :3].abs().mean(-1)[mask].mean().item(),
                (rough - rough_t)[[SHORT, TALL]].abs().max().item(),
                (emis - emis_t)[EMITTER].abs().max().item())

    def image_loss():
        _, img = render(sc, arrays, w, h, 1 << 22, 64, tex.detach(), rough.detach(), emis.detach())
        return ((img[:, :3] - target) ** 2).mean().item()

    e0, l0 = errors(), image_loss()
    for step in range(steps):
        opt.zero_grad()
        img = DiffRender.apply(tex, rough, emis, sc, arrays, w, h, step * spp, spp, (1 << 24) + step * spp)
        loss = ((img[:, :3] - target) ** 2).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            tex.clamp_(0.01, 1.0)
            rough.clamp_(0.1, 1.0)
            emis.clamp_(min=0.0)
    e1, l1 = errors(), image_loss()
    print("texel / roughness / emission error:", e0, "->", e1, " image loss (64 spp):", l0, "->", l1)
    assert e1[0] < 0.6 * e0[0]
    assert e1[1] < 0.5 * e0[1]
    assert e1[2] < 0.1 * e0[2]
    assert l1 < 0.25 * l0


def test_primal_converged_rmse_against_fp64_reference(diff_scene):
    """32 spp of the differentiable configuration (512^2) against the committed 512-spp FP64 oracle render: the GPU
    primal and the FP32 oracle estimator of the same samples have the same error against the converged image."""
    from lumen_gb300.scene import film_rmse
    arrays, sc, osc = diff_scene
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "diff_512_fp64_ref.npy"))
    ref = ref.reshape(-1, 3)
    w = h = 512
    tex, rough, emis = scene_params(arrays)
    cam, film = render(sc, arrays, w, h, 0, 32, tex, rough, emis)
    sc.sync()
    ref4 = torch.from_numpy(np.concatenate([ref, np.ones((len(ref), 1), np.float32)], 1)).cuda()
    rmse_gpu = film_rmse(sc.ctx, film, ref4, 0)
    cpu = osc.diff(cam, DEPTH, w, h, 0, 32, fp64=False)
    rmse_cpu = float(np.sqrt(((cpu - ref) ** 2).mean()))
    assert 0.0 < rmse_gpu < 0.5
    np.testing.assert_allclose(rmse_gpu, rmse_cpu, rtol=0.02)
