"""CPU tests of the oracle: known answers for the integer utilities, the watertight ray/triangle contract,
BVH queries against exhaustive testing, and the path integrator's internal consistency."""
import numpy as np
import pytest

import reference_py
from lumen_gb300 import procedural


def test_pcg4d_known_answers(oracle):
    rng = np.random.default_rng(0)
    v = rng.integers(0, 2**32, (512, 4), dtype=np.uint64).astype(np.uint32)
    v[0] = [0, 0, 0, 0]
    v[1] = [0xFFFFFFFF] * 4
    got = oracle.pcg4d(v)
    want = np.array([reference_py.pcg4d([int(c) for c in row]) for row in v], np.uint32)
    assert np.array_equal(got, want)


def test_rand_stream_in_unit_interval():
    xs = reference_py.rand_stream(3, 7, 11, 4096)
    assert min(xs) >= 0.0 and max(xs) < 1.0
    assert abs(np.mean(xs) - 0.5) < 0.02


def test_offset_ray_known_answers(oracle):
    rng = np.random.default_rng(1)
    p = rng.uniform(-3, 3, (2000, 3)).astype(np.float32)
    p[:200] *= np.float32(0.01)  # inside the |p| < 1/32 band
    p[200, :] = 0.0
    n = rng.standard_normal((2000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    got = oracle.offset_ray(p, n)
    want = np.array([reference_py.offset_ray(a, b) for a, b in zip(p.tolist(), n.tolist())], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    np.testing.assert_array_equal(procedural.offset_ray(p, n).view(np.uint32), want.view(np.uint32))


def _fan(n=16, z=0.0):
    """A closed fan of n triangles around the origin in the plane z, sharing the centre vertex and edges."""
    ang = np.linspace(0, 2 * np.pi, n + 1)
    ring = np.stack([np.cos(ang), np.sin(ang), np.full_like(ang, z)], -1).astype(np.float32)
    tv = np.zeros((n, 9), np.float32)
    for i in range(n):
        tv[i, 0:3] = (0, 0, z)
        tv[i, 3:6] = ring[i]
        tv[i, 6:9] = ring[i + 1]
    return tv


def _rays(o, d, tmin=0.0, tmax=1e30):
    o = np.atleast_2d(np.asarray(o, np.float32))
    d = np.atleast_2d(np.asarray(d, np.float32))
    r = np.zeros((max(len(o), len(d)), 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def test_watertight_shared_vertex_and_edges(oracle):
    tv = _fan(16)
    # rays straight down through the shared centre vertex and through points on shared edges
    pts = [(0.0, 0.0)]
    for i in range(16):
        a = 2 * np.pi * i / 16
        for r in (0.25, 0.5, 0.75):
            pts.append((r * np.cos(a), r * np.sin(a)))
    o = [(x, y, 1.0) for x, y in pts]
    rays = _rays(o, (0, 0, -1))
    hits = oracle.brute_closest(tv, rays)
    assert (hits["prim"] != 0xFFFFFFFF).all(), "a ray through a shared vertex or edge leaked through the fan"
    np.testing.assert_allclose(hits["t"], 1.0, rtol=1e-6)
    # tilted rays through the centre vertex from many directions
    rng = np.random.default_rng(2)
    d = rng.standard_normal((500, 3))
    d[:, 2] = -np.abs(d[:, 2]) - 0.2
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = -d * 2.0
    hits = oracle.brute_closest(tv, _rays(o.astype(np.float32), d.astype(np.float32)))
    assert (hits["prim"] != 0xFFFFFFFF).all()


def test_tie_break_lowest_prim(oracle):
    tri = np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], np.float32)
    tv = np.concatenate([tri, tri, tri])  # three coincident triangles
    rays = _rays([(0.1, 0.0, 1.0), (-0.2, -0.3, -2.0)], [(0, 0, -1), (0, 0, 1)])
    for hits in (oracle.brute_closest(tv, rays), oracle.bvh(tv).closest(rays)):
        assert (hits["prim"] == 0).all()


def test_axis_parallel_and_degenerate(oracle):
    tv = np.array([
        [0, 0, 1, 1, 0, 1, 0, 1, 1],        # triangle in z = 1
        [0, 0, 2, 0, 0, 2, 0, 0, 2],        # degenerate point triangle
        [0, 0, 3, 1, 1, 3, 2, 2, 3],        # degenerate line triangle
    ], np.float32)
    rays = _rays([(0.25, 0.25, 0.0), (0.25, 0.25, 5.0), (5.0, 0.25, 1.0)], [(0, 0, 1), (0, 0, -1), (-1, 0, 0)])
    hits = oracle.brute_closest(tv, rays)
    assert hits["prim"][0] == 0 and hits["prim"][1] == 0
    assert hits["prim"][2] == 0xFFFFFFFF  # grazing a triangle in its own plane never hits (det == 0)
    b = oracle.bvh(tv)
    assert np.array_equal(b.closest(rays), hits)


def test_tmin_tmax_window(oracle):
    tv = np.array([[-1, -1, 2, 1, -1, 2, 0, 1, 2]], np.float32)
    rays = _rays([(0, 0, 0)] * 4, [(0, 0, 1)] * 4)
    rays[:, 3] = [0.0, 2.0, 2.5, 0.0]
    rays[:, 7] = [10.0, 10.0, 10.0, 1.5]
    hits = oracle.brute_closest(tv, rays)
    assert list(hits["prim"]) == [0, 0, 0xFFFFFFFF, 0xFFFFFFFF]
    occ = oracle.brute_any(tv, rays)
    assert list(occ) == [1, 1, 0, 0]


@pytest.mark.parametrize("seed", [0, 1])
def test_bvh_matches_brute_force(oracle, seed):
    arrays = procedural.traversal_scene(sphere_freq=8, n_random=3000, seed=seed + 1)
    tv = arrays.tri_verts()
    rays = np.concatenate([
        procedural.incoherent_rays(arrays, 3000, seed=seed + 10),
        procedural.primary_rays(48, 48),
    ])
    b = oracle.bvh(tv)
    got = b.closest(rays)
    want = oracle.brute_closest(tv, rays)
    assert np.array_equal(got, want)
    anyr = rays.copy()
    anyr[:, 7] = 0.5
    assert np.array_equal(b.any(anyr), oracle.brute_any(tv, anyr))


def test_empty_scene(oracle):
    tv = np.zeros((0, 9), np.float32)
    rays = _rays([(0, 0, 0)], [(0, 0, 1)])
    b = oracle.bvh(tv)
    assert b.closest(rays)["prim"][0] == 0xFFFFFFFF
    assert b.any(rays)[0] == 0


class _Cam:
    pass


def _camera(oracle, arrays, w, h):
    c = _Cam()
    c.inv_view, c.inv_projection = oracle.camera(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    return c


def test_path_film_is_progressive_mean_of_samples(oracle):
    cb = procedural.cornell_box()
    sc = oracle.scene(cb)
    cam = _camera(oracle, cb, 24, 16)
    film = sc.film(cam, 8, 24, 16, 0, 3)
    s = [sc.samples(cam, 8, 24, 16, f)[0] for f in range(3)]
    m = s[0].copy()
    for f in (1, 2):
        w = np.float32(1.0) / np.float32(f + 1)
        m = m * (np.float32(1.0) - w) + s[f] * w
    np.testing.assert_array_equal(film[:, :3], m)


def test_path_deterministic_and_fp64_close(oracle):
    cb = procedural.cornell_box()
    sc = oracle.scene(cb)
    cam = _camera(oracle, cb, 32, 32)
    a, _ = sc.samples(cam, 8, 32, 32, 4)
    b, _ = sc.samples(cam, 8, 32, 32, 4)
    assert np.array_equal(a, b)
    d, _ = sc.samples(cam, 8, 32, 32, 4, fp64=True)
    close = np.abs(a - d) <= 1e-3 * np.maximum(np.abs(d), 1e-2)
    assert close.mean() > 0.97
    assert a.mean() > 0.05  # the box is lit


def test_camera_center_ray_looks_along_minus_dir(oracle):
    cb = procedural.cornell_box()
    iv, ip = oracle.camera(cb.camera_pos, cb.camera_dir, 45.0, 64, 64)
    IV = iv.reshape(4, 4).T
    IP = ip.reshape(4, 4).T
    t = IP @ np.array([0, 0, 1, 1.0])
    d = IV @ np.array([*(t[:3] / np.linalg.norm(t[:3])), 0.0])
    np.testing.assert_allclose(d[:3], [0, 0, -1], atol=1e-6)
    np.testing.assert_allclose((IV @ np.array([0, 0, 0, 1.0]))[:3], cb.camera_pos, atol=1e-6)


def test_diff_estimator_equals_path_at_scene_values(oracle):
    """With the parameters equal to the scene's values the detached estimator is the path estimator."""
    a = procedural.cornell_diff()
    sc = oracle.scene(a)
    cam = _camera(oracle, a, 32, 32)
    film = sc.film(cam, 6, 32, 32, 0, 4)
    em = np.zeros((len(a.materials), 3), np.float32)
    em[3] = 17.0
    d = sc.diff(cam, 6, 32, 32, 0, 4, tex_id=0, texels=a.textures[0], rough=a.materials["roughness"], emis=em,
                fp64=False)
    # the film is Lumen's running FP32 mean, the diff image a double mean of the same FP32 samples
    np.testing.assert_allclose(d, film[:, :3], rtol=1e-3, atol=1e-6)
    assert np.array_equal(d, sc.diff(cam, 6, 32, 32, 0, 4, fp64=False))


def test_diff_estimator_is_linear_in_emission_and_smooth_in_parameters(oracle):
    """FP64, common random numbers: the image is exactly linear in the emission, and central differences of a
    texel and of a roughness are stable under halving h (no path changes with the parameters)."""
    a = procedural.cornell_diff()
    sc = oracle.scene(a)
    w = h = 24
    cam = _camera(oracle, a, w, h)
    em = np.zeros((len(a.materials), 3), np.float32)
    em[3] = 17.0
    base = sc.diff(cam, 6, w, h, 0, 2, emis=em)
    np.testing.assert_allclose(sc.diff(cam, 6, w, h, 0, 2, emis=2 * em), 2 * base, rtol=1e-13, atol=0)
    wts = np.random.default_rng(1).uniform(-1, 1, base.shape)

    def fd(make, step):
        return ((sc.diff(cam, 6, w, h, 0, 2, **make(step)) - sc.diff(cam, 6, w, h, 0, 2, **make(-step))) * wts).sum()

    tex = a.textures[0]

    def texel(step):
        t = tex.copy()
        t[:, :, :3] += np.float32(step)  # every texel at once: a directional derivative
        return {"tex_id": 0, "texels": t}

    def rough(step):
        r = a.materials["roughness"].copy()
        r[6] += np.float32(step)
        return {"rough": r}

    for make in (texel, rough):
        g1 = fd(make, 1e-3) / 2e-3
        g2 = fd(make, 5e-4) / 1e-3
        assert abs(g1) > 1e-3
        np.testing.assert_allclose(g1, g2, rtol=2e-3)


def _np_vcm_table(pos4, mn, mx, radius, screen):
    """utils.glsl:62-65 hash of vcm_commons.glsl:17-23 cells over the VCM.cpp:144-147 grid, written sequentially."""
    f32 = np.float32
    mn, mx = np.asarray(mn, f32), np.asarray(mx, f32)
    d = mx - mn
    max_comp = d.max()
    base = int(f32(max_comp / f32(radius)))
    res = [max(int(f32(d[k] * f32(base) / max_comp)), 1) for k in range(3)]
    p = pos4[:, :3].astype(f32)
    cell = ((p - mn) / d * np.asarray(res, f32)).astype(np.int32)
    with np.errstate(over="ignore"):
        h = ((cell[:, 0].astype(np.uint32) * np.uint32(73856093)) ^ (cell[:, 1].astype(np.uint32) * np.uint32(19349663)) ^
             (cell[:, 2].astype(np.uint32) * np.uint32(83492791))) % np.uint32(10 * screen)
    count = np.zeros(10 * screen, np.uint32)
    rep = np.zeros(10 * screen, np.uint32)
    for i in np.nonzero(pos4[:, 3] >= 0)[0]:
        count[h[i]] += 1
        rep[h[i]] = i
    return count, rep


def test_vcm_photon_table_matches_independent_restatement(oracle):
    from oracle_lib import vcm_grid
    rng = np.random.default_rng(4)
    n, screen = 5000, 700
    pos4 = np.concatenate([rng.uniform(-1.2, 1.2, (n, 3)), np.where(rng.uniform(size=(n, 1)) < 0.1, -1.0, 1.0)], 1)
    pos4[:50, :3] = pos4[50:100, :3]  # coincident photons share a slot
    mn, mx, radius = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), 0.05
    count, rep = vcm_grid(oracle, pos4.astype(np.float32), mn, mx, radius, screen)
    want_c, want_r = _np_vcm_table(pos4.astype(np.float32), mn, mx, radius, screen)
    assert np.array_equal(count, want_c) and np.array_equal(rep, want_r)
    assert count.sum() == (pos4[:, 3] >= 0).sum() and (count > 1).any()


def _vcm_oracle_run(oracle, arrays, w, h, iters, depth, flags, use_vm=1, spot_angle=0.0, alpha=2.0 / 3.0):
    from oracle_lib import VcmParams
    from lumen_gb300.scene import camera_lookat, camera_forward, scene_radius, vcm_radius
    sc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    st = sc.vcm_state(w, h, depth)
    R = scene_radius(arrays)
    for it in range(iters):
        p = VcmParams()
        p.max_depth, p.num_lights, p.light_triangle_count = depth, len(arrays.lights), arrays.light_triangle_count
        p.scene_min[:] = [float(v) for v in arrays.positions.min(0)]
        p.scene_max[:] = [float(v) for v in arrays.positions.max(0)]
        p.radius = vcm_radius(R, 1.0, it, alpha)
        p.spot_angle = spot_angle
        p.use_vm, p.use_vc = use_vm, 1
        p.light_seed, p.eye_seed, p.frame_num, p.flags = 1000 + it, 5000 + it, it, flags
        sc.vcm_iteration(cam, view, proj, p, st)
    return sc, cam, st



def test_vcm_oracle_max_depth_one_known_answer(oracle):
    """At max depth 1 every subpath has one segment: the light pass stops before its camera connection
    (vcm_commons.glsl:367-372), the eye pass's light connection needs depth < max_depth (:565), and a merge's
    path length (:269) exceeds the maximum. So each pixel's single sample is exactly the emission its jittered
    camera ray sees: 17 on the Cornell box's emitter, else 0 (black sky), and no splat is written."""
    cb = procedural.cornell_box()
    _, _, st = _vcm_oracle_run(oracle, cb, 32, 32, 1, 1, 0)
    film = st["film"][:, :3]
    lit = (film > 0.0).any(axis=1)
    assert lit.sum() > 0
    assert np.array_equal(film[lit], np.full((int(lit.sum()), 3), 17.0, np.float32))
    assert not film[~lit].any() and not st["splat"].any()

def test_vcm_oracle_is_deterministic_and_energy_consistent(oracle):
    """With every connection accumulated (LGB_VCM_ACCUMULATE) and a non-reflecting emitter, VCM converges to the
    path tracer's image. (With the white emitter of the Cornell box the path tracer itself gains energy from its
    stale-payload quirk on BSDF-MIS rays that start on the emitter and miss, pt_commons.glsl:32-33.)"""
    cb = procedural.cornell_box()
    m = cb.materials.copy()
    m["albedo"][3] = 0.0
    cb.materials = m
    sc, cam, st = _vcm_oracle_run(oracle, cb, 32, 32, 48, 8, 1)
    _, _, st2 = _vcm_oracle_run(oracle, cb, 32, 32, 48, 8, 1)
    assert np.array_equal(st["film"], st2["film"])
    pt = sc.film(cam, 8, 32, 32, 0, 256)
    vcm_mean, pt_mean = st["film"][:, :3].mean(), pt[:, :3].mean()
    assert abs(vcm_mean - pt_mean) < 0.03 * pt_mean, (vcm_mean, pt_mean)
    assert not np.isnan(st["film"]).any()


def test_vcm_oracle_spot_cone(oracle):
    """The spot cone parameter: 30 degrees equals the reference's fixed cone exactly; a 10 degree cone lights
    fewer pixels of the caustics scene than the fixed one, and a 20 degree one sits between them."""
    arrays = procedural.vcm_scene(60, 24)
    films = {a: _vcm_oracle_run(oracle, arrays, 32, 32, 1, 4, 0, spot_angle=a, alpha=0.75)[2]["film"]
             for a in (0.0, 30.0, 20.0, 10.0)}
    assert np.array_equal(films[0.0], films[30.0])
    lit = {a: int((f[:, :3].sum(1) > 1e-4).sum()) for a, f in films.items()}
    assert 0 < lit[10.0] < lit[20.0] < lit[0.0], lit


def test_sppm_oracle_is_deterministic_and_plausible(oracle):
    """The oracle's SPPM: the same seed gives the same film; radii shrink as photons are gathered; the image is
    within 25 % of the path tracer's mean (the two estimators share the eye pass's direct lighting but differ in
    the reference's quirks: the path tracer's stale BSDF-MIS payload brightens the white emitter's surround)."""
    import oracle_lib
    from lumen_gb300.scene import camera_lookat
    cb = procedural.cornell_box()
    sc = oracle.scene(cb)
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 32, 32)
    films = []
    for _ in range(2):
        st = oracle_lib.sppm_state(32, 32, 6)
        for f in range(8):
            p = oracle_lib.SppmParams()
            p.max_depth, p.num_lights, p.light_triangle_count = 6, len(cb.lights), cb.light_triangle_count
            p.base_radius, p.seed, p.frame_num = 0.03, 5, f
            oracle_lib.sppm_iteration(sc, cam, p, st)
        films.append(st["film"].copy())
    assert np.array_equal(films[0], films[1]) and not np.isnan(films[0]).any()
    vp = st["vp"].reshape(-1, 32)
    assert vp[:, 3].min() < 0.03 and vp[:, 3].max() <= 0.03
    pt = sc.film(cam, 6, 32, 32, 0, 32)
    assert abs(films[0][:, :3].mean() - pt[:, :3].mean()) < 0.25 * pt[:, :3].mean()


def _restir_frames(oracle, arrays, w, h, frames, seed=11, flags=0, accumulate=1):
    import oracle_lib
    from lumen_gb300.scene import camera_forward, camera_lookat
    sc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    st = oracle_lib.restir_state(w, h)
    means = []
    for f in range(frames):
        p = oracle_lib.RestirParams()
        p.num_lights, p.light_triangle_count = len(arrays.lights), arrays.light_triangle_count
        p.seed, p.frame_num, p.do_spatiotemporal, p.enable_accumulation = seed, f, 1 if f > 0 else 0, accumulate
        p.flags = flags
        oracle_lib.restir_iteration(sc, cam, view, proj, p, st)
        means.append(st["film"][:, :3].copy())
    return sc, cam, st, means


def test_restir_oracle_is_deterministic_and_matches_direct_light(oracle):
    """The oracle's ReSTIR DI on the Cornell box. The same seed gives the same film. Frame 0 (no reuse over time)
    is close to the path tracer's direct light (depth-2 minus depth-1 images) on the pixels that do not see the
    emitter (there the path tracer's stale BSDF-MIS payload adds light ReSTIR does not have). With Lumen's spatial
    sample count the per-frame image brightens frame after frame; with LGB_RESTIR_SPATIAL_COUNT_FIX it holds a
    steady level, somewhat below the direct light (reused samples are not tested for visibility where they are
    reused, and a pixel whose own sample was occluded does not reuse: ReSTIR's usual darkening)."""
    cb = procedural.cornell_box()
    sc, cam, st, quirk = _restir_frames(oracle, cb, 32, 32, 10, accumulate=0)
    _, _, st2, _ = _restir_frames(oracle, cb, 32, 32, 10, accumulate=0)
    assert np.array_equal(st["film"], st2["film"]) and not np.isnan(st["film"]).any()
    emitter = sc.film(cam, 1, 32, 32, 0, 64)[:, :3].sum(1) > 0
    direct = (sc.film(cam, 2, 32, 32, 0, 256)[:, :3] - sc.film(cam, 1, 32, 32, 0, 256)[:, :3])[~emitter].mean()
    f0 = quirk[0][~emitter].mean()
    assert abs(f0 - direct) < 0.15 * direct, (f0, direct)
    assert quirk[-1][~emitter].mean() > 2.0 * f0  # the reference's estimate grows with the frames
    _, _, _, fixed = _restir_frames(oracle, cb, 32, 32, 10, flags=1, accumulate=0)
    levels = [m[~emitter].mean() for m in fixed[1:]]
    assert max(levels) < 1.2 * min(levels), levels
    assert 0.6 * direct < min(levels) and max(levels) < 1.1 * direct, (levels, direct)


def _bdpt_frames(oracle, arrays, w, h, frames, depth=6, seed=7, spot_angle=0.0, check=(0, 0, -1)):
    import oracle_lib
    from lumen_gb300.scene import camera_forward, camera_lookat
    sc = oracle.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, w, h)
    view, proj = camera_forward(cam)
    st = oracle_lib.bdpt_state(w, h)
    for f in range(frames):
        p = oracle_lib.BdptParams()
        p.max_depth, p.num_lights, p.light_triangle_count = depth, len(arrays.lights), arrays.light_triangle_count
        p.seed, p.frame_num, p.spot_angle = seed, f, spot_angle
        p.check_flags, p.check_len, p.check_s = check
        oracle_lib.bdpt_iteration(sc, cam, view, proj, p, st)
    return sc, cam, st


def test_bdpt_oracle_is_deterministic_and_matches_path_tracer(oracle):
    """The oracle's BDPT on the Cornell box with a non-reflecting emitter (the path tracer's stale BSDF-MIS
    payload quirk then has nothing to add): the same seed gives the same film, and off the emitter the image is
    within 8 % of the path tracer's (BDPT traces pixel centres only, bdpt.rgen:40, the path tracer jitters). The
    emitter pixels hold its emission (s = 0, t = 2, MIS weight 1)."""
    cb = procedural.cornell_box()
    m = cb.materials.copy()
    m["albedo"][3] = 0.0
    cb.materials = m
    sc, cam, st = _bdpt_frames(oracle, cb, 32, 32, 48)
    _, _, st2 = _bdpt_frames(oracle, cb, 32, 32, 48)
    assert np.array_equal(st["film"], st2["film"]) and not np.isnan(st["film"]).any()
    emitter = sc.film(cam, 1, 32, 32, 0, 64)[:, :3].sum(1) > 0
    pt = sc.film(cam, 6, 32, 32, 0, 256)[:, :3]
    b = st["film"][:, :3]
    assert abs(b[~emitter].mean() / pt[~emitter].mean() - 1.0) < 0.08, (b[~emitter].mean(), pt[~emitter].mean())
    assert b.max() >= 17.0 * 0.99  # emission 17 seen directly at some pixel centre


def test_bdpt_oracle_spot_cone_and_depth(oracle):
    """The caustics scene: 30 degrees equals the reference's fixed spot cone; a longer path length only adds
    light."""
    arrays = procedural.vcm_scene(60, 24)
    films = {a: _bdpt_frames(oracle, arrays, 24, 24, 2, 4, spot_angle=a)[2]["film"] for a in (0.0, 30.0)}
    assert np.array_equal(films[0.0], films[30.0])
    short = _bdpt_frames(oracle, arrays, 24, 24, 8, 2)[2]["film"][:, :3].mean()
    long = _bdpt_frames(oracle, arrays, 24, 24, 8, 8)[2]["film"][:, :3].mean()
    assert 0.0 < short < long


def test_bdpt_oracle_every_bsdf_type():
    """The oracle's BDPT on a loaded scene with diffuse, conductor, dielectric and principled materials, a spot
    light (a delta light: vertex 0 has pdf_fwd = 0 and is skipped by the MIS sums) and an emissive lamp (an area
    light), so the s = 1 strategies' MIS weight often reads the flags of a light other than the one they sampled
    (kept from the reference): deterministic, finite and lit."""
    import os
    import oracle_lib
    from lumen_gb300 import build, host_scene
    if not os.path.exists(host_scene.HOST_LIB):
        build.build_library()
    here = os.path.dirname(os.path.abspath(__file__))
    arrays, info = host_scene.load_scene(os.path.join(here, "golden", "scenes", "mixed_bdpt.json"))
    assert int(info.path_length) == 5 and len(arrays.lights) == 2
    assert sorted(int(f) & 7 for f in arrays.lights["light_flags"]) == [1, 2]  # spot, area
    assert set(int(t) for t in arrays.materials["bsdf_type"]) >= {1, 8, 16, 32}
    ora = oracle_lib.Oracle()
    films = [_bdpt_frames(ora, arrays, 20, 16, 3, 5)[2]["film"] for _ in range(2)]
    assert np.array_equal(films[0], films[1])
    assert np.isfinite(films[0]).all() and films[0][:, :3].mean() > 0.0


def test_bdpt_oracle_strategies_agree(oracle):
    """No Lumen output exists to pin the BDPT restatement, so its pdfs and MIS weights are checked against each
    other. For paths of 2 and 3 segments on the Cornell box, each connection strategy alone (MIS weight 1: light
    tracing, vertex connections, next-event estimation, the camera path hitting the emitter) is an estimate of
    the same radiance, and so is the MIS-weighted sum over them: all agree within 10 % at 64 frames of 32 x 32
    (observed within 4 %). Restricting the film to one strategy keeps the random numbers of the others, so the
    weighted parts add up to the weighted total to rounding."""
    cb = procedural.cornell_box()
    mean = lambda check: float(_bdpt_frames(oracle, cb, 32, 32, 64, check=check)[2]["film"][:, :3].mean())
    for k in (2, 3):
        total = mean((1, k, -1))
        assert total > 0.0
        for s in range(k + 1):
            alone = mean((3, k, s))
            assert abs(alone / total - 1.0) < 0.10, (k, s, alone, total)
        parts = sum(mean((1, k, s)) for s in range(k + 1))
        assert abs(parts - total) <= 1e-5 * total, (k, parts, total)


def test_bdpt_oracle_path_length_one_known_answer(oracle):
    """With path length 1 the only strategy is the camera ray hitting the emitter (s = 0, t = 2: throughput 1, MIS
    weight 1, bdpt.rgen:52-58), so every pixel of the film is exactly the emission of what its centre sees: 17 on
    the Cornell box's emitter, 0 elsewhere, in every frame."""
    cb = procedural.cornell_box()
    film = _bdpt_frames(oracle, cb, 32, 32, 3, depth=1)[2]["film"][:, :3]
    lit = (film > 0.0).any(axis=1)
    assert lit.sum() > 0
    assert np.array_equal(film[lit], np.full((int(lit.sum()), 3), 17.0, np.float32))
    assert not film[~lit].any()
