"""GPU tests of batched rendering (lgb_batch_*): several scenes and views in one wavefront.

Every path of a batch is seeded and computed as lgb_render_path computes it, so each job's film must be
bit-identical to the film of the same job rendered alone, whatever the chunking (small path capacities force
chunks that mix segments of several jobs and split jobs across chunks)."""
import os
import warnings

import numpy as np
import pytest

from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Batch, Context, GpuScene, camera_lookat, path_params

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

DEPTH = 12


@pytest.fixture(scope="module")
def ctx():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return Context(0)


@pytest.fixture(scope="module")
def scenes(ctx):
    out = []
    for seed, tris in ((7, 2000), (8, 12000), (9, 5000)):
        arrays = procedural.batch_scene(seed, tris)
        sc = GpuScene(ctx, arrays)
        sc.build()
        out.append((arrays, sc))
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    sc.build()
    out.append((cb, sc))
    return out


# (scene, width, height, frame0, spp): uneven sizes, two views of scene 0, a continuation from frame 3
JOBS = [(0, 48, 40, 0, 3), (1, 64, 64, 0, 5), (2, 32, 32, 0, 2), (3, 56, 48, 0, 4), (0, 40, 40, 0, 6),
        (3, 32, 32, 3, 2)]


def _camera(arrays, w, h, view=0):
    pos = np.array(arrays.camera_pos, np.float64)
    if view:
        pos = pos + np.array([0.6, 0.3, 0.0])
    return camera_lookat(tuple(pos), arrays.camera_dir, arrays.fov, w, h)


def _films(jobs, seed_film=None):
    films = []
    for k, (_, w, h, frame0, _) in enumerate(jobs):
        f = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
        if frame0 and seed_film is not None:
            f.copy_(seed_film[k])
        films.append(f)
    return films


def _alone(scenes, jobs, films):
    for k, (si, w, h, frame0, spp) in enumerate(jobs):
        arrays, sc = scenes[si]
        cam = _camera(arrays, w, h, view=k == 4)
        sc.render_path(cam, path_params(arrays, DEPTH), frame0, spp, films[k])
        sc.sync()


def _batched(ctx, scenes, jobs, films, opts=None, tune=False):
    batch = Batch(ctx, [sc for _, sc in scenes])
    js = []
    for k, (si, w, h, frame0, spp) in enumerate(jobs):
        arrays, _ = scenes[si]
        js.append(Batch.job(si, _camera(arrays, w, h, view=k == 4), path_params(arrays, DEPTH), frame0, spp, films[k]))
    best = batch.tune(js) if tune else None
    batch.render(js, opts)
    batch.sync()
    return batch, best


def _start_films(scenes):
    """Films for the jobs that continue from frame 3: the first three frames rendered alone."""
    pre = {}
    for k, (si, w, h, frame0, _) in enumerate(JOBS):
        if frame0:
            arrays, sc = scenes[si]
            f = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
            sc.render_path(_camera(arrays, w, h), path_params(arrays, DEPTH), 0, frame0, f)
            sc.sync()
            pre[k] = f
    return [pre.get(k) for k in range(len(JOBS))]


# chunk_paths: 0 = path regeneration with the default chunk (16 x the capacity: here one chunk whose ~60k paths
# run through 4096 or 6000 slots), 1 = no regeneration (chunks of at most the capacity), 20000 = regeneration over
# several chunks, each ending with its films before the next starts.
# traversal: 0 = by the batch's size (coherent here), 2 = the incoherent variant (same hits, other warp schedule).
@pytest.mark.parametrize("capacity,stack,chunk,traversal", [
    (0, 0, 0, 0), (4096, 0, 0, 0), (6000, 0, 0, 0), (0, 1, 0, 0), (6000, 1, 0, 0), (4096, 0, 1, 0), (6000, 0, 1, 0),
    (4096, 0, 20000, 0), (6000, 1, 20000, 0), (4096, 0, 0, 2), (6000, 1, 20000, 2)])
def test_batched_films_equal_films_rendered_alone(ctx, scenes, capacity, stack, chunk, traversal):
    start = _start_films(scenes)
    want = _films(JOBS, start)
    _alone(scenes, JOBS, want)
    got = _films(JOBS, start)
    opts = None
    if capacity or stack or chunk or traversal:
        opts = abi.BatchOpts()
        opts.path_capacity = capacity  # below some images: raised to the largest image
        opts.work_blocks_per_sm = 4
        opts.stack_placement = stack  # the stack's bottom in shared memory gives the same hits
        opts.chunk_paths = chunk
        opts.traversal = traversal
    _batched(ctx, scenes, JOBS, got, opts)
    for k in range(len(JOBS)):
        a, b = got[k].cpu().numpy(), want[k].cpu().numpy()
        assert np.array_equal(a, b), f"job {k}: max diff {np.abs(a - b).max()}"
        assert (a[:, 3] == 1.0).all() and a[:, :3].mean() > 0.0


@pytest.mark.parametrize("chunk", [0, 1])
def test_batched_jobs_of_different_depths(ctx, scenes, chunk):
    """Jobs with path depths 1, 2, 5 and 12 in one batch: with regeneration the wavefront holds paths of every depth
    at once (each path reads its own depth), and every film still equals the job rendered alone."""
    depths = [1, 2, 5, 12]
    jobs = [(0, 40, 32, 0, 3), (1, 48, 48, 0, 4), (2, 32, 40, 0, 5), (3, 56, 48, 0, 2)]
    want = _films(jobs)
    for k, (si, w, h, frame0, spp) in enumerate(jobs):
        arrays, sc = scenes[si]
        sc.render_path(_camera(arrays, w, h), path_params(arrays, depths[k]), frame0, spp, want[k])
        sc.sync()
    got = _films(jobs)
    batch = Batch(ctx, [sc for _, sc in scenes])
    js = [Batch.job(si, _camera(scenes[si][0], w, h), path_params(scenes[si][0], depths[k]), frame0, spp, got[k])
          for k, (si, w, h, frame0, spp) in enumerate(jobs)]
    opts = abi.BatchOpts()
    opts.path_capacity = 4096  # raised to the largest image; the ~22k paths then regenerate through the slots
    opts.chunk_paths = chunk
    batch.render(js, opts)
    batch.sync()
    for k in range(len(jobs)):
        assert np.array_equal(got[k].cpu().numpy(), want[k].cpu().numpy()), f"job {k} (depth {depths[k]})"
    batch.close()


def test_large_scene_traversal_variants_agree(ctx):
    """A 40 000-triangle scene renders alone with the incoherent traversal variant (from 2^15 triangles); the same
    job batched with the coherent variant forced gives the same film."""
    arrays = procedural.batch_scene(11, 40000)
    sc = GpuScene(ctx, arrays)
    sc.build()
    cam = _camera(arrays, 64, 48)
    alone = torch.zeros((64 * 48, 4), dtype=torch.float32, device="cuda")
    sc.render_path(cam, path_params(arrays, DEPTH), 0, 4, alone)
    sc.sync()
    batched = torch.zeros_like(alone)
    batch = Batch(ctx, [sc])
    opts = abi.BatchOpts()
    opts.traversal = abi.TRAVERSAL_COHERENT
    batch.render([Batch.job(0, cam, path_params(arrays, DEPTH), 0, 4, batched)], opts)
    batch.sync()
    a, b = alone.cpu().numpy(), batched.cpu().numpy()
    assert np.array_equal(a, b), f"max diff {np.abs(a - b).max()}"
    assert a[:, :3].mean() > 0.0
    bad = abi.BatchOpts()
    bad.traversal = 3
    with pytest.raises(abi.LgbError):
        batch.render([Batch.job(0, cam, path_params(arrays, DEPTH), 0, 1, batched)], bad)
    batch.close()


def test_tuner_picks_options_and_leaves_films(ctx, scenes):
    films = _films(JOBS)
    for f in films:
        f.fill_(-1.0)
    batch = Batch(ctx, [sc for _, sc in scenes])
    js = []
    for k, (si, w, h, frame0, spp) in enumerate(JOBS):
        arrays, _ = scenes[si]
        js.append(Batch.job(si, _camera(arrays, w, h, view=k == 4), path_params(arrays, DEPTH), 0, spp, films[k]))
    best = batch.tune(js)
    batch.sync()
    assert best.path_capacity in (1 << 20, 1 << 21, 1 << 22, 1 << 23)
    assert best.work_blocks_per_sm in (2, 4, 8, 16)
    assert best.stack_placement in (abi.STACK_LOCAL, abi.STACK_SHARED)
    assert all(bool((f == -1.0).all()) for f in films)
    for f in films:
        f.zero_()
    batch.render(js)  # tuned options
    batch.sync()
    want = _films(JOBS)
    for k, (si, w, h, _, spp) in enumerate(JOBS):
        arrays, sc = scenes[si]
        sc.render_path(_camera(arrays, w, h, view=k == 4), path_params(arrays, DEPTH), 0, spp, want[k])
        sc.sync()
        assert np.array_equal(films[k].cpu().numpy(), want[k].cpu().numpy())


def test_batch_error_paths(ctx, scenes):
    arrays, sc = scenes[0]
    batch = Batch(ctx, [sc])
    film = torch.zeros((32 * 32, 4), dtype=torch.float32, device="cuda")
    cam = _camera(arrays, 32, 32)
    with pytest.raises(abi.LgbError):
        batch.render([Batch.job(1, cam, path_params(arrays, DEPTH), 0, 1, film)])  # no scene 1
    with pytest.raises(abi.LgbError):
        batch.render([Batch.job(0, cam, path_params(arrays, DEPTH), 0, 1, film)] * 129)  # too many jobs
    bad = path_params(arrays, DEPTH)
    bad.num_lights = 99
    with pytest.raises(abi.LgbError):
        batch.render([Batch.job(0, cam, bad, 0, 1, film)])
    bad_opts = abi.BatchOpts()
    bad_opts.stack_placement = 2
    with pytest.raises(abi.LgbError):
        batch.render([Batch.job(0, cam, path_params(arrays, DEPTH), 0, 1, film)], bad_opts)
    misaligned = torch.zeros(32 * 32 * 4 + 4, dtype=torch.float32, device="cuda")[1:]  # 4-byte offset
    with pytest.raises(abi.LgbError):
        batch.render([Batch.job(0, cam, path_params(arrays, DEPTH), 0, 1, misaligned)])
    # a scene rebuilt after the batch was made is refused
    other = GpuScene(ctx, procedural.batch_scene(3, 500))
    other.build()
    b2 = Batch(ctx, [other])
    other.build()
    with pytest.raises(abi.LgbError):
        b2.render([Batch.job(0, _camera(other.arrays, 32, 32), path_params(other.arrays, DEPTH), 0, 1, film)])
    b2.close()
    # a scene without a BVH cannot join a batch
    fresh = GpuScene(ctx, procedural.batch_scene(4, 500))
    with pytest.raises(abi.LgbError):
        Batch(ctx, [fresh])
    batch.render([Batch.job(0, cam, path_params(arrays, DEPTH), 0, 2, film)])
    batch.sync()
    assert film[:, :3].mean().item() > 0.0


def test_batch_render_refuses_a_capturing_stream(ctx, scenes):
    """A render is one launch of the batch's own graph; inside a caller's stream capture it is refused (its job
    table upload would replay later staging) and nothing is captured."""
    arrays, sc = scenes[0]
    batch = Batch(ctx, [sc])
    film = torch.zeros((32 * 32, 4), dtype=torch.float32, device="cuda")
    job = Batch.job(0, _camera(arrays, 32, 32), path_params(arrays, DEPTH), 0, 1, film)
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        graph.capture_begin()
        try:
            with pytest.raises(abi.LgbError) as e:
                batch.render([job], stream=side.cuda_stream)
        finally:
            with warnings.catch_warnings():  # the captured graph is empty, which torch reports
                warnings.simplefilter("ignore")
                graph.capture_end()
    assert e.value.status == 6  # LGB_ERR_UNSUPPORTED
    batch.render([job])  # the batch is still usable
    batch.sync()
    assert film[:, :3].mean().item() > 0.0
    batch.close()


def test_tuning_cache_persists_choices(tmp_path):
    """lgb_create's tuning cache: the first tune of a batch times the candidates and records the choice; a second
    context on the same cache file (a later process on the same kind of device) gets that choice without timing
    anything, and a batch of another shape is tuned and added as a second entry."""
    path = str(tmp_path / "tuning.txt")

    def tune(ctx, jobs):
        scs = []
        for seed, tris in ((7, 2000), (8, 12000), (9, 5000)):
            arrays = procedural.batch_scene(seed, tris)
            sc = GpuScene(ctx, arrays)
            sc.build()
            scs.append((arrays, sc))
        films = _films(jobs)
        batch = Batch(ctx, [sc for _, sc in scs])
        js = [Batch.job(si, _camera(scs[si][0], w, h), path_params(scs[si][0], DEPTH), 0, spp, films[k])
              for k, (si, w, h, _, spp) in enumerate(jobs)]
        best = batch.tune(js)
        batch.sync()
        batch.close()
        return best

    jobs = [(0, 48, 40, 0, 3), (1, 64, 64, 0, 5), (2, 32, 32, 0, 2)]
    first = tune(Context(0, tuning_cache=path), jobs)
    assert first.from_cache == 0
    lines = open(path).read().splitlines()
    assert len(lines) == 1 and ";abi=2;jobs=3;" in lines[0]
    second = tune(Context(0, tuning_cache=path), jobs)
    assert second.from_cache == 1
    assert (second.path_capacity, second.work_blocks_per_sm, second.stack_placement) == \
        (first.path_capacity, first.work_blocks_per_sm, first.stack_placement)
    other = tune(Context(0, tuning_cache=path), jobs[:2])
    assert other.from_cache == 0
    assert len(open(path).read().splitlines()) == 2
    # an unreadable cache is ignored: tuning still works
    bad = tune(Context(0, tuning_cache=str(tmp_path / "missing_dir" / "t.txt")), jobs)
    assert bad.from_cache == 0
