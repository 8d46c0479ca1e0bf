"""GPU parity tests of the BVH builder and the closest/any-hit kernels against the CPU oracle, through the
C ABI. Contract: primitive ids bit-exact (lowest id wins ties), t/u/v within 1e-6 relative (the FP32
sequence is shared, so they are expected to be bit-identical), occlusion bits exact."""
import os

import numpy as np
import pytest

import oracle_lib
from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

T_RTOL = 1e-6


@pytest.fixture(scope="module")
def ctx():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return Context(0)


def gpu_closest(sc, rays):
    d_rays = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    d_hits = torch.empty((len(rays), 4), dtype=torch.int32, device="cuda")
    sc.trace_closest(d_rays, d_hits)
    sc.sync()
    return d_hits.cpu().numpy().view(np.uint32).reshape(-1).view(oracle_lib.HIT_DTYPE)


def gpu_any(sc, rays):
    d_rays = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    d_bits = torch.zeros(((len(rays) + 31) // 32,), dtype=torch.int32, device="cuda")
    sc.trace_any(d_rays, d_bits)
    sc.sync()
    bits = d_bits.cpu().numpy().view(np.uint32)
    return ((bits[np.arange(len(rays)) >> 5] >> (np.arange(len(rays)) & 31).astype(np.uint32)) & 1).astype(np.uint8)


def assert_hits_equal(got, want):
    assert np.array_equal(got["prim"], want["prim"]), \
        f"{(got['prim'] != want['prim']).sum()} of {len(got)} primitive ids differ"
    hit = want["prim"] != 0xFFFFFFFF
    for k in ("t", "u", "v"):
        g, w = got[k][hit], want[k][hit]
        np.testing.assert_allclose(g, w, rtol=T_RTOL, atol=1e-7 if k != "t" else 0.0)


def _tri_rays(o, d, tmin=0.0, tmax=1e30):
    o = np.atleast_2d(np.asarray(o, np.float32))
    d = np.atleast_2d(np.asarray(d, np.float32))
    r = np.zeros((max(len(o), len(d)), 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def test_small_scene_matches_oracle(ctx, oracle):
    arrays = procedural.traversal_scene(sphere_freq=40, n_random=20000, seed=1)
    sc = GpuScene(ctx, arrays)
    st = sc.build()
    assert st.num_tris == arrays.num_tris and st.num_nodes > 0 and 1 <= st.max_depth <= 49
    rays = np.concatenate([procedural.incoherent_rays(arrays, 65536, seed=3),
                           procedural.primary_rays(128, 128, pos=(0.0, 0.0, -4.0))])
    b = oracle.bvh(arrays.tri_verts())
    got = gpu_closest(sc, rays)
    want = b.closest(rays)
    assert_hits_equal(got, want)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), "t/u/v not bit-identical to the oracle"
    short = rays.copy()
    short[:, 7] = 0.5
    assert np.array_equal(gpu_any(sc, short), b.any(short))


@pytest.mark.parametrize("leaf_max,rounds", [(1, 0), (2, 0), (3, 0), (3, 0xFFFFFFFF), (2, 6)])
def test_leaf_sizes_and_treelet_rounds(ctx, oracle, leaf_max, rounds):
    arrays = procedural.traversal_scene(sphere_freq=12, n_random=3000, seed=4)
    sc = GpuScene(ctx, arrays)
    sc.build(leaf_max=leaf_max, treelet_rounds=rounds)
    rays = procedural.incoherent_rays(arrays, 20000, seed=9)
    assert_hits_equal(gpu_closest(sc, rays), oracle.bvh(arrays.tri_verts()).closest(rays))


def _scene_from_tris(tv):
    from lumen_gb300.procedural import _Builder
    from lumen_gb300.scene import LIGHT_DTYPE, diffuse
    b = _Builder()
    b.add(tv.reshape(-1, 3, 3).astype(np.float64), np.tile(np.array([0, 0, 1.0]), (len(tv), 3, 1)), 0)
    return b.arrays([diffuse((0.5, 0.5, 0.5))], np.zeros(0, LIGHT_DTYPE), 0, (0, 0, 0), (0, 0, 1), 45.0)


def test_watertight_edges_ties_and_parallel_rays(ctx, oracle):
    n = 16
    ang = np.linspace(0, 2 * np.pi, n + 1)
    ring = np.stack([np.cos(ang), np.sin(ang), np.zeros_like(ang)], -1).astype(np.float32)
    fan = np.zeros((n, 9), np.float32)
    for i in range(n):
        fan[i, 3:6] = ring[i]
        fan[i, 6:9] = ring[i + 1]
    dup = np.array([[-1, -1, 2, 1, -1, 2, 0, 1, 2]] * 3, np.float32)   # coincident: lowest id must win
    tv = np.concatenate([fan, dup])
    arrays = _scene_from_tris(tv)
    sc = GpuScene(ctx, arrays)
    sc.build()
    pts = [(0.0, 0.0)] + [(r * np.cos(2 * np.pi * i / n), r * np.sin(2 * np.pi * i / n))
                          for i in range(n) for r in (0.25, 0.5, 0.999)]
    rays = [_tri_rays([(x, y, 1.0) for x, y in pts], (0, 0, -1)),
            _tri_rays([(0.1, 0.0, 5.0), (0.0, 0.0, 2.5)], (0, 0, -1)),
            _tri_rays([(-5, 0.25, 2.0), (0.5, -5, 0.0)], [(1, 0, 0), (0, 1, 0)]),
            _tri_rays([(0, 0, 1)] * 3, (0, 0, -1), tmin=2.0, tmax=1.0)]  # empty interval
    rays = np.concatenate(rays)
    got = gpu_closest(sc, rays)
    want = oracle.brute_closest(arrays.tri_verts(), rays)
    assert_hits_equal(got, want)
    assert (got["prim"][:len(pts)] < n).all(), "a ray through a shared vertex or edge leaked"
    assert got["prim"][len(pts)] == n  # first of the coincident triangles
    assert np.array_equal(gpu_any(sc, rays), oracle.brute_any(arrays.tri_verts(), rays))


def test_zero_rays_and_error_paths(ctx):
    arrays = procedural.traversal_scene(sphere_freq=4, n_random=10, seed=5)
    sc = GpuScene(ctx, arrays)
    d_rays = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    d_hits = torch.zeros((4, 4), dtype=torch.int32, device="cuda")
    with pytest.raises(abi.LgbError) as e:
        sc.trace_closest(d_rays, d_hits)  # before lgb_bvh_build
    assert e.value.status == 4
    sc.build()
    sc.trace_closest(d_rays, d_hits, n=0)
    with pytest.raises(abi.LgbError) as e:
        sc.trace_closest(d_rays[:, 1:], d_hits)  # 4-byte-offset ray buffer
    assert e.value.status == 1
    sc.sync()


def test_rebuild_is_query_equivalent(ctx):
    arrays = procedural.traversal_scene(sphere_freq=20, n_random=5000, seed=6)
    rays = procedural.incoherent_rays(arrays, 30000, seed=1)
    sc = GpuScene(ctx, arrays)
    sc.build()
    a = gpu_closest(sc, rays)
    b = gpu_closest(sc, rays)
    sc.build()
    c = gpu_closest(sc, rays)
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_full_size_traversal_config(ctx, oracle):
    """The 1M-triangle configuration: 1M primary + 4M incoherent closest-hit rays and 4M any-hit rays at
    tmax 0.5. Every ray is checked with size-independent properties; a 65 536-ray sample against the oracle."""
    arrays = procedural.traversal_scene()
    sc = GpuScene(ctx, arrays)
    st = sc.build()
    assert st.num_tris == 1_000_000
    inc = procedural.incoherent_rays(arrays, 4_000_000, seed=3)
    prim = procedural.primary_rays(1024, 1024, pos=(0.0, 0.0, -4.0))
    rays = np.concatenate([prim, inc])
    got = gpu_closest(sc, rays)
    hit = got["prim"] != 0xFFFFFFFF
    assert (got["prim"][hit] < 1_000_000).all()
    assert (got["t"][hit] >= rays[hit, 3]).all() and (got["t"][hit] <= rays[hit, 7]).all()
    assert (got["u"][hit] >= 0).all() and (got["v"][hit] >= 0).all() and (got["u"][hit] + got["v"][hit] <= 1.0 + 1e-6).all()
    assert hit[:len(prim)].mean() > 0.2
    short = inc.copy()
    short[:, 7] = 0.5
    occ = gpu_any(sc, short)
    near = (got["prim"][len(prim):] != 0xFFFFFFFF) & (got["t"][len(prim):] <= 0.5)
    assert np.array_equal(occ.astype(bool), near), "occlusion disagrees with the closest hit on the same rays"
    rng = np.random.default_rng(0)
    sample = rng.choice(len(rays), 65536, replace=False)
    b = oracle.bvh(arrays.tri_verts())
    assert_hits_equal(got[sample], b.closest(rays[sample]))


@pytest.mark.parametrize("n", [1, 31, 33, 70_000, 1_300_001])
def test_host_buffer_queries_equal_device_queries(ctx, n):
    """lgb_trace_closest_host / lgb_trace_any_host (chunked copies overlapped with traversal) give exactly the
    device-buffer results, for one chunk, ragged sizes and several chunks (the last one partial)."""
    arrays = procedural.traversal_scene(sphere_freq=40, n_random=20000, seed=7)
    sc = GpuScene(ctx, arrays)
    sc.build()
    rays = procedural.incoherent_rays(arrays, n, seed=11)
    rays[:, 7] = np.where(np.arange(n) % 2 == 0, 0.5, rays[:, 7])  # half short rays: mixed occlusion
    want = gpu_closest(sc, rays)
    want_occ = gpu_any(sc, rays)
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.full((n, 4), -7, dtype=torch.int32).pin_memory()
    h_bits = torch.full(((n + 31) // 32,), -1, dtype=torch.int32).pin_memory()
    sc.trace_closest_host(h_rays, h_hits)
    sc.trace_any_host(h_rays, h_bits)
    sc.sync()
    got = h_hits.numpy().view(np.uint32).reshape(-1).view(oracle_lib.HIT_DTYPE)
    assert np.array_equal(got, want)
    bits = h_bits.numpy().view(np.uint32)
    occ = ((bits[np.arange(n) >> 5] >> (np.arange(n) & 31).astype(np.uint32)) & 1).astype(np.uint8)
    assert np.array_equal(occ, want_occ)
    assert 0 < occ.sum() < n or n < 100
    # pageable host memory works too (the copies are then synchronous)
    h2 = torch.zeros((n, 4), dtype=torch.int32)
    sc.trace_closest_host(torch.from_numpy(rays), h2)
    sc.sync()
    assert np.array_equal(h2.numpy().view(np.uint32).reshape(-1).view(oracle_lib.HIT_DTYPE), want)


def test_host_buffer_query_errors(ctx):
    arrays = procedural.traversal_scene(sphere_freq=8, n_random=100, seed=2)
    sc = GpuScene(ctx, arrays)
    rays = torch.zeros((4, 8), dtype=torch.float32)
    hits = torch.zeros((4, 4), dtype=torch.int32)
    with pytest.raises(abi.LgbError):
        sc.trace_closest_host(rays, hits)  # no BVH yet
    sc.build()
    import ctypes as C
    with pytest.raises(abi.LgbError):
        from lumen_gb300.scene import _check
        _check(sc.lib, sc.ctx.handle, sc.lib.lgb_trace_closest_host(sc.handle, None, C.c_void_p(hits.data_ptr()), 4, None))
    sc.trace_closest_host(rays[:0], hits[:0])  # zero rays: nothing to do
    sc.sync()


def test_context_outlives_its_scenes_whatever_the_destroy_order(ctx):
    """lgb_destroy of a context that scenes and batches still use only marks it; the last lgb_scene_destroy /
    lgb_batch_destroy frees it (a garbage collector may finalise the context first). No CUDA error is left behind."""
    import ctypes as C
    from lumen_gb300.scene import Batch
    lib = abi.load()
    own = Context(0)
    arrays = procedural.traversal_scene(sphere_freq=8, n_random=200, seed=5)
    sc = GpuScene(own, arrays)
    sc.build()
    batch = Batch(own, [sc])
    lib.lgb_destroy(own.handle)  # the context goes first
    own.handle = None
    batch.close()
    sc.close()
    rays = procedural.incoherent_rays(arrays, 1000, seed=2)
    other = GpuScene(ctx, arrays)  # another context keeps working, with no stale error
    other.build()
    hits = gpu_closest(other, rays)
    assert (hits["prim"] != 0xFFFFFFFF).any()
    other.close()


def test_visit_budget_sets_the_device_status_word(ctx, oracle):
    """The error path of the bounded traversal loop, driven without any fault: a per-ray budget of 2 node visits
    runs out on a sound 100k-triangle tree, the kernel sets the visit-limit bit of the scene's status word and
    every ray ends; lgb_sync reports LGB_ERR_DEVICE_STATUS once and clears the word, and with the default budget
    restored the same query is clean and equals the oracle."""
    arrays = procedural.traversal_scene(sphere_freq=60, n_random=30_000)
    rays = procedural.incoherent_rays(arrays, 50_000, seed=9)
    sc = GpuScene(ctx, arrays)
    sc.build()
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.zeros((len(rays), 4), dtype=torch.int32, device="cuda")
    sc.set_visit_limit(2)
    sc.trace_closest(d_rays, d_hits)
    with pytest.raises(abi.LgbError) as e:
        sc.sync()
    assert e.value.status == 5 and "visit limit" in str(e.value)
    d_bits = torch.zeros(((len(rays) + 31) // 32,), dtype=torch.int32, device="cuda")
    sc.trace_any(d_rays, d_bits)
    with pytest.raises(abi.LgbError):
        sc.sync()
    sc.sync()  # the word was cleared by the failing sync
    sc.set_visit_limit(0)
    got = gpu_closest(sc, rays)
    assert_hits_equal(got, oracle.bvh(arrays.tri_verts()).closest(rays))
