"""GPU test of lgb_render_path_noalloc, the path-integrator entry point that never allocates device memory.

Some callers cannot let a library call cudaMalloc while they render: a host that budgets all device memory
up front, or one that cannot take the device-wide synchronisation of cudaFree inside its frame loop. The
no-alloc entry point serves them from a fixed device array; this test checks through the C ABI that it
produces the same film as lgb_render_path on two calls in a row (the array keeps the previous call's
contents, so the second call checks that nothing stale leaks through), that the call leaves the device's
free memory unchanged, and that an image beyond its limit is refused. This file is collected last so that a
failure here cannot stop the rest of the suite.
"""
import ctypes as C
import os

import numpy as np
import pytest

from lumen_gb300 import abi, build, procedural
from lumen_gb300.scene import Context, GpuScene, camera_lookat, path_params

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _noalloc(sc, cam, params, frame0, spp, film):
    return sc.lib.lgb_render_path_noalloc(sc.handle, C.byref(cam), C.byref(params), frame0, spp,
                                          C.c_void_p(film.data_ptr()), None)


def test_noalloc_matches_allocating_entry_point():
    """Same kernels, same arena layout and same chunks of frames as lgb_render_path, so the films are equal bit
    for bit. On a fresh scene the no-alloc call comes first and must leave the device's free memory unchanged
    (lgb_render_path would allocate its arena on that first call); a warm-up call on another scene beforehand
    loads the library's kernels and looks the fixed array up, which is set-up, not a per-call allocation."""
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    ctx = Context(0)
    cb = procedural.cornell_box()
    w = h = 64
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, w, h)
    params = path_params(cb, 8)
    warm = GpuScene(ctx, cb)
    warm.build()
    scratch = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    assert _noalloc(warm, cam, params, 0, 1, scratch) == abi.LGB_OK
    warm.sync()
    sc = GpuScene(ctx, cb)
    sc.build()
    ref = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    got = torch.zeros((w * h, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for call, (frame0, spp) in enumerate(((0, 4), (4, 6))):  # two calls in a row, the second continuing the mean
        free_before = torch.cuda.mem_get_info()[0]
        st = _noalloc(sc, cam, params, frame0, spp, got)
        assert st == abi.LGB_OK, sc.lib.lgb_last_error(ctx.handle)
        sc.sync()
        assert torch.cuda.mem_get_info()[0] == free_before, "the no-alloc entry point allocated device memory"
        sc.render_path(cam, params, frame0, spp, ref)
        sc.sync()
        assert np.array_equal(got.cpu().numpy(), ref.cpu().numpy()), f"call {call}: films differ"
    assert float(got[:, :3].mean()) > 0.05


def test_noalloc_rejects_images_beyond_its_arena():
    ctx = Context(0)
    cb = procedural.cornell_box()
    sc = GpuScene(ctx, cb)
    sc.build()
    cam = camera_lookat(cb.camera_pos, cb.camera_dir, cb.fov, 256, 256)
    film = torch.zeros((256 * 256, 4), dtype=torch.float32, device="cuda")
    st = _noalloc(sc, cam, path_params(cb, 8), 0, 1, film)
    assert st == 1
    assert b"16384" in sc.lib.lgb_last_error(ctx.handle)
    sc.sync()
