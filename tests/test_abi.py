"""CPU tests of the C ABI boundary: liblgb.so loads, exports every function include/lgb.h declares, its
struct layouts match the header, and the host-only camera helper agrees with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from lumen_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    return abi.load()


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "lgb.h")).read()
    return re.findall(r"LGB_API\s+[\w\s\*]+?\b(lgb_\w+)\s*\(", src)


def test_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), f"{n} is declared in lgb.h but not exported"
        assert n in abi.SIGNATURES, f"{n} has no ctypes signature"
    assert set(abi.SIGNATURES) == set(names)
    assert lib.lgb_abi_version() == 1


def test_struct_layouts():
    assert C.sizeof(abi.Ray) == 32
    assert C.sizeof(abi.Hit) == 16
    assert C.sizeof(abi.Material) == 104
    assert C.sizeof(abi.Light) == 128
    assert C.sizeof(abi.Mesh) == 16
    assert C.sizeof(abi.Camera) == 136
    assert C.sizeof(abi.PathParams) == 48
    assert C.sizeof(abi.BuildStats) == 56


def test_camera_lookat_matches_oracle(lib, oracle):
    from lumen_gb300.scene import camera_lookat
    for pos, d, fov, w, h in [((0, 0, 3.5), (0, 0, 1), 45.0, 256, 256), ((0.7, 0.5, 17.5), (0, 0, 2), 45, 1280, 720),
                              ((1, 2, 3), (-1, 0.2, 0.3), 60, 100, 50)]:
        cam = camera_lookat(pos, d, fov, w, h)
        iv, ip = oracle.camera(pos, d, fov, w, h)
        np.testing.assert_allclose(np.array(cam.inv_view[:]), iv, rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(np.array(cam.inv_projection[:]), ip, rtol=1e-6, atol=1e-6)


def test_camera_lookat_rejects_bad_arguments(lib):
    cam = abi.Camera()
    p = (C.c_float * 3)(0, 0, 0)
    up = (C.c_float * 3)(0, 1, 0)
    assert lib.lgb_camera_lookat(p, up, 45.0, 16, 16, C.byref(cam)) == 1  # looking straight up
    assert lib.lgb_camera_lookat(p, (C.c_float * 3)(0, 0, 1), 0.0, 16, 16, C.byref(cam)) == 1
    assert lib.lgb_camera_lookat(p, (C.c_float * 3)(0, 0, 1), 45.0, 0, 16, C.byref(cam)) == 1


def test_null_handles_are_rejected(lib):
    assert lib.lgb_bvh_build(None, None, None) == 1
    assert lib.lgb_trace_closest(None, None, None, 0, None) == 1
    assert lib.lgb_sync(None, None) == 1
    assert lib.lgb_last_error(None) == b"null context"
