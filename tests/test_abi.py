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
    assert lib.lgb_abi_version() == 2


def test_struct_layouts():
    assert C.sizeof(abi.Ray) == 32
    assert C.sizeof(abi.Hit) == 16
    assert C.sizeof(abi.Material) == 104
    assert C.sizeof(abi.Light) == 128
    assert C.sizeof(abi.Mesh) == 16
    assert C.sizeof(abi.Camera) == 136
    assert C.sizeof(abi.PathParams) == 48
    assert C.sizeof(abi.BuildStats) == 56
    assert C.sizeof(abi.DiffParams) == 32
    assert C.sizeof(abi.DiffGrads) == 24
    assert C.sizeof(abi.BatchJob) == 208
    assert C.sizeof(abi.BatchOpts) == 32
    assert C.sizeof(abi.SppmParams) == 64
    assert C.sizeof(abi.RestirParams) == 64
    assert C.sizeof(abi.BdptParams) == 64


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


def test_ctypes_layouts_match_the_header(tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler gives the header's struct."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"lgb_ray": abi.Ray, "lgb_hit": abi.Hit, "lgb_material": abi.Material, "lgb_light": abi.Light,
               "lgb_mesh": abi.Mesh, "lgb_camera": abi.Camera, "lgb_path_params": abi.PathParams,
               "lgb_build_opts": abi.BuildOpts, "lgb_build_stats": abi.BuildStats, "lgb_diff_params": abi.DiffParams,
               "lgb_diff_grads": abi.DiffGrads, "lgb_batch_job": abi.BatchJob, "lgb_batch_opts": abi.BatchOpts,
               "lgb_vcm_params": abi.VcmParams, "lgb_sppm_params": abi.SppmParams,
               "lgb_restir_params": abi.RestirParams, "lgb_bdpt_params": abi.BdptParams}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lgb.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, *_ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I" + inc, str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                          text=True).stdout.splitlines())
    for cname, py in mirrors.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for fname, *_ in py._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(py, fname).offset, f"{cname}.{fname}"
