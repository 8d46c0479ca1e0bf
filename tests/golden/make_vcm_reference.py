"""Generates tests/golden/vcm_torus_256_fp64_ref.npy: the VCM caustics configuration (dielectric torus, 200k
triangles, on a diffuse plane; spot light with a 20 degree cone; max depth 10; merge radius 0.01 x scene radius
shrinking with alpha = 0.75) at 256 x 256, 2048 iterations of the CPU oracle's VCM in FP64 (light seeds
100000 + i, eye seeds 500000 + i: independent of the seeds 1000 + i / 5000 + i the GPU renders use). Ray queries,
random numbers and the photon table's cell keys are FP32 as in every oracle render; the shading, MIS and film
arithmetic is FP64. bench.py and the tests measure the RMSE of 64 GPU iterations against it.

Run:  python tests/golden/make_vcm_reference.py  (about six minutes on 8 cores)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle_lib  # noqa: E402
from lumen_gb300 import procedural  # noqa: E402
from lumen_gb300.scene import camera_forward, camera_lookat, scene_radius, vcm_params, vcm_radius  # noqa: E402

W = H = 256
ITERS = 2048
DEPTH = 10
SPOT = 20.0
ALPHA = 0.75


def oracle_params(arrays, it):
    p = vcm_params(arrays, DEPTH, vcm_radius(scene_radius(arrays), 1.0, it, ALPHA), 100000 + it, 500000 + it, it,
                   spot_angle=SPOT)
    op = oracle_lib.VcmParams()
    for name in ("max_depth", "num_lights", "light_triangle_count", "radius", "use_vm", "use_vc", "light_seed",
                 "eye_seed", "frame_num", "flags", "spot_angle"):
        setattr(op, name, getattr(p, name))
    op.sky_col[:] = list(p.sky_col)
    op.scene_min[:] = list(p.scene_min)
    op.scene_max[:] = list(p.scene_max)
    return op


def main():
    ora = oracle_lib.Oracle()
    arrays = procedural.vcm_scene()
    sc = ora.scene(arrays)
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, W, H)
    view, proj = camera_forward(cam)
    t0 = time.time()
    film = sc.vcm_render_f64(cam, view, proj, [oracle_params(arrays, it) for it in range(ITERS)])
    img = film[:, :3].reshape(H, W, 3).astype(np.float32)
    np.save(os.path.join(HERE, "vcm_torus_256_fp64_ref.npy"), img)
    print(f"done in {time.time() - t0:.1f} s, mean {img.mean(axis=(0, 1))}")


if __name__ == "__main__":
    main()
