"""Generates tests/golden/batch_scene{1,13,21}_128_fp64_ref.npy: three scenes of the batched-rendering
configuration (procedural.batch_config(): scene 1 with 10 915 triangles, scene 13 with 66 573, scene 21 with
216 452; principled and dielectric materials, quad lights, max depth 12) rendered by the CPU oracle in FP64 at
128 x 128 with 2048 samples per pixel (frames 100000-102047, independent of the frames 0.. the GPU renders). They
are the converged references bench.py measures the batched and the scene-by-scene renders against.

Run:  python tests/golden/make_batch_references.py  (a few minutes on 8 cores)
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

SCENES = (1, 13, 21)
W = H = 128
SPP = 2048
DEPTH = 12
FRAME0 = 100000


class Cam:
    pass


def main():
    ora = oracle_lib.Oracle()
    cfg = procedural.batch_config()
    for idx in SCENES:
        seed, tris, _, _, _ = cfg[idx]
        arrays = procedural.batch_scene(seed, tris)
        cam = Cam()
        cam.inv_view, cam.inv_projection = ora.camera(arrays.camera_pos, arrays.camera_dir, arrays.fov, W, H)
        sc = ora.scene(arrays)
        t0 = time.time()
        img = sc.mean_f64(cam, DEPTH, W, H, FRAME0, SPP).reshape(H, W, 3).astype(np.float32)
        np.save(os.path.join(HERE, f"batch_scene{idx}_128_fp64_ref.npy"), img)
        print(f"scene {idx} ({tris} triangles) done in {time.time() - t0:.1f} s, mean {img.mean(axis=(0, 1))}")


if __name__ == "__main__":
    main()
