"""Generates tests/golden/cornell_256_fp64_ref.npy: the Cornell-box configuration (256 x 256, max depth 8)
rendered by the CPU oracle in FP64 with 2048 samples per pixel (frames 0-2047 of the same per-pixel RNG
streams). It is the converged reference that bench.py and the tests measure RMSE against.

Run:  python tests/golden/make_cornell_reference.py  (about a minute on 8 cores)
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

W = H = 256
SPP = 2048
DEPTH = 8


class Cam:
    pass


def main():
    ora = oracle_lib.Oracle()
    cb = procedural.cornell_box()
    cam = Cam()
    cam.inv_view, cam.inv_projection = ora.camera(cb.camera_pos, cb.camera_dir, cb.fov, W, H)
    sc = ora.scene(cb)
    t0 = time.time()
    film = sc.film(cam, DEPTH, W, H, 0, SPP, fp64=True)
    img = film[:, :3].reshape(H, W, 3).astype(np.float32)
    np.save(os.path.join(HERE, "cornell_256_fp64_ref.npy"), img)
    print(f"done in {time.time() - t0:.1f} s, mean {img.mean(axis=(0, 1))}")


if __name__ == "__main__":
    main()
