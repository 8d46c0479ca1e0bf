"""Generates tests/golden/diff_512_fp64_ref.npy: the differentiable configuration's scene (Cornell box with a
64 x 64 albedo texture on the back wall and two GGX conductor boxes; 512 x 512, max depth 6) rendered by the CPU
oracle's differentiable estimator in FP64 with 512 samples per pixel (frames 0-511 of the per-pixel RNG
streams), scene parameters unchanged. It is the converged reference that bench.py and the tests measure the
primal's RMSE against.

Run:  python tests/golden/make_diff_reference.py  (about a minute on 8 cores)
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
from lumen_gb300.scene import camera_lookat  # noqa: E402

W = H = 512
SPP = 512
DEPTH = 6


def main():
    ora = oracle_lib.Oracle()
    arrays = procedural.cornell_diff()
    cam = camera_lookat(arrays.camera_pos, arrays.camera_dir, arrays.fov, W, H)
    t0 = time.time()
    img = ora.scene(arrays).diff(cam, DEPTH, W, H, 0, SPP, fp64=True)
    img = img.reshape(H, W, 3).astype(np.float32)
    np.save(os.path.join(HERE, "diff_512_fp64_ref.npy"), img)
    print(f"done in {time.time() - t0:.1f} s, mean {img.mean(axis=(0, 1))}")


if __name__ == "__main__":
    main()
