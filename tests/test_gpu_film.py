"""GPU tests of lgb_film_rmse: the true RMSE (mode 0) and the value Lumen reports (mode 1: per 1024-pixel
group the minimum of its 32-pixel warp sums, calc_rmse.comp:37, then sqrt(sum) / (3 N), output_rmse.comp:23),
each against a numpy restatement."""
import os

import numpy as np
import pytest

from lumen_gb300 import abi, build
from lumen_gb300.scene import Context, film_rmse

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def lumen_reported(a, b):
    d = ((b[:, :3] - a[:, :3]) ** 2).sum(1).astype(np.float64)
    n = len(d)
    total = 0.0
    for g in range(0, n, 1024):
        grp = d[g:g + 1024]
        warps = [grp[w:w + 32].sum() for w in range(0, len(grp), 32)]
        total += min(warps)
    return np.sqrt(total) / (3 * n)


@pytest.mark.parametrize("n", [1, 1000, 4096, 70001])
def test_rmse_modes(n):
    if not os.path.exists(abi.LIB_PATH):
        build.build_library()
    ctx = Context(0)
    rng = np.random.default_rng(n)
    a = rng.random((n, 4)).astype(np.float32)
    b = (a + rng.normal(0, 0.1, (n, 4))).astype(np.float32)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    want = np.sqrt(((b[:, :3].astype(np.float64) - a[:, :3]) ** 2).sum() / (3 * n))
    np.testing.assert_allclose(film_rmse(ctx, da, db, 0), want, rtol=1e-6)
    np.testing.assert_allclose(film_rmse(ctx, da, db, 1), lumen_reported(a, b), rtol=1e-5)
    assert film_rmse(ctx, da, da, 0) == 0.0
