"""CPU tests of bench.py's CPU-oracle legs (the cpu_baseline entries beside the VCM, SPPM, ReSTIR DI and BDPT
measurements): each runs on a tiny image and reports a positive rate in the bench's format."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("kind", ["vcm", "sppm", "restir_di", "bdpt"])
def test_cpu_integrator_rate(kind):
    sys.path.insert(0, ROOT)
    import bench
    from lumen_gb300 import abi, procedural
    if kind == "vcm":
        arrays, kw = procedural.vcm_scene(40, 16), {"spot_angle": 20.0}
    else:
        arrays = procedural.cornell_box()
        kw = {"base_radius": 0.03} if kind == "sppm" else ({"flags": abi.RESTIR_SPATIAL_COUNT_FIX} if kind == "restir_di" else {})
    out = bench.cpu_integrator_rate(kind, arrays, 8, 8, 2, 4, **kw)
    assert out["value"] > 0.0 and out["unit"] == "Msamples/s" and out["kind"] == "port" and out["cores"] >= 1
    assert "8x8" in out["sample"]
