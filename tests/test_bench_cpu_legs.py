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


def test_cpu_oracle_steps():
    """The one CPU-oracle timing method of the traversal line (cpu_baseline and --impl reference)."""
    sys.path.insert(0, ROOT)
    import bench
    from lumen_gb300 import procedural
    arrays = procedural.traversal_scene(sphere_freq=8, n_random=300)
    rays = procedural.incoherent_rays(arrays, bench.CPU_WINDOW + 1000, seed=3)
    vals, threads = bench.cpu_oracle_steps(arrays, rays, 2, 1)
    assert len(vals) == 2 and min(vals) > 0.0 and threads >= 1


def test_traffic_record_is_used_only_for_its_sources(tmp_path, monkeypatch):
    """bench.py takes the DRAM / L2 bytes of the committed ncu record only when the record names the SHA-256 of the
    traversal sources being run; a stale record gives nulls and says so."""
    import hashlib
    import json
    sys.path.insert(0, ROOT)
    import bench
    h = hashlib.sha256()
    for name in bench.TRAVERSAL_SOURCES:
        (tmp_path / os.path.dirname(name)).mkdir(parents=True, exist_ok=True)
        (tmp_path / name).write_bytes(name.encode())
        h.update(name.encode())
    (tmp_path / "profiles").mkdir()
    rec = {"source_sha256": h.hexdigest(), "dram_bytes_per_ray": 60.0, "l2_bytes_per_ray": 900.0, "command": "ncu x"}
    (tmp_path / "profiles" / "trace_closest_incoherent_1M.ncu.json").write_text(json.dumps(rec))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    got = bench.measured_traffic(1000)
    assert got["dram_bytes"] == 60000.0 and got["l2_bytes"] == 900000.0 and "ncu x" in got["source"]
    (tmp_path / bench.TRAVERSAL_SOURCES[0]).write_bytes(b"changed")
    got = bench.measured_traffic(1000)
    assert got["dram_bytes"] is None and got["l2_bytes"] is None and "stale" in got["source"]
