"""The host loader on every JSON scene Lumen ships (scenes/**/*.json of the reference checkout): each loads, every
mesh references a material, and each material's type, albedo and emission follow the scene file the way
LumenScene::load_lumen_scene (LumenScene.cpp:231-513) reads them. The scene files are read where the reference
checkout is (LUMEN_REFERENCE_DIR); the test is skipped where there is none."""
import glob
import json
import os

import numpy as np
import pytest

from lumen_gb300 import abi

REF = os.environ.get("LUMEN_REFERENCE_DIR", "")
SCENES = sorted(glob.glob(os.path.join(REF, "scenes", "**", "*.json"), recursive=True)) if REF else []
TYPES = {"diffuse": abi.BSDF_DIFFUSE, "mirror": abi.BSDF_MIRROR, "glass": abi.BSDF_GLASS,
         "dielectric": abi.BSDF_DIELECTRIC, "conductor": abi.BSDF_CONDUCTOR, "principled": abi.BSDF_PRINCIPLED}


@pytest.mark.skipif(not SCENES, reason="no reference checkout with shipped scenes")
def test_every_shipped_json_scene_loads():
    from lumen_gb300 import host_scene
    for path in SCENES:
        arrays, info = host_scene.load_scene(path)
        with open(path) as f:
            j = json.load(f)
        name = os.path.relpath(path, REF)
        assert len(arrays.indices) % 3 == 0 and len(arrays.indices) > 0, name
        assert len(arrays.materials) == len(j["bsdfs"]), name
        assert (arrays.meshes["material_index"] < len(arrays.materials)).all(), name
        for m, b in zip(arrays.materials, j["bsdfs"]):
            assert m["bsdf_type"] == TYPES.get(b["type"], 0), (name, b["type"])
            if b["type"] in ("diffuse", "mirror", "glass") and "albedo" in b:
                np.testing.assert_allclose(m["albedo"], b["albedo"], rtol=1e-6, err_msg=name)
            np.testing.assert_allclose(m["emissive_factor"], b.get("emissive_factor", [0, 0, 0]), rtol=1e-6,
                                       err_msg=name)
        assert len(arrays.lights) >= len(j.get("lights", [])), name
