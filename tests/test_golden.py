"""Golden vectors from the reference itself (tests/golden/make_golden.py): the reference host
code's BVH arrays (as SHA-256 digests) and the reference GLSL path tracer's per-path radiance
(compiled for the CPU). The product's host layer must reproduce the arrays and the oracle
must reproduce every path exactly."""
import json

import numpy as np
import pytest

import oracle
from tests.conftest import ROOT
from tests.golden import cases

GOLD = ROOT / "tests" / "golden"
META = json.loads((GOLD / "scenes.json").read_text())
PATHS = np.load(GOLD / "shader_paths.npz")


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_scene_arrays_match_reference_digests(name):
    a, p, extras = cases.build(name)
    m = META[name]
    for k in cases.KEYS:
        assert cases.digest(a[k]) == m["digests"][k], k
    assert int(a["top_level_index"]) == m["top_level_index"]


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_oracle_paths_equal_reference_shader(name):
    a, _, extras = cases.build(name)
    p = cases.stored_params(META[name])
    view, keep = cases.make_view(a, extras)
    spp = cases.CASES[name]
    acc, paths, _ = oracle.render(view, p, 0, spp, want_paths=True)
    gold = PATHS[name]
    assert paths.shape == gold.shape
    same = np.all((paths == gold) | (np.isnan(paths) & np.isnan(gold)), axis=-1)
    assert same.all(), f"{(~same).sum()} of {same.size} paths differ"


def test_oracle_postprocess_equals_reference_shader():
    """The display pass (postprocess.glsl:126-171 with TiledRenderer's uniforms) against the
    reference shader compiled for the CPU: every tone map, CA form, vignette and the preview
    path, bit for bit."""
    gold = np.load(GOLD / "postprocess.npz")
    acc = gold["input"]
    settings = cases.post_settings()
    assert len(gold.files) == len(settings) + 1
    for k, q in enumerate(settings):
        _, rgbf = oracle.postprocess(acc, q, cases.POST_SAMPLES)
        ref = gold[f"setting{k}"]
        same = (rgbf.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(rgbf) & np.isnan(ref))
        assert same.all(), f"setting {k} (tone map {q.tonemap}): {(~same).sum()} values differ"
