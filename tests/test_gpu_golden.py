"""The CUDA pipeline against fixtures generated by the reference library itself.

Same cases as test_oracle_golden.py (seeded scenes rebuilt from their specs, inputs
checked bit-identical), rendered on the GPU: counters and SHA-256 of colour, depth,
per-pixel drawPixel count and winning primitive must equal the reference's.  Includes the
full-size configurations: all 100 textured-cube frames, all 32 icosphere-7 poses at 1080p,
the 1,048,576-triangle soup at 3840x2160, and the Benchmark.cpp-shaped scene.
"""
import pytest

from softwarerenderer_gb300 import scenes

from .golden_cases import cases, case_id, digest
from .parity import gpu_render

pytestmark = pytest.mark.gpu
CASES = cases()


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_gpu_matches_reference_fixture(gpu_lib, case):
    sc = scenes.scene_from_spec(case["spec"])
    assert scenes.scene_digest(sc) == case["inputs"], "scene inputs differ from the fixture's"
    got, st = gpu_render(sc)
    assert int(st["fragments"]) == case["stats"]["fragments"]
    assert digest(got) == case["sha256"]
