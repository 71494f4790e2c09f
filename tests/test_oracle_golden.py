"""The CPU oracle port against fixtures generated by the reference library itself.

Every case rebuilds its seeded scene, checks that the inputs are bit-identical to the ones
the fixture was made from, renders it with the port and compares the reference's counters
and the SHA-256 of colour, depth, per-pixel fragment count and winning primitive.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes

from .golden_cases import cases, case_id, digest

CASES = cases()


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_port_matches_reference_fixture(port, case):
    sc = scenes.scene_from_spec(case["spec"])
    assert scenes.scene_digest(sc) == case["inputs"], "scene inputs differ from the fixture's"
    tg = scenes.Target(sc)
    st = port.draw(sc, tg)
    assert {k: int(st[k]) for k in ("fragments", "outside", "primitives")} == case["stats"]
    assert digest(tg.arrays()) == case["sha256"]
