"""OBJ ingestion (swr_obj_*, the reference examples' ObjData loader) and the examples'
random generator.  Parity: seeded OBJ texts covering the syntax the reference handles are
loaded by the reference's own ObjData (compiled by oracle/Makefile, where the reference
checkout exists) and by the library; vertex and index arrays must agree bit for bit.
The subtractive generator behind the Benchmark scene is pinned the same way."""
import os

import numpy as np
import pytest

from softwarerenderer_gb300 import _lib, scenes
from softwarerenderer_gb300.obj import ObjMesh, load_obj


def _fmt(rng, x):
    k = int(rng.integers(0, 6))
    if k == 0:
        return f"{x:.6f}"
    if k == 1:
        return f"{x:g}"
    if k == 2:
        return f"{x:e}"
    if k == 3:
        return f"{x:+.3f}"
    if k == 4:
        return repr(float(np.float32(x)))
    return f"{x:.9g}"


def obj_text(seed):
    """A seeded OBJ file: positions, normals, texcoords in assorted number formats, faces of
    3 to 6 vertices in every reference form, comments, blank and unknown lines, CRLF and
    tab separators, one- and two-vertex faces."""
    rng = np.random.default_rng(seed)
    nv, nn, nt = (int(x) for x in rng.integers(1, 40, 3))
    eol = "\r\n" if seed % 3 == 0 else "\n"
    sep = lambda: " " if rng.random() < 0.8 else "\t"  # noqa: E731
    lines = ["# generated", "mtllib none.mtl", "o thing", ""]
    for _ in range(nv):
        xs = [_fmt(rng, v) for v in rng.normal(size=3 + int(rng.random() < 0.1))]
        lines.append("v" + "".join(sep() + x for x in xs))
    for _ in range(nn):
        lines.append("vn" + "".join(sep() + _fmt(rng, v) for v in rng.normal(size=3)))
    for _ in range(nt):
        lines.append("  vt" + "".join(sep() + _fmt(rng, v) for v in rng.random(2 + int(rng.random() < 0.2))))
    lines += ["g group", "s 1", "usemtl m"]
    for _ in range(int(rng.integers(5, 60))):
        k = int(rng.choice([1, 2, 3, 3, 3, 4, 4, 5, 6]))
        form = int(rng.integers(0, 4))
        words = []
        for _ in range(k):
            v = int(rng.integers(1, nv + 1))
            t = int(rng.integers(1, nt + 1))
            n = int(rng.integers(1, nn + 1))
            words.append([f"{v}", f"{v}/{t}", f"{v}//{n}", f"{v}/{t}/{n}"][form if rng.random() < 0.9 else int(rng.integers(0, 4))])
        lines.append("f " + " ".join(words))
        if rng.random() < 0.1:
            lines.append("# comment " + str(rng.random()))
        if rng.random() < 0.05:
            lines.append("")
    return (eol.join(lines) + (eol if seed % 2 else "")).encode()


@pytest.fixture(scope="module")
def ref():
    from oracle import oracle
    if not os.path.exists(oracle.PATHS["ref"]):
        pytest.skip("reference library not built (needs the reference checkout)")
    return oracle.load("ref")


@pytest.mark.parametrize("seed", range(40))
def test_obj_matches_reference(ref, tmp_path, seed):
    text = obj_text(seed)
    path = tmp_path / f"m{seed}.obj"
    path.write_bytes(text)
    rv, ri = ref.ref_obj(str(path))
    v, i = load_obj(str(path))
    assert v.tobytes() == rv.tobytes()
    assert np.array_equal(i, ri)
    v2, i2 = load_obj(text)  # the same text from memory
    assert v2.tobytes() == v.tobytes() and np.array_equal(i2, i)


def test_obj_fan_and_dedup():
    v, i = load_obj(b"v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0.5 0.25\nvn 0 0 1\n"
                    b"f 1/1/1 2/1/1 3/1/1 4/1/1\nf 1/1/1 3/1/1 4\n")
    assert np.array_equal(i, [0, 1, 2, 0, 2, 3, 0, 2, 4])
    assert v.shape == (5, 8)
    assert np.array_equal(v[0], [0, 0, 0, 0, 0, 1, 0.5, 0.25])
    assert np.array_equal(v[4], [0, 1, 0, 0, 0, 0, 0, 0])  # "4": zero normal and texcoord entries


def test_obj_short_faces_add_their_first_vertex():
    v, i = load_obj(b"v 1 2 3\nv 4 5 6\nf 2\nf 1 2\n")
    assert i.size == 0 and v.shape == (2, 8)
    assert np.array_equal(v[:, :3], [[4, 5, 6], [1, 2, 3]])


@pytest.mark.parametrize("text", [b"v 0 0 0\nf 1 2 3\n", b"v 0 0 0\nf 1/1/1/1 1 1\n", b"v 0 0 0\nf -1 1 1\n",
                                  b"v 0 0 0\nf\n", b"v 0 0 0\nvt 0 0\nf 1/2 1 1\n"])
def test_obj_rejects_undefined_inputs(text):
    with pytest.raises(_lib.SwrError) as e:
        ObjMesh(text)
    assert e.value.code == _lib.SWR_EINVAL


@pytest.mark.parametrize("seed", [0, 1, 42, -7, 2 ** 31 - 1, -2 ** 31])
def test_subtractive_random_matches_reference(ref, seed):
    want = ref.ref_random(seed, 5000)
    got = scenes.SubtractiveRandom(seed).next_doubles(5000)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
