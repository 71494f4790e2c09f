"""GPU: meshes ingested from OBJ text feed the pipeline directly -- swr_obj_upload fills
device buffers identical to the host arrays, and the interleaved 32-byte records drawn as
two attribute streams render bit-exactly like the oracle."""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.obj import ObjMesh

from .parity import describe, diff, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mesh():
    return ObjMesh(scenes.icosphere_obj_text(4))


def test_upload_matches_host_arrays(gpu_lib, mesh):
    v, i = mesh.arrays()
    dv, di = mesh.upload()
    assert dv.cpu().numpy().tobytes() == v.tobytes()
    assert np.array_equal(di.cpu().numpy(), i)


@pytest.mark.parametrize("pose", [0, 1, 5, 9])
def test_obj_mesh_renders_like_oracle(gpu_lib, port, mesh, pose):
    v, i = mesh.arrays()
    sc = scenes.obj_scene(v, i, pose=pose)
    ref, rst = oracle_render(port, sc)
    got, gst = gpu_render(sc)
    bad = diff(ref, got)
    assert not bad, "; ".join(describe(ref, got, k) for k in bad)
    assert gst["fragments"] == rst["fragments"] > 0
