"""Shaders the library does not ship, through the reference's C++ API and the C ABI.

tests/cpp/user_shader_test.cu defines its own VertexShaderBase / PixelShaderBase classes
(tests/cpp/user_shaders.h: two attribute streams, four affine and three perspective
variables, a pixel shader that depth-tests into its own buffers and reads
PixelData::computePerspectiveDerivatives, and an order-only one), draws them with
swr::Rasterizer / swr::VertexProcessor from include/swr/Renderer.h (setPixelShader<PS>(),
setVertexShader<VS>(), drawElements, drawTriangleList) and with swr_set_vertex_program /
swr_set_pixel_program through the C ABI.  Both must equal, bit for bit, the reference
library running the same classes (tests/golden/user_shader.json, made by
tests/golden/make_user_golden.py): colour, depth and per-pixel drawPixel count, for
triangles in all raster and cull modes (with near-plane clipping and 1024-primitive
batches), lines, points and the direct rasterizer path.
"""
import hashlib
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "softwarerenderer_gb300", "_build")
EXE = os.path.join(BUILD, "user_shader_test")
SRC = os.path.join(ROOT, "tests", "cpp", "user_shader_test.cu")
GOLDEN = os.path.join(ROOT, "tests", "golden", "user_shader.json")


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def build_program():
    """Compile the test program the way an application would: its own nvcc unit, the
    library's flags for exact binary32 arithmetic, linked against libswr_gb300.so."""
    from softwarerenderer_gb300 import build
    lib = build.build()
    deps = [SRC, lib, os.path.join(ROOT, "include", "swr", "Renderer.h"),
            os.path.join(ROOT, "tests", "cpp", "user_shaders.h"), os.path.join(ROOT, "tests", "cpp", "user_scene.h")]
    deps += [os.path.join(build.CSRC, f) for f in os.listdir(build.CSRC) if f.endswith((".h", ".cuh"))]
    if os.path.exists(EXE) and all(os.path.getmtime(d) <= os.path.getmtime(EXE) for d in deps):
        return EXE
    cmd = [_nvcc(), *build.ARCH, "-O3", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
           "-ftz=false", "--expt-relaxed-constexpr", "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "tests", "cpp"), SRC,
           "-L", BUILD, "-lswr_gb300", "-Xlinker", "-rpath=" + BUILD, "-o", EXE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return EXE


def test_user_shader_program_builds():
    """The header-only front-end compiles a caller's own shaders into the pipeline."""
    if _nvcc() is None:
        pytest.skip("nvcc not found")
    assert os.path.exists(build_program())


@pytest.mark.gpu
def test_user_shaders_match_the_reference(gpu_lib, tmp_path):
    exe = build_program()
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    golden = json.load(open(GOLDEN))
    w, h = golden["width"], golden["height"]
    n = w * h * 4
    for case in golden["cases"]:
        k = case["case"]
        raws = {}
        for path in ("template", "capi"):
            raw = open(os.path.join(tmp_path, f"{k}_{path}.bin"), "rb").read()
            assert len(raw) == 3 * n
            got = {name: hashlib.sha256(raw[i * n:(i + 1) * n]).hexdigest()[:32]
                   for i, name in enumerate(("color", "depth", "count"))}
            assert got == case["sha256"], (k, path, got, case["sha256"])
            raws[path] = raw
        assert raws["template"] == raws["capi"], k
