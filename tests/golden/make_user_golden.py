"""Generate tests/golden/user_shader.json: the reference library itself running shader
classes it does not ship (tests/cpp/user_shaders.h) on the seeded scenes of
tests/cpp/user_scene.h.

oracle/user_shader_ref.cpp compiles the reference's src/renderer sources unmodified with
those classes (make -C oracle user-ref; needs SWR_REFERENCE naming the reference checkout)
and writes each case's framebuffer; this script records a SHA-256 of its colour, depth and
per-pixel drawPixel-count buffers.  The GPU test (tests/test_user_shader.py) draws the same
classes through include/swr/Renderer.h and the C ABI and compares.

    SWR_REFERENCE=/path/to/SoftwareRenderer python tests/golden/make_user_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "user_shader.json")
W, H = 320, 240


def split(raw):
    n = W * H * 4
    return {"color": raw[:n], "depth": raw[n:2 * n], "count": raw[2 * n:3 * n]}


def digest(raw):
    return {k: hashlib.sha256(v).hexdigest()[:32] for k, v in split(raw).items()}


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "user-ref"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "user_shader_ref")
    cases = []
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([exe, d], check=True, stdout=subprocess.DEVNULL)
        k = 0
        while os.path.exists(os.path.join(d, f"{k}_ref.bin")):
            raw = open(os.path.join(d, f"{k}_ref.bin"), "rb").read()
            cnt = memoryview(split(raw)["count"]).cast("I")
            cases.append({"case": k, "sha256": digest(raw), "fragments": int(sum(cnt)),
                          "pixels": int(sum(1 for c in cnt if c))})
            k += 1
    with open(OUT, "w") as f:
        json.dump({"generator": "reference library (src/renderer) via oracle/user_shader_ref.cpp",
                   "width": W, "height": H, "cases": cases}, f, indent=1)
    print(f"{len(cases)} cases -> {OUT}")


if __name__ == "__main__":
    sys.exit(main())
