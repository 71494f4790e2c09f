"""Golden fixtures produced by the reference library itself (tests/golden/make_golden.py)."""
import hashlib
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    with open(os.path.join(HERE, "golden", "golden.json")) as f:
        return json.load(f)["cases"]


def digest(arrays):
    return {k: hashlib.sha256(memoryview(v).cast("B")).hexdigest()[:32] for k, v in arrays.items()}


def case_id(c):
    sp = c["spec"]
    return c["name"] + "".join(f"-{k}{v}" for k, v in sp.items() if k not in ("kind",))


HEAVY = ("soup1048576", "benchmark40960")
