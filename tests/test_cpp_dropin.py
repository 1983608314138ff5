"""The C++ drop-in (mytrim_gb300/cpp/trim_gpu.h) compiles against the reference's
own headers and hands the reference objects to the C ABI unchanged."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_SRCS = ["element.C", "material.C", "sample.C", "ion.C", "trim.C", "simconf.C", "sample_solid.C",
            "sample_layers.C", "sample_clusters.C", "shim/point.C"]


def test_flatten_reference_objects(tmp_path):
    from conftest import REFERENCE
    if REFERENCE is None or not (REFERENCE / "trim.h").exists():
        pytest.skip("reference headers not present")
    exe = tmp_path / "flatten"
    subprocess.run(["g++", "-O1", "-std=c++17", f"-I{REFERENCE}", f"-I{ROOT / 'include'}",
                    f"-I{ROOT / 'mytrim_gb300' / 'cpp'}", f'-DMYTRIM_DATA_DIR="{REFERENCE / "data"}"',
                    str(ROOT / "tests" / "cpp" / "flatten_reference.cpp"),
                    *[str(REFERENCE / s) for s in REF_SRCS], "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = out[0].split()
    assert rows[1] == "92" and float(rows[2]) == 62.93 and float(rows[3]) == 1.066
    layers = out[1].split()
    assert layers[1] == "2" and float(layers[2]) == 100.0 and float(layers[3]) == 1000.0
    assert layers[5:8] == ["2", "0", "0"]
    el = [l.split() for l in out if l.startswith("el ")]
    assert [(int(e[4]), float(e[7])) for e in el] == [(14, 15.0), (8, 28.0), (14, 15.0)]
    ion = [l for l in out if l.startswith("ion ")][0].split()
    assert ion[1] == "33" and float(ion[3]) == 50000.0 and float(ion[4]) == 5.0
    cl = [l for l in out if l.startswith("clusters ")][0].split()
    # geometry 1, two materials, two clusters, hash 8x6x4, second centre x, second radius
    assert cl[1:7] == ["1", "2", "2", "8", "6", "4"] and float(cl[7]) == 200.0 and float(cl[8]) == 7.5
