"""Event streams in the reference's text formats (mytrim_gb300/streams.py).

The number format is std::ostream's default (six significant digits, as
IonBase's operator<< prints, ion.C:74-79); a C++ program checks that Python's %g
writes the same text for the same doubles."""
import subprocess

import numpy as np

from mytrim_gb300 import _ffi as F
from mytrim_gb300 import streams

DT = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("E", "<f8"), ("aux", "<f8"), ("m", "<f8"), ("key", "<u8"),
               ("primary", "<i8"), ("sim", "<i4"), ("kind", "<i4"), ("Z", "<i4"), ("gen", "<i4"), ("state", "<i4"),
               ("tag", "<i4")])
VALUES = [0.0, 1.0, 123.456789, 1e-7, 2.5e12, -3.25, 63.546, 99999.95, 1234567.0, 0.000123456789]


def events():
    e = np.zeros(4, dtype=DT)
    e[0] = (10.5, 50.0, 49.75, 24.0, 3.0, 63.546, 7, 0, 0, F.EV_VACANCY, 29, 1, 0, 4)  # born in cluster 4
    e[1] = (11.0, 50.1, 49.8, 2.5, 3.0, 63.546, 7, 0, 0, F.EV_DISSIPATE, 29, 1, 0, -1)
    e[2] = (12.0, 50.2, 49.9, 1.25, 0.0, 63.546, 9, 0, 0, F.EV_REST, 29, 2, 3, -1)
    e[3] = (13.0, 50.3, 50.0, 40.0, 3.0, 63.546, 9, 0, 0, F.EV_BRANCH, 29, 3, 0, -1)
    return e


def test_defect_and_phonon_lines():
    d = list(streams.defect_log(events()))
    assert d == ["V 10.5 50 49.75 29 63.546 24 7 1 4 ", "I 12 50.2 49.9 29 63.546 1.25 9 2 -1 "]
    p = list(streams.phonon_log(events()))
    # sorted by primary, path key, then event kind (branch before rest)
    assert p == ["5.5 11 50.1 49.8 29 63.546 2.5 7 1 -1 ", "3 13 50.3 50 29 63.546 40 9 3 -1 ",
                 "1.25 12 50.2 49.9 29 63.546 1.25 9 2 -1 "]


def test_number_format_is_ostreams(tmp_path):
    src = tmp_path / "fmt.cpp"
    src.write_text("#include <iostream>\nint main(){double v;while(std::cin>>v)std::cout<<v<<'\\n';}\n")
    exe = tmp_path / "fmt"
    subprocess.run(["g++", "-O1", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], input="\n".join(repr(v) for v in VALUES), capture_output=True, text=True,
                         check=True).stdout.split()
    assert out == ["%g" % v for v in VALUES]


def test_vac_map_follows_trimvacmap():
    e = np.zeros(6, dtype=DT)
    # (x, y) over w = (100, 100) on a 20 x 20 map: cells int(x / 5), int(y / 5)
    e[0] = (12.0, 3.0, 0.0, 10.0, 3.0, 69.7, 1, 0, 0, F.EV_VACANCY, 31, 1, 0, -1)
    e[1] = (12.5, 4.9, 0.0, 10.0, 3.0, 69.7, 1, 0, 0, F.EV_VACANCY, 31, 1, 0, -1)
    e[2] = (103.0, 3.0, 0.0, 10.0, 3.0, 74.9, 1, 0, 0, F.EV_VACANCY, 33, 1, 0, -1)   # x wraps: cell 0
    e[3] = (-8.0, 3.0, 0.0, 10.0, 3.0, 74.9, 1, 0, 0, F.EV_VACANCY, 33, 1, 0, -1)    # int(-1.6) = -1: dropped
    e[4] = (12.0, 3.0, 0.0, 10.0, 3.0, 69.7, 1, 0, 0, F.EV_REST, 31, 1, 3, -1)       # not a vacancy
    e[5] = (-3.0, 3.0, 0.0, 10.0, 3.0, 74.9, 1, 0, 0, F.EV_VACANCY, 33, 1, 0, -1)    # int(-0.6) = 0: cell 0
    m = streams.vac_map(e, (100.0, 100.0), (31, 33))
    assert m.shape == (20, 20, 3)
    assert m[2, 0, 0] == 2 and m[0, 0, 1] == 2 and m.sum() == 4
