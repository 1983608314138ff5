"""Regenerate the runstopping fixtures of tests/golden/runstopping from the reference.

Each case is a runstopping input (JSON, written here) and what runstopping prints
for it ("E S_e" per line), computed by the reference library itself
(oracle/_ref/ref_runstopping, built from the reference sources by
oracle/Makefile "make ref").  The ions and targets are the reference's stopping
validation cases (H and He in Fe, C in W) plus a compound target.

Needs the reference checkout ($MYTRIM_REFERENCE, else oracle/Makefile's REF).

Usage: python tests/golden/make_runstopping_golden.py
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "runstopping"
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle_io  # noqa: E402
from mytrim_gb300 import runstopping  # noqa: E402

REF = oracle_io.reference_dir()
if REF is None:
    sys.exit("the reference checkout is needed: set MYTRIM_REFERENCE")

FE = {"rho": 7.8658, "elements": [{"Z": 26, "mass": 55.847, "fraction": 1}]}
CASES = {
    "h_on_fe": {"ion": {"Z": 1, "mass": 1.008, "energy": {"begin": 10000, "end": 10000000, "mult": 1.1}}, "material": FE},
    "he_on_fe": {"ion": {"Z": 2, "mass": 4.003, "energy": {"begin": 10000, "end": 10000000, "mult": 1.1}}, "material": FE},
    "c_on_w": {"ion": {"Z": 6, "mass": 12, "energy": {"begin": 10000, "end": 10000000, "step": 100000}},
               "material": {"rho": 19.35, "elements": [{"Z": 74, "mass": 183.85, "fraction": 1}]}},
    "ag_on_sio2": {"ion": {"Z": 47, "mass": 106.905, "energy": [10, 100, 1000, 3000, 10000, 30000, 100000, 300000,
                                                              1000000, 3000000, 10000000]},
                   "material": {"rho": 2.2, "elements": [{"Z": 14, "mass": 28.086, "fraction": 1},
                                                         {"Z": 8, "mass": 15.999, "fraction": 2}]}},
}


def main():
    oracle_io.build(REF)
    OUT.mkdir(exist_ok=True)
    for name, block in CASES.items():
        text = "// runstopping input\n" + json.dumps({"stopping": block}, indent=2) + "\n"
        (OUT / f"{name}.json").write_text(text)
        req = runstopping.load(text)
        out = oracle_io.runstopping_reference(req.Z, req.m, req.material, req.energies)
        (OUT / f"{name}.out").write_text(out)
        print(name, len(req.energies), "energies")


if __name__ == "__main__":
    main()
