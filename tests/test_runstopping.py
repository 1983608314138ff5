"""runstopping front-end (mytrim_gb300/cpp/runstopping_gpu.cpp, mytrim_gb300/runstopping.py).

CPU checks: the committed outputs of the reference library
(tests/golden/runstopping, made by tests/golden/make_runstopping_golden.py) list
exactly the energies the loader builds, the oracle's stopping matches them, and
malformed inputs are rejected with runstopping's messages (apps/runstopping.C:66-173)
by both the loader and the compiled front-end.  The GPU runs are in
test_gpu_runstopping.py.
"""
import copy
import json
import subprocess
from pathlib import Path

import pytest

from mytrim_gb300 import runstopping as S
from mytrim_gb300.runmytrim import InputError

GOLD = Path(__file__).resolve().parent / "golden" / "runstopping"
CASES = sorted(p.stem for p in GOLD.glob("*.json"))


@pytest.fixture(scope="module")
def frontend(engine_lib):
    from mytrim_gb300 import build
    return build.build_frontend(name="runstopping_gpu")


def read_out(path):
    return [tuple(float(v) for v in l.split()) for l in Path(path).read_text().splitlines() if l.strip()]


@pytest.mark.parametrize("case", CASES)
def test_energies_match_reference(case):
    req = S.load((GOLD / f"{case}.json").read_text())
    gold = read_out(GOLD / f"{case}.out")
    assert len(gold) == len(req.energies)
    assert [f"{E:g}" for E in req.energies] == [l.split()[0] for l in (GOLD / f"{case}.out").read_text().splitlines()]


@pytest.mark.parametrize("case", CASES)
def test_oracle_stopping_matches_reference(oracle_built, case):
    req = S.load((GOLD / f"{case}.json").read_text())
    got = oracle_built.stopping(req.Z, req.m, req.material, req.energies)
    for (E, se), g in zip(read_out(GOLD / f"{case}.out"), got):
        assert g == pytest.approx(se, rel=6e-6), E  # the reference prints 6 significant digits


def base():
    return {"stopping": {"ion": {"Z": 1, "mass": 1.008, "energy": 1000.0},
                         "material": {"rho": 2.33, "elements": [{"Z": 14, "mass": 28.086, "fraction": 1}]}}}


def _set(path, value):
    def f(d):
        node = d
        for k in path[:-1]:
            node = node[k]
        if value is None:
            del node[path[-1]]
        else:
            node[path[-1]] = value
        return d
    return f


BAD = [
    (lambda d: {"x": d["stopping"]}, "No 'stopping' top level block found in input"),
    (_set(["stopping", "material"], None), "Must specify a 'material' block in the input file"),
    (_set(["stopping", "material", "rho"], None), "Missing 'rho'"),
    (_set(["stopping", "material", "elements"], 5), "Missing 'elements' in material"),
    (_set(["stopping", "material", "elements", 0, "fraction"], None), "Missing 'fraction' in element 0"),
    (_set(["stopping", "ion"], None), "Must specify an 'ion' block in the input file"),
    (_set(["stopping", "ion", "mass"], None), "Missing 'mass' in ion block"),
    (_set(["stopping", "ion", "energy"], "hot"), "Missing or invalid 'energy' in ion block"),
    (_set(["stopping", "ion", "energy"], {"end": 5}), "Missing 'begin' in energy block"),
    (_set(["stopping", "ion", "energy"], {"begin": 5}), "Missing 'end' in energy block"),
    (_set(["stopping", "ion", "energy"], {"begin": 5, "end": 10}), "Specify either 'step' or 'mult' energy block"),
    (_set(["stopping", "ion", "energy"], {"begin": 5, "end": 10, "step": 1, "mult": 2}),
     "Specify either 'step' or 'mult' energy block"),
    (_set(["stopping", "ion", "energy"], {"begin": 5, "end": 10, "mult": 1.0}), "'mult' must be larger than 1.0"),
]


@pytest.mark.parametrize("k", range(len(BAD)))
def test_input_errors(frontend, k):
    edit, msg = BAD[k]
    text = json.dumps(edit(copy.deepcopy(base())))
    with pytest.raises(InputError) as e:
        S.load(text)
    assert str(e.value) == msg
    r = subprocess.run([str(frontend)], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert r.stderr.splitlines()[-1] == "ERROR: " + msg


def test_energy_forms():
    d = base()
    d["stopping"]["ion"]["energy"] = [10, 20.5]
    assert S.load(json.dumps(d)).energies == [10.0, 20.5]
    d["stopping"]["ion"]["energy"] = {"begin": 1.0, "end": 2.0, "step": 0.1}
    got = S.load(json.dumps(d)).energies
    E, want = 1.0, []
    while E <= 2.0:
        want.append(E)
        E += 0.1
    assert got == want and len(got) == 10  # accumulated rounding drops the end point, as in the reference
