"""runmytrim front-end (mytrim_gb300/cpp/runmytrim_gpu.cpp, mytrim_gb300/runmytrim.py).

CPU checks:
* the oracle's output writers reproduce, byte for byte, the files the
  reference's own plugins (TrimVacCount, TrimVacEnergyCount, TrimRange, compiled
  from the reference sources) wrote for the committed inputs
  (tests/golden/runmytrim, made by tests/golden/make_runmytrim_golden.py);
* the compiled front-end and the Python loader read every input the same way;
* both reject malformed inputs with runmytrim's messages (apps/runmytrim.C:103-285).
The GPU runs of the front-end are in test_gpu_runmytrim.py.
"""
import copy
import json
import subprocess
from pathlib import Path

import pytest

from mytrim_gb300 import runmytrim as R

GOLD = Path(__file__).resolve().parent / "golden" / "runmytrim"
CASES = sorted(p.stem for p in GOLD.glob("*.json"))


@pytest.fixture(scope="module")
def frontend(engine_lib):
    from mytrim_gb300 import build
    return build.build_frontend()


def test_cases_present():
    assert len(CASES) >= 7
    types = {R.load((GOLD / f"{c}.json").read_text()).output_type for c in CASES}
    assert types == set(R.OUTPUT_TYPES)


@pytest.mark.parametrize("case", CASES)
def test_oracle_writer_matches_reference_plugins(oracle_built, case, tmp_path):
    inp = R.load((GOLD / f"{case}.json").read_text())
    oracle_built.write_outputs(inp.sim, inp.output_type, inp.base, seed=inp.seed, philox=False, cwd=tmp_path,
                               scale=inp.scale)
    assert (tmp_path / inp.output_file).read_bytes() == (GOLD / inp.output_file).read_bytes()


def describe(inp: R.RunmytrimInput) -> str:
    """The text runmytrim_gpu --check-input prints for an input."""
    s = inp.sim
    g = lambda v: f"{v:.17g}"  # noqa: E731
    lines = [f"type {inp.output_type}", f"base {inp.base}", f"seed {inp.seed}", f"scale {g(inp.scale)}",
             f"primaries {s.n_primaries}", f"primaries_only {int(s.primaries_only)}",
             f"ion {s.Z} {g(s.m)} {g(s.E)} {g(s.Ef)}", "box " + " ".join(g(v) for v in s.box())]
    for l in s.layers:
        lines.append(f"layer {g(l.thickness)} {g(l.rho)}")
        for e in l.elements:
            lines.append(f"element {e.Z} {g(e.m)} {g(e.t)} {g(e.Edisp)} {g(e.Elbind)}")
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("case", CASES)
def test_frontend_reads_inputs_like_loader(frontend, case):
    text = (GOLD / f"{case}.json").read_text()
    r = subprocess.run([str(frontend), "--check-input"], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout == describe(R.load(text))
    assert "Building" in r.stderr


def test_element_defaults_carry_over():
    """An omitted edisp / elbind keeps the previous element's value across layers."""
    inp = R.load((GOLD / "ar_sio2_si_vac.json").read_text())
    got = [(e.Edisp, e.Elbind) for l in inp.sim.layers for e in l.elements]
    assert got == [(15.0, 2.0)] * 3
    assert inp.scale == 10.0 and inp.sim.Ef == 5.0


def test_json_syntax_of_jsoncpp():
    text = """// comment
    {"mytrim": {/* block */ "options": {"seed": 3, "seed": 4,},
      "ion": {"Z": 1, "mass": 1.008, "energy": 1000, "number": 5,},
      "sample": {"layers": [{"thickness": 100, "rho": 2.33, "elements": [{"Z": 14, "mass": 28.0855,
                 "fraction": 1}],},]},
      "output": {"type": "range", "base": "a\\"b // not a comment"}}}
    trailing text is ignored"""
    inp = R.load(text.replace("trailing text is ignored", ""))
    assert inp.seed == 4 and inp.base == 'a"b // not a comment' and inp.output_type == "range"
    assert inp.sim.mode == "range"


def base_doc():
    return {"mytrim": {"options": {"seed": 1},
                       "ion": {"Z": 29, "mass": 63.546, "energy": 1000, "number": 10},
                       "sample": {"layers": [{"thickness": 1000, "rho": 8.96,
                                              "elements": [{"Z": 29, "mass": 63.546, "fraction": 1}]}]},
                       "output": {"type": "vaccount", "base": "x"}}}


def _edit(path, value):
    def f(d):
        node = d
        for k in path[:-1]:
            node = node[k]
        if value is _DEL:
            del node[path[-1]]
        else:
            node[path[-1]] = value
        return d
    return f


_DEL = object()
BAD = [
    (lambda d: {"other": d["mytrim"]}, "No 'mytrim' top level block found in input"),
    (_edit(["mytrim", "sample"], _DEL), "Must specify a 'sample' block in the input file"),
    (_edit(["mytrim", "sample", "layers"], {}), "sample.layers must be an array"),
    (_edit(["mytrim", "sample", "layers", 0, "thickness"], _DEL), "No 'thickness' found for layer 0"),
    (_edit(["mytrim", "output"], _DEL), "Must specify an 'output' block in the input file"),
    (_edit(["mytrim", "output", "type"], 3), "output.type must be a string"),
    (_edit(["mytrim", "output", "type"], "phonons"), "Unknown output type phonons"),
    (_edit(["mytrim", "sample", "layers", 0, "rho"], "dense"), "Missing 'rho' in layer 0"),
    (_edit(["mytrim", "sample", "layers", 0, "elements"], _DEL), "Missing 'elements' in layer 0"),
    (_edit(["mytrim", "sample", "layers", 0, "elements", 0, "mass"], _DEL), "Missing 'mass' in element 0 in layer 0"),
    (_edit(["mytrim", "sample", "layers", 0, "elements", 0, "Z"], True), "Missing 'Z' in element 0 in layer 0"),
    (_edit(["mytrim", "ion"], _DEL), "Must specify an 'ion' block in the input file"),
    (_edit(["mytrim", "ion", "energy"], _DEL), "Missing 'energy' in ion block"),
    (_edit(["mytrim", "ion", "number"], "many"), "Missing 'number' in ion block"),
]


@pytest.mark.parametrize("k", range(len(BAD)))
def test_input_errors(frontend, k):
    edit, msg = BAD[k]
    text = json.dumps(edit(copy.deepcopy(base_doc())))
    with pytest.raises(R.InputError) as e:
        R.load(text)
    assert str(e.value) == msg
    r = subprocess.run([str(frontend), "--check-input"], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert r.stderr.splitlines()[-1] == "ERROR: " + msg


def test_frontend_rejects_arguments_and_bad_json(frontend):
    r = subprocess.run([str(frontend), "input.json"], input="", capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "stdin" in r.stderr
    r = subprocess.run([str(frontend), "--check-input"], input='{"mytrim": {', capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and r.stderr.startswith("ERROR: cannot parse")


def test_reference_length_scale_profiles():
    """The reference's length-scale test (tests/json/README.md: the xe_on_uo2 vacancy
    profile against the xe_on_uo2_scale10 one with depth x 10): in the reference's own
    output files the 1 A bins of the scale-1 run, summed ten at a time, give the 10 A
    bins of the scale-10 run exactly, except bin 0, which TrimVacCount's truncating
    int() also fills from the first sample unit in front of the surface (-1 A at scale
    1, -10 A at scale 10)."""
    import numpy as np
    a = np.loadtxt(GOLD / "json_xe_on_uo2_vac.dat")
    b = np.loadtxt(GOLD / "json_xe_on_uo2_scale10_vac.dat")
    rebinned = np.zeros((len(b), 2))
    np.add.at(rebinned, a[:, 0].astype(int) // 10, a[:, 1:])
    assert np.array_equal(rebinned[1:], b[1:, 1:])
    assert (b[0, 1:] >= rebinned[0]).all()
    assert (GOLD / "json_xe_on_uo2.summary").read_text() == (GOLD / "json_xe_on_uo2_scale10.summary").read_text()
