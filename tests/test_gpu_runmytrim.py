"""runmytrim_gpu on the GB300 against the oracle.

With the FP64 path and the oracle's counter-based streams (same master seed),
the front-end's output files are byte-identical to the ones the oracle's
writers produce -- and those writers are pinned byte for byte to the
reference's own plugins (test_runmytrim.py).  The FP32 path is checked
statistically against the FP64 path.
"""
import json
import subprocess
from pathlib import Path

import pytest

from mytrim_gb300 import runmytrim as R

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "runmytrim"
CASES = sorted(p.stem for p in GOLD.glob("*.json"))


@pytest.fixture(scope="module")
def frontend(engine_lib):
    from mytrim_gb300 import build
    return build.build_frontend()


def run_frontend(frontend, text, cwd, precision="fp64"):
    r = subprocess.run([str(frontend), "--precision", precision], input=text, capture_output=True, text=True,
                       cwd=cwd, timeout=600)
    assert r.returncode == 0, r.stderr
    summary = {}
    for line in r.stderr.splitlines():
        if ": " in line and line.split(": ")[0] in ("Vacancies/ion", "Electronic energy loss/ion"):
            k, v = line.split(": ")
            summary[k] = float(v)
    return summary


@pytest.mark.parametrize("case", CASES)
def test_fp64_files_identical_to_oracle(frontend, oracle_built, case, tmp_path):
    text = (GOLD / f"{case}.json").read_text()
    inp = R.load(text)
    (tmp_path / "gpu").mkdir()
    (tmp_path / "ora").mkdir()
    summary = run_frontend(frontend, text, tmp_path / "gpu")
    tallies, _ = oracle_built.write_outputs(inp.sim, inp.output_type, inp.base, seed=inp.seed, philox=True,
                                            cwd=tmp_path / "ora", scale=inp.scale)
    got = (tmp_path / "gpu" / inp.output_file).read_bytes()
    want = (tmp_path / "ora" / inp.output_file).read_bytes()
    assert len(want) > 0
    assert got == want
    n = inp.sim.n_primaries
    # summary lines carry 6 significant digits
    assert summary["Vacancies/ion"] == pytest.approx(tallies["vacancies"] / n, rel=1e-5)
    assert summary["Electronic energy loss/ion"] == pytest.approx(tallies["Eel"] / n, rel=1e-5)


def read_vac(path):
    rows = [l.split() for l in Path(path).read_text().splitlines() if l.strip()]
    return [(int(a), int(b), int(c)) for a, b, c in rows]


@pytest.mark.parametrize("precision", ["fp32", "surrogate"])
def test_fast_paths_agree_statistically(frontend, precision, tmp_path):
    text = (GOLD / "cu_on_cu_vac.json").read_text()
    inp = R.load(text)
    for p in ("fp64", precision):
        (tmp_path / p).mkdir()
        run_frontend(frontend, text, tmp_path / p, precision=p)
    a = read_vac(tmp_path / "fp64" / inp.output_file)
    b = read_vac(tmp_path / precision / inp.output_file)
    # 1-unit depth bins from 0 upwards without gaps in the x column
    assert [r[0] for r in b] == list(range(len(b)))
    va, vb = sum(r[1] for r in a), sum(r[1] for r in b)
    ra, rb = sum(r[2] for r in a), sum(r[2] for r in b)
    assert abs(va - vb) < 0.05 * va
    assert abs(ra - rb) < 0.1 * ra + 10


def test_deep_histogram_grows(frontend, oracle_built, tmp_path):
    """Protons damage far deeper than a thin target's 4096 first bins: the first run
    drops events past its bins and is repeated with more, and the file still
    matches the oracle's."""
    text = json.dumps({"mytrim": {"options": {"seed": 12},
                                  "ion": {"Z": 1, "mass": 1.008, "energy": 100000, "number": 40},
                                  "sample": {"layers": [{"thickness": 10, "rho": 2.33,
                                                         "elements": [{"Z": 14, "mass": 28.086, "fraction": 1}]}]},
                                  "output": {"type": "vaccount", "base": "deep"}}})
    inp = R.load(text)
    (tmp_path / "gpu").mkdir()
    (tmp_path / "ora").mkdir()
    run_frontend(frontend, text, tmp_path / "gpu")
    oracle_built.write_outputs(inp.sim, inp.output_type, inp.base, seed=inp.seed, philox=True, cwd=tmp_path / "ora")
    rows = read_vac(tmp_path / "gpu" / inp.output_file)
    assert len(rows) > 4096
    assert (tmp_path / "gpu" / inp.output_file).read_bytes() == (tmp_path / "ora" / inp.output_file).read_bytes()
