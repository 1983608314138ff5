"""runstopping_gpu on the GB300: its FP64 output is the reference library's, line
for line (tests/golden/runstopping); the FP32 table path agrees to 5e-3."""
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "runstopping"
CASES = sorted(p.stem for p in GOLD.glob("*.json"))


@pytest.fixture(scope="module")
def frontend(engine_lib):
    from mytrim_gb300 import build
    return build.build_frontend(name="runstopping_gpu")


def run(frontend, text, precision):
    r = subprocess.run([str(frontend), "--precision", precision], input=text, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


@pytest.mark.parametrize("case", CASES)
def test_fp64_output_is_the_reference(frontend, case):
    out = run(frontend, (GOLD / f"{case}.json").read_text(), "fp64")
    assert out == (GOLD / f"{case}.out").read_text()


@pytest.mark.parametrize("case", CASES)
def test_fp32_table_close(frontend, case):
    out = run(frontend, (GOLD / f"{case}.json").read_text(), "fp32")
    gold = [l.split() for l in (GOLD / f"{case}.out").read_text().splitlines()]
    got = [l.split() for l in out.splitlines()]
    assert [g[0] for g in got] == [g[0] for g in gold]
    for g, w in zip(got, gold):
        assert float(g[1]) == pytest.approx(float(w[1]), rel=5e-3)
