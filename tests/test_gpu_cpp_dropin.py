"""The C++ drop-in on the GPU: TrimGPU (mytrim_gb300/cpp/trim_gpu.h), the TrimBase
subclass a reference user constructs with (SimconfType *, SampleBase *) (trim.h:39-42),
runs whole batches through runPrimaries and runBatch.

tests/cpp/trim_gpu_run.cpp builds the reference's objects in code -- a SampleLayers
of SiO2 on Si with a CUT entrance, a SampleSolid of Cu, IonBase templates with a
tilted direction and a final energy -- and runs them through TrimGPU, with
_potential switched to Moliere for the batch.  It compiles against tests/cpp/mirror,
which declares the reference's class and field names (the reference's headers are
not on the GPU machine; tests/test_cpp_dropin.py compiles trim_gpu.h against them on
the CPU).  Every total equals, bit for bit, the same simulations run
through the Python front end, and the SimconfType tallies (vacancies_created,
EelTotal, EnucTotal) receive the sums, as the reference's hooks add to them.
"""
import math
import subprocess
from pathlib import Path

import pytest

from mytrim_gb300 import Engine
from mytrim_gb300 import _ffi as F
from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
FIELDS = ("primaries", "members", "collisions", "vacancies", "replacements", "interstitials", "substitutionals",
          "lost")


@pytest.fixture(scope="module")
def runner(engine_lib, tmp_path_factory):
    lib = Path(engine_lib).parent
    exe = tmp_path_factory.mktemp("dropin") / "trim_gpu_run"
    inc = ["-I" + str(ROOT / "tests" / "cpp" / "mirror")]
    subprocess.run(["g++", "-O2", "-std=c++17", *inc, "-I" + str(ROOT / "include"),
                    "-I" + str(ROOT / "mytrim_gb300" / "cpp"), str(ROOT / "tests" / "cpp" / "trim_gpu_run.cpp"),
                    "-L" + str(lib), "-lmytrim_gpu", "-Wl,-rpath," + str(lib), "-o", str(exe)], check=True)
    tables = ROOT / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    out = subprocess.run([str(exe), str(tables)], capture_output=True, text=True, check=True).stdout
    res = {}
    for line in out.splitlines():
        p = line.split()
        if p[0] == "tot":
            res[p[1]] = dict(zip(FIELDS, map(int, p[2:10])), Eel=float.fromhex(p[10]), Enuc=float.fromhex(p[11]))
        elif p[0] == "simconf":
            res["simconf"] = (int(p[1]), float.fromhex(p[2]), float.fromhex(p[3]))
    return res


def _layers(n, potential="universal"):
    t = 7.0 * math.pi / 180.0  # the expression the C++ program evaluates
    return SimSpec(layers=[LayerSpec(100.0, 2.2, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0),
                                                  ElementSpec(8, 15.999, 2.0, 28.0, 3.0)]),
                           LayerSpec(1e7, 2.33, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0)])],
                   Z=5, m=11.009, E=10e3, Ef=3.0, n_primaries=n, dir=(math.cos(t), math.sin(t), 0.0),
                   pos=(0.0, 0.0, 0.0), size=(1e9, 1e9, 1e9), bc=(F.BC_CUT, F.BC_INF, F.BC_INF),
                   potential=potential)


def _solid(n, potential="universal"):
    return SimSpec(layers=[LayerSpec(1e7, 8.96, [ElementSpec(29, 63.546, 1.0, 25.0, 3.0)])], Z=29, m=63.546, E=5e3,
                   Ef=5.0, n_primaries=n, dir=(1.0, 0.0, 0.0), pos=(0.0, 50.0, 50.0), size=(1e7, 100.0, 100.0),
                   potential=potential)


def _same(got, want):
    for k in FIELDS:
        assert got[k] == want[k], (k, got[k], want[k])
    # the per-primary energy sums take each lane's share through FP64 atomics in the
    # order the lanes reach them, so two runs agree to rounding, not to the bit
    for k in ("Eel", "Enuc"):
        assert math.isclose(got[k], want[k], rel_tol=1e-12), (k, got[k], want[k])


def test_run_primaries_equals_engine(runner):
    e = Engine(precision="fp64", seed=17)
    want = e.run([_layers(3000)])[0]
    e.close()
    assert want["vacancies"] > 0 and want["lost"] > 0
    _same(runner["boron_primaries"], want)


def test_run_batch_honours_potential_and_equals_engine(runner):
    e = Engine(precision="fp64", seed=18)
    want = e.run([_layers(3000, "moliere"), _solid(500, "moliere")])
    e.close()
    _same(runner["batch_boron_moliere"], want[0])
    _same(runner["batch_copper_moliere"], want[1])
    # the potential changed the run: the universal-potential boron run differs
    assert runner["batch_boron_moliere"]["collisions"] != runner["boron_primaries"]["collisions"]


def test_simconf_tallies_receive_the_sums(runner):
    runs = [runner[k] for k in ("boron_primaries", "batch_boron_moliere", "batch_copper_moliere")]
    vac, eel, enuc = runner["simconf"]
    assert vac == sum(r["vacancies"] for r in runs)
    assert eel == runs[0]["Eel"] + runs[1]["Eel"] + runs[2]["Eel"]
    assert enuc == runs[0]["Enuc"] + runs[1]["Enuc"] + runs[2]["Enuc"]
