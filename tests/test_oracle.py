"""The CPU oracle is pinned to the reference before anything is compared with it.

* mtoracle (the C++ restatement) reproduces the reference library bit for bit on
  the committed fixtures (tests/golden/ref_records.json, made by the reference
  itself through oracle/_ref/ref_driver) and, where the reference sources are
  present, on fresh runs of the reference;
* it reproduces the reference's published vacancies/ion table within Monte Carlo
  error (validation/vacancy_count/vacancy_count_comparison.dat);
* its electronic stopping follows the SRIM tables the reference validates
  against (validation/*/srim_stopping.dat);
* the reference's own golden regression (tests/uo2) passes with the reference
  build used here.
"""
import json
import math
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLD = ROOT / "tests" / "golden"
sys.path.insert(0, str(GOLD))

from golden_cases import CASES  # noqa: E402
from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec  # noqa: E402

SCALARS = ("primaries", "members", "collisions", "vacancies", "replacements", "interstitials",
           "substitutionals", "lost", "Eel", "Enuc", "Elost", "Eunfollowed", "range_n", "sx", "sxx",
           "sy", "syy", "sz", "szz", "vac_s2", "eel_s2", "enuc_s2", "coll_s2", "sputtered", "backscattered",
           "Esputtered", "Evoxel")


@pytest.mark.parametrize("case", sorted(CASES))
def test_restatement_matches_reference_fixture(oracle_built, case):
    gold = json.loads((GOLD / "ref_records.json").read_text())[case]
    sim, seed, nrec = CASES[case]
    got = oracle_built.run(sim, seed=seed, philox=False, records=nrec)
    for k in SCALARS:
        assert got[k] == gold[k], (case, k, got[k], gold[k])
    for h in ("hist_range", "hist_vac", "hist_repl", "vox_depth"):
        assert got[h] == gold[h], (case, h)
    assert got["records"] == gold["records"]


def _ref_available(oracle_built):
    return oracle_built.REF_DRIVER.exists()


@pytest.mark.parametrize("seed", [1, 99])
def test_restatement_matches_reference_live(oracle_built, seed):
    if not _ref_available(oracle_built):
        pytest.skip("reference sources not present: fixtures cover the pin")
    sims = [
        SimSpec(layers=[LayerSpec(1000.0, 2.2, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0),
                                                ElementSpec(8, 15.999, 2.0, 28.0, 3.0)]),
                        LayerSpec(1e5, 10.49, [ElementSpec(47, 107.868, 1.0)])],
                Z=79, m=196.967, E=30e3, n_primaries=6, bc=(2, 0, 2), size=(1e6, 200.0, 200.0),
                hist_range_bin=7.0, hist_range_n=80, hist_vac_bin=3.0, hist_vac_n=80),
        SimSpec(layers=[LayerSpec(1e5, 2.33, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0)])], Z=3, m=7.016,
                E=40e3, n_primaries=20, mode="range", primaries_only=True),
        SimSpec(layers=[LayerSpec(1e5, 8.96, [ElementSpec(29, 63.546, 1.0, 25.0, 3.0)])], Z=29, m=63.546,
                E=3e3, n_primaries=10, potential="moliere", hist_range_bin=5.0, hist_range_n=50),
        SimSpec(layers=[LayerSpec(1e5, 2.26, [ElementSpec(6, 12.011, 1.0, 28.0, 3.0)])], Z=36, m=83.798,
                E=5e3, n_primaries=10, potential="ckr"),
        SimSpec(layers=[LayerSpec(1e5, 3.21, [ElementSpec(14, 28.086, 1.0, 35.0, 3.0),
                                              ElementSpec(6, 12.011, 1.0, 20.0, 3.0)])],
                Z=54, m=131.29, E=10e3, n_primaries=10, mode="primaries", max_generation=seed % 2 + 1),
        SimSpec(layers=[LayerSpec(300.0, 10.0, [ElementSpec(92, 235.0, 1.0), ElementSpec(8, 16.0, 2.0)]),
                        LayerSpec(300.0, 3.5, [ElementSpec(54, 132.0, 1.0)])],
                Z=54, m=132.0, E=10e3, n_primaries=6, pos=(0.0, 150.0, 150.0), size=(300.0, 300.0, 300.0),
                geometry="clusters", clusters=np.array([[60.0, 150.0, 150.0, 25.0], [200.0, 100.0, 120.0, 15.0]]),
                cluster_hash=(10, 10, 10)),
    ]
    for sim in sims:
        a = oracle_built.run(sim, seed=seed, philox=False, records=sim.n_primaries)
        b = oracle_built.run(sim, seed=seed, philox=False, records=sim.n_primaries, reference=True)
        a.pop("wall_s"), b.pop("wall_s")
        a.pop("seed_sq")  # the restatement's count of repeated seeds; the driver has none
        assert a == b


def _vacancy_row(energy_kev):
    t = json.loads((GOLD / "vacancy_table.json").read_text())
    for row in t["rows"]:
        if row[0] == energy_kev:
            return row[1:]
    raise KeyError(energy_kev)


# (pair, column offset in the table, Z1, m1, rho, Z2, m2)
PAIRS = {"Si - C": (0, 14, 27.977, 2.253, 6, 12.01), "Xe - U": (4, 54, 131.904, 19.043, 92, 238.0),
         "Cu - Cu": (8, 29, 63.546, 8.92, 29, 63.546)}


@pytest.mark.parametrize("pair,energy_kev,mode,n", [
    ("Cu - Cu", 1, "exact", 1000), ("Cu - Cu", 10, "exact", 1000), ("Cu - Cu", 1, "kp", 10000),
    ("Cu - Cu", 10, "kp", 10000), ("Si - C", 1, "exact", 1000), ("Xe - U", 1, "exact", 1000),
    ("Si - C", 10, "kp", 10000),
])
def test_published_vacancy_table(oracle_built, pair, energy_kev, mode, n):
    """The reference's published MyTRIM vacancies/ion (validation/vacancy_count) are
    reproduced by the oracle with the reference's own inputs (seed 2344)."""
    off, Z1, m1, rho, Z2, m2 = PAIRS[pair]
    published = _vacancy_row(energy_kev)[off + (1 if mode == "exact" else 0)]
    sim = SimSpec(layers=[LayerSpec(100000.0, rho, [ElementSpec(Z2, m2, 1.0)])], Z=Z1, m=m1,
                  E=energy_kev * 1000.0, n_primaries=n, mode="vaccount" if mode == "exact" else "range")
    r = oracle_built.run_parallel(sim, seed=2344, philox=False, procs=4)
    mean = r["vacancies"] / n
    err = math.sqrt(max(r["vac_s2"] / n - mean * mean, 0.0) / (n - 1))
    # the published numbers come from an older build of the same code: allow 3 sigma
    # plus 2 % for the difference in version
    assert abs(mean - published) <= 3 * err + 0.02 * published, (mean, err, published)


def test_srim_stopping_tables(oracle_built):
    """Electronic stopping of H, He in Fe and C in W follows SRIM's tables
    (validation/*/srim_stopping.dat) as closely as the reference's fit does."""
    srim = json.loads((GOLD / "srim_stopping.json").read_text())
    for case, d in srim.items():
        layer = LayerSpec(1.0, d["rho"], [ElementSpec(z, m, t) for z, m, t in d["elements"]])
        got = oracle_built.stopping(d["Z1"], d["m1"], layer, d["E_eV"])
        rel = [abs(g - s) / s for g, s in zip(got, d["dEdx_eV_per_A"])]
        # the SRIM-95 fit of the reference against a later SRIM: the light ions agree
        # within 3 % above 100 keV; everywhere within 25 %, on average within 10 %
        # (the reference asserts no tolerance; these bounds pin its present agreement)
        assert max(rel) < 0.25, (case, max(rel))
        assert sum(rel) / len(rel) < 0.10, (case, sum(rel) / len(rel))
        if d["Z1"] <= 2:
            hi = [r for r, e in zip(rel, d["E_eV"]) if e >= 1e5]
            assert max(hi) < 0.03, (case, max(hi))


def test_reference_uo2_golden(oracle_built, tmp_path):
    """The reference's own regression test (tests/uo2/test.sh) passes with the
    reference library as built by oracle/Makefile."""
    from conftest import REFERENCE
    exe = ROOT / "oracle" / "_ref" / "mytrim_uo2"
    gold = REFERENCE / "tests" / "uo2" / "gold" if REFERENCE else None
    if not exe.exists() or gold is None or not gold.exists():
        pytest.skip("reference sources not present")
    env = dict(os.environ, MYTRIM_SEED="39172")
    subprocess.run([str(exe), "out", "10", "0.1", "1"], cwd=tmp_path, env=env, check=True,
                   capture_output=True)
    for name in ("out.Erec", "out.clcoor", "out.dist"):
        got = [l.split() for l in (tmp_path / name).read_text().splitlines() if l.strip()]
        ref = [l.split() for l in (gold / name).read_text().splitlines() if l.strip()]
        assert len(got) == len(ref)
        for a, b in zip(got, ref):
            for x, y in zip(a, b):
                assert abs(float(x) - float(y)) <= 1e-4


def test_length_scale_invariance(oracle_built):
    """The reference's length-scale check (tests/json: the xe_on_uo2 input at length
    scale 1 and 10 gives the same vacancy profile), made exact for the restatement: a
    sample in units of 10 A, ten times thinner with ten times finer bins, follows the
    same cascades (flight lengths are drawn in A and divided by the scale, trim.C:45-46),
    so the integer tallies agree and the depth profiles agree up to bin-edge rounding."""
    uo2 = [ElementSpec(92, 238.03, 1.0, 40.0, 3.0), ElementSpec(8, 15.999, 2.0, 20.0, 3.0)]
    runs = []
    for scale in (1.0, 10.0):
        sim = SimSpec(layers=[LayerSpec(1e6 / scale, 10.97, uo2)], Z=54, m=131.29, E=30e3, n_primaries=100,
                      hist_vac_bin=10.0 / scale, hist_vac_n=300, hist_range_bin=10.0 / scale, hist_range_n=300)
        runs.append(oracle_built.run(sim, seed=8, scale=scale))
    a, b = runs
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials", "range_n"):
        assert a[k] == b[k], k
    assert math.isclose(a["sx"], 10.0 * b["sx"], rel_tol=1e-9)
    assert np.abs(np.subtract(a["hist_vac"], b["hist_vac"])).sum() <= 0.002 * a["vacancies"]
    assert np.abs(np.subtract(a["hist_range"], b["hist_range"])).sum() <= 2
