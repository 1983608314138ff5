"""Size-independent properties of the GPU engine at the full sizes of the five
measurement configurations (GB300; called through the C ABI):

* C1, Cu 100 keV into Cu, 10^4 primaries, FP64: energy conservation to 1e-12, the
  range histogram holds every primary that came to rest; FP32 (10^6) within 1 % of
  FP64 (10^5);
* C2, B 10 keV and As 50 keV at 7 deg into SiO2 / Si, 10^6 primaries each, FP32:
  energy conservation, the lateral histogram and the range histogram account for
  every stopped primary inside their extent, two primary shards reproduce the whole
  run's integer tallies exactly, and FP32 is within 1 % of FP64 (10^6 B, 10^5 As);
* C3, 4096 independent simulations (about 5.9e7 primaries), FP32: every
  simulation conserves energy and ran all its primaries;
* C4, Ag 200 keV into Si, 10^7 primaries, FP32: energy conservation; the FP32
  path's and the surrogate path's (2^21 primaries) range, straggle, lateral spread,
  vacancies and energy split each within 1 % of the FP64 path's (2^18 primaries);
* C5, Au 1 MeV into Ag / Cu / Si, 2^20 of the 10^8 primaries (about 7 s), FP32 with
  256^3 voxels accumulated in FP64: the FP32 tally is the FP64 totals rounded once,
  the voxel total equals the energy deposited inside the box, which is at most the
  total deposit; four primary shards add up to the whole run cell by cell;
  sputtered atoms and backscattered ions counted.

"Within 1 %" means: the relative difference is under 1 % and the combined standard
error under 1/3 %, so that a 1 % error would show at 3 sigma (parity_stats.py).
"""
import math

import numpy as np
import pytest

from mytrim_gb300 import Engine
from mytrim_gb300 import workloads as W
from mytrim_gb300.engine import SimSpec

import parity_stats as PS

pytestmark = pytest.mark.gpu

INT_KEYS = ("members", "collisions", "vacancies", "replacements", "interstitials", "substitutionals", "lost",
            "range_n")


def _conserved(t, E0, n, rel):
    total = t["Eel"] + t["Enuc"] + t["Elost"] + t["Eunfollowed"]
    assert abs(total - E0 * n) <= rel * E0 * n, (total, E0 * n)


def _run(prec, sims, seed=1):
    e = Engine(precision=prec, seed=seed)
    try:
        return e.run(sims)
    finally:
        e.close()


def test_c1_cu_self_ion_fp64():
    sim = W.cu_self_ion(n_primaries=10_000)
    t = _run("fp64", [sim])[0]
    assert t["primaries"] == 10_000
    _conserved(t, sim.E, 10_000, 1e-12)
    beyond = t["range_n"] - int(np.sum(t["hist_range"]))
    assert 0 <= beyond <= t["range_n"]  # stops past 200 nm fall outside the histogram
    f = _run("fp32", [sim])[0]
    _conserved(f, sim.E, 10_000, 2e-6)
    # FP32 against FP64 on the same physics, on samples that resolve 1 %: 10^6 and 10^5
    _, pf = PS.run_primaries("fp32", SimSpec(**{**sim.__dict__, "n_primaries": 1_000_000}), seed=3)
    _, pd = PS.run_primaries("fp64", SimSpec(**{**sim.__dict__, "n_primaries": 100_000}), seed=4)
    PS.assert_within_one_percent(pf, pd, "fp32 cu100k_cu")


@pytest.mark.parametrize("ion", ["boron", "arsenic"])
def test_c2_layered_implants(ion):
    n = 1_000_000
    sim = W.boron_implant(n) if ion == "boron" else W.arsenic_implant(n)
    t, pt = PS.run_primaries("fp32", sim, seed=1)
    assert t["primaries"] == n
    _conserved(t, sim.E, n, 2e-6)
    # every primary that came to rest inside the lateral window is in the lateral
    # histogram, every one that stopped within 300 nm in the range histogram
    assert 0 < int(np.sum(t["hist_lateral"])) <= t["range_n"]
    assert 0 < int(np.sum(t["hist_range"])) <= t["range_n"]
    assert t["range_n"] + t["backscattered"] == n  # CUT surface: the rest left through x < 0
    # two primary shards reproduce the whole run
    parts = [_run("fp32", [SimSpec(**{**sim.__dict__, "n_primaries": k, "first_primary": f})])[0]
             for f, k in ((0, n // 2), (n // 2, n - n // 2))]
    for k in INT_KEYS:
        assert t[k] == parts[0][k] + parts[1][k], k
    assert np.array_equal(t["hist_range"], parts[0]["hist_range"] + parts[1]["hist_range"])
    assert np.array_equal(t["hist_lateral"], parts[0]["hist_lateral"] + parts[1]["hist_lateral"])
    # FP32 against FP64 (the FP64 run at full size for boron, a tenth for arsenic)
    n64 = n if ion == "boron" else n // 10
    d, pd = PS.run_primaries("fp64", SimSpec(**{**sim.__dict__, "n_primaries": n64}), seed=2)
    _conserved(d, sim.E, n64, 1e-12)
    PS.assert_within_one_percent(pt, pd, f"fp32 {ion}")


def test_c3_batched_simulations():
    sims = W.batched_uneven(n_sims=4096, seed=1)
    out = _run("fp32", sims)
    assert len(out) == 4096
    total = sum(s.n_primaries for s in sims)
    assert total > 3e7
    assert sum(t["primaries"] for t in out) == total
    for s, t in zip(sims, out):
        assert t["primaries"] == s.n_primaries
        _conserved(t, s.E, s.n_primaries, 1e-5)


def test_c4_silver_into_silicon_against_fp64():
    """C4 at full size: the FP32 path's 10^7 primaries and the surrogate path's 2^21,
    each against 2^18 primaries of the FP64 plain path: mean range, straggle, lateral
    spread, vacancies, electronic and nuclear loss per ion within 1 %, on samples that
    show a 1 % error at 3 sigma."""
    sim = W.silver_into_silicon(n_primaries=10_000_000)
    f, pf = PS.run_primaries("fp32", sim, seed=1)
    assert f["primaries"] == 10_000_000
    _conserved(f, sim.E, 10_000_000, 2e-6)
    d, p64 = PS.run_primaries("fp64", SimSpec(**{**sim.__dict__, "n_primaries": 1 << 18}), seed=2)
    _conserved(d, sim.E, 1 << 18, 1e-12)
    PS.assert_within_one_percent(pf, p64, "fp32 ag200k_si")
    from mytrim_gb300.train_surrogate import PARAMS
    g, pg = PS.run_primaries("surrogate", SimSpec(**{**sim.__dict__, "n_primaries": 1 << 21}), seed=3,
                             params=np.load(PARAMS))
    _conserved(g, sim.E, 1 << 21, 2e-6)
    PS.assert_within_one_percent(pg, p64, "surrogate ag200k_si")


def test_c5_gold_deposition_voxels():
    n = 1 << 20
    sim = W.gold_deposition(n_primaries=n, voxels=256)
    e = Engine(precision="fp32", seed=1)
    t = e.run([sim])[0]
    vox = e.voxels(0)
    vox64 = e.voxels(0, fp64=True)
    e.close()
    assert vox.shape == (256, 256, 256)
    _conserved(t, sim.E, n, 2e-6)
    # the FP32 tally is each cell's FP64 total rounded once
    assert np.array_equal(vox, vox64.astype(np.float32))
    inside = float(vox64.sum())
    assert math.isclose(inside, t["Evoxel"], rel_tol=1e-9)
    assert 0.5 * (t["Eel"] + t["Enuc"]) < t["Evoxel"] <= (t["Eel"] + t["Enuc"]) * (1 + 1e-6)
    assert t["sputtered"] > 0 and t["backscattered"] > 0
    assert t["Esputtered"] > 0.0
    # FP64 cell totals: four primary shards add up to the whole run cell by cell, to
    # the rounding of the lanes' short FP32 runs of deposits (a few 1e-8 of each,
    # grouped differently when the primaries are split); an FP32 cell total would
    # add the rounding of every one of its ~1e5 runs (1e-5 .. 1e-3 here)
    parts = np.zeros_like(vox64)
    for k in range(4):
        e = Engine(precision="fp32", seed=1)
        e.run([SimSpec(**{**sim.__dict__, "n_primaries": n // 4, "first_primary": k * (n // 4)})])
        parts += e.voxels(0, fp64=True)
        e.close()
    big = vox64 > 1e-6 * vox64.max()
    assert np.allclose(parts[big], vox64[big], rtol=1e-6, atol=0.0)
    assert float(vox64.max()) > 1e6  # the entrance cells collect millions of deposits' worth
