"""GPU parity of the cascade engine, through the C ABI (libmytrim_gpu.so).

* stopping: the FP64 device stopping equals the oracle's getrstop to 1e-12;
  the FP32 table to 2e-4;
* trajectories: the FP64 engine's per-member records equal, bit for bit, the host
  build of the same code (oracle/_build/replay_host) on the same Philox streams;
* statistics: FP64 discrete totals equal the oracle on the same Philox streams;
  FP32 agrees with FP64 within 1 %, on samples large enough to show a 1 % error
  at 3 sigma (2e5 primaries; universal, Moliere and C-Kr potentials, clusters);
* properties at full size: energy conservation, sharding invariance, overflow
  drains, error returns instead of hangs.
"""
import ctypes as C
import math
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "tests" / "golden"))

from golden_cases import CASES  # noqa: E402
from mytrim_gb300 import Engine, summarize  # noqa: E402
from mytrim_gb300 import _ffi as F  # noqa: E402
from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec  # noqa: E402
from mytrim_gb300 import workloads as W  # noqa: E402
import parity_stats as PS  # noqa: E402
import fp32_scatter_model  # noqa: E402

pytestmark = pytest.mark.gpu

TARGETS = {
    "Si": LayerSpec(1.0, 2.33, [ElementSpec(14, 28.086, 1.0)]),
    "Fe": LayerSpec(1.0, 7.8658, [ElementSpec(26, 55.847, 1.0)]),
    "W": LayerSpec(1.0, 19.35, [ElementSpec(74, 183.85, 1.0)]),
    "SiO2": LayerSpec(1.0, 2.2, [ElementSpec(14, 28.086, 1.0), ElementSpec(8, 15.999, 2.0)]),
    "C": LayerSpec(1.0, 2.253, [ElementSpec(6, 12.01, 1.0)]),
}
IONS = [(1, 1.008), (2, 4.003), (5, 11.009), (14, 27.977), (29, 63.546), (47, 106.905), (79, 196.967), (92, 238.05)]


@pytest.mark.parametrize("target", sorted(TARGETS))
def test_stopping_fp64_matches_oracle(gpu_engine, oracle_built, target):
    E = np.logspace(0, 7.2, 97)
    layer = TARGETS[target]
    for Z1, m1 in IONS:
        want = np.array(oracle_built.stopping(Z1, m1, layer, E))
        got = gpu_engine.stopping(Z1, m1, layer, E, precision="fp64")
        rel = np.abs(got - want) / np.abs(want)
        assert rel.max() < 1e-12, (target, Z1, rel.max())


@pytest.mark.parametrize("target", ["Si", "SiO2", "W"])
def test_stopping_fp32_table(gpu_engine, oracle_built, target):
    E = np.logspace(0.5, 6.3, 301)
    layer = TARGETS[target]
    for Z1, m1 in IONS:
        want = np.array(oracle_built.stopping(Z1, m1, layer, E))
        got = gpu_engine.stopping(Z1, m1, layer, E, precision="fp32")
        rel = np.abs(got - want) / np.abs(want)
        # linear interpolation in ln E: 1e-5 typical; up to a few 1e-3 next to the
        # kinks where the stopping fit switches branch (material.C:251-268)
        assert np.quantile(rel, 0.95) < 1e-4, (target, Z1, np.quantile(rel, 0.95))
        assert rel.max() < 5e-3, (target, Z1, rel.max())


def _host(args, stdin):
    exe = ROOT / "oracle" / "_build" / "replay_host"
    tables = ROOT / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    r = subprocess.run([str(exe), str(tables), *args], input=stdin, capture_output=True, text=True, check=True)
    return np.array([float.fromhex(v) for v in r.stdout.split()])


@pytest.mark.parametrize("target", sorted(TARGETS))
def test_stopping_fp64_bitwise_vs_host_build(gpu_engine, target):
    layer = TARGETS[target]
    E = np.logspace(-1, 7.2, 211)
    for Z1, m1 in IONS:
        head = f"{Z1} {m1!r} {layer.rho!r} {len(layer.elements)} " + " ".join(
            f"{e.Z} {e.m!r} {e.t!r}" for e in layer.elements)
        want = _host(["--stopping"], head + "\n" + "\n".join(repr(float(x)) for x in E) + "\n")
        got = gpu_engine.stopping(Z1, m1, layer, E, precision="fp64")
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, (target, Z1, E[bad[:5]], got[bad[:5]], want[bad[:5]])


POTENTIALS = ["universal", "moliere", "ckr"]


@pytest.mark.parametrize("pot", range(3))
def test_scatter_fp64_bitwise_vs_host_build(gpu_engine, pot):
    rng = np.random.default_rng(3 + pot)
    eps = 10 ** rng.uniform(-5, 1.5, 20000)
    b = rng.uniform(0, 1, 20000) ** 0.5 * 40 + 1e-6
    want = _host(["--scatter", str(pot)], "\n".join(f"{float(x)!r} {float(y)!r}" for x, y in zip(eps, b)) + "\n")
    got = gpu_engine.scatter(eps, b, precision="fp64", potential=POTENTIALS[pot])
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, (eps[bad[:5]], b[bad[:5]], got[bad[:5]], want[bad[:5]])


@pytest.mark.parametrize("pot", POTENTIALS)
def test_scatter_fp32_matches_fp64(gpu_engine, pot):
    rng = np.random.default_rng(4)
    eps = 10 ** rng.uniform(-4, 1.5, 50000)
    b = rng.uniform(0, 1, 50000) ** 0.5 * 30 + 1e-4
    s64 = gpu_engine.scatter(eps, b, precision="fp64", potential=pot)
    s32 = gpu_engine.scatter(eps, b, precision="fp32", potential=pot)
    model = fp32_scatter_model.s2(pot, eps, b)
    big = s64 > 1e-3
    # the FP32 algorithm (tabulated Newton start for the universal and Moliere
    # potentials) at FP32 rounding; the FP32 form has no cancellation: large angles
    # to 1e-4, small angles to 1e-2
    rel = np.abs(s32 - model) / model
    assert np.quantile(rel[big], 0.99) < 1e-4, np.quantile(rel[big], [0.5, 0.9, 0.99])
    assert np.quantile(rel, 0.99) < 1e-2, np.quantile(rel, [0.5, 0.9, 0.99])
    # against the reference's iterates (the FP64 path): the v, v1 of the magic
    # formula come from the iterate before the last Newton step, which the start
    # point moves within the stopping test's tolerance -- p99 0.5 % (universal),
    # 0.55 % (Moliere); C-Kr starts where the reference does
    rel64 = np.abs(s32 - s64) / s64
    bound = 1e-4 if pot == "ckr" else 1e-2
    assert np.quantile(rel64[big], 0.99) < bound, np.quantile(rel64[big], [0.5, 0.9, 0.99])
    assert np.quantile(rel64, 0.99) < 1e-2, np.quantile(rel64, [0.5, 0.9, 0.99])


def test_potentials_change_the_scattering(gpu_engine):
    """The three potentials give different angles in the screened regime and the
    same Rutherford limit above reduced energy 10 (trim.C:172-179)."""
    eps = np.array([0.01, 0.1, 1.0, 20.0])
    b = np.array([1.0, 1.0, 1.0, 0.05])
    s = [gpu_engine.scatter(eps, b, precision="fp64", potential=p) for p in POTENTIALS]
    assert np.all(s[0][:3] != s[1][:3]) and np.all(s[0][:3] != s[2][:3])
    assert s[0][3] == s[1][3] == s[2][3]
    with pytest.raises(F.EngineError):
        gpu_engine.scatter(eps, b, precision="fp64", potential=3)


def _replay(oracle_built, sim, seed):
    txt = oracle_built.spec_text(sim, seed=seed, philox=True)
    exe = ROOT / "oracle" / "_build" / "replay_host"
    r = subprocess.run([str(exe), str(oracle_built.TABLES)], input=txt, capture_output=True, text=True,
                       check=True)
    rows = []
    for line in r.stdout.splitlines():
        p = line.split()
        rows.append((int(p[0]), int(p[1]), int(p[2]), int(p[3]), int(p[4]), int(p[5]),
                     *(float.fromhex(v) for v in p[6:11])))
    return sorted(rows)


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_trajectories_bitwise_vs_host_build(oracle_built, engine_lib, case):
    sim, seed, _ = CASES[case]
    e = Engine(precision="fp64", seed=seed)
    e.set_record_capacity(200_000)
    e.run([sim])
    rec = e.records()
    e.close()
    got = sorted((int(r["key"]), int(r["species"]), int(r["gen"]), int(r["state"]), int(r["ncoll"]),
                  int(r["nvac"]), float(r["E"]), float(r["x"]), float(r["y"]), float(r["z"]), float(r["eel"]))
                 for r in rec)
    want = _replay(oracle_built, sim, seed)
    assert len(got) == len(want)
    diff = [(a, b) for a, b in zip(got, want) if a != b]
    assert not diff, (len(diff), diff[:3])


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_totals_equal_oracle_on_same_streams(oracle_built, engine_lib, case):
    sim, seed, _ = CASES[case]
    e = Engine(precision="fp64", seed=seed)
    g = e.run([sim])[0]
    e.close()
    o = oracle_built.run(sim, seed=seed, philox=True)
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials", "substitutionals", "lost",
              "range_n"):
        assert g[k] == o[k], (case, k, g[k], o[k])
    for k in ("Eel", "Enuc", "sx", "sxx"):
        assert math.isclose(g[k], o[k], rel_tol=1e-9, abs_tol=1e-6), (case, k, g[k], o[k])
    assert list(g["hist_range"]) == o["hist_range"]


def _z(a, b, key):
    ea, eb = a[key + "_err"], b[key + "_err"]
    return abs(a[key] - b[key]) / math.sqrt(ea * ea + eb * eb)


# FP32 against FP64: within 1 %, resolved at 3 sigma (parity_stats); the FP64 path
# against the reference's own streams at 10^6 ions is in test_gpu_parity_configs.py
N_FP32_CHECK = 200_000


@pytest.mark.parametrize("name", ["cu", "as_layered"])
def test_fp32_matches_fp64(engine_lib, name):
    if name == "cu":
        sim = W.cu_self_ion(n_primaries=N_FP32_CHECK, E=20e3)
    else:
        sim = W.arsenic_implant(n_primaries=N_FP32_CHECK)
        sim.E = 20e3
    _, p64 = PS.run_primaries("fp64", sim, seed=5)
    _, p32 = PS.run_primaries("fp32", sim, seed=6)
    PS.assert_within_one_percent(p32, p64, name)


@pytest.mark.parametrize("case", ["cu_cu_moliere", "kr_c_ckr"])
def test_fp32_matches_fp64_other_potentials(engine_lib, case):
    sim = SimSpec(**{**CASES[case][0].__dict__, "n_primaries": N_FP32_CHECK})
    _, p64 = PS.run_primaries("fp64", sim, seed=9)
    _, p32 = PS.run_primaries("fp32", sim, seed=10)
    PS.assert_within_one_percent(p32, p64, case)


def test_invalid_potential_is_rejected(engine_lib):
    sim = SimSpec(**{**CASES["cu_cu_moliere"][0].__dict__, "n_primaries": 4})
    s = sim.to_c()
    s.potential = 3
    e = Engine(precision="fp64")
    assert e.lib.mtg_prepare(e.ctx, C.byref(s), 1) == 1  # MTG_ERR_BAD_INPUT
    e.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("potential", ["universal", "moliere"])
def test_kernel_levels_agree(engine_lib, prec, potential):
    """The kernel variants (chosen by the features a run uses: none, member records,
    the event log; the Moliere potential takes the geometry-level variants) give the
    same tallies on the same streams: lean, mid and events with the universal
    potential, geometry and full with Moliere."""
    sim = SimSpec(**{**CASES["as_sio2_si_cut"][0].__dict__, "n_primaries": 400, "potential": potential})
    want = ("lean", "mid", "events") if potential == "universal" else ("geometry", "geometry", "full")
    out = []
    for level, name in zip(("plain", "records", "events"), want):
        e = Engine(precision=prec, seed=4)
        if level == "records":
            e.set_record_capacity(1 << 20)
        if level == "events":
            e.set_event_log([F.EV_VACANCY], 1 << 20)
        out.append(e.run([sim])[0])
        assert F.KERNEL_LEVELS[e.stats()["kernel_level"]] == name, (level, name)
        e.close()
    for r in out[1:]:
        if prec == "fp64":
            # the same FP64 arithmetic in every variant: identical trajectories
            for k in ("members", "collisions", "vacancies", "replacements", "interstitials", "lost", "range_n"):
                assert r[k] == out[0][k], k
            for k in ("Eel", "Enuc", "Elost"):
                assert math.isclose(r[k], out[0][k], rel_tol=1e-9), k
            assert list(r["hist_range"]) == list(out[0]["hist_range"])
        else:
            # FP32: the compiler may contract differently per variant; same statistics
            for k in ("members", "collisions", "vacancies", "Eel", "Enuc"):
                assert abs(r[k] - out[0][k]) <= 0.03 * abs(out[0][k]), k


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_energy_conservation(engine_lib, prec):
    sim = W.arsenic_implant(n_primaries=2000)
    e = Engine(precision=prec, seed=3)
    t = e.run([sim])[0]
    e.close()
    total = t["Eel"] + t["Enuc"] + t["Elost"] + t["Eunfollowed"]
    tol = 1e-12 if prec == "fp64" else 2e-6
    assert abs(total - sim.E * sim.n_primaries) <= tol * sim.E * sim.n_primaries


def test_sharded_runs_reproduce_the_whole(engine_lib):
    """Primary ranges run separately sum to the unsplit run (integer tallies exactly)."""
    sim = W.cu_self_ion(n_primaries=1500, E=5e3)
    e = Engine(precision="fp64", seed=9)
    whole = e.run([sim])[0]
    parts = []
    for first, n in ((0, 700), (700, 800)):
        s = SimSpec(**{**sim.__dict__, "n_primaries": n, "first_primary": first})
        parts.append(e.run([s])[0])
    e.close()
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials", "range_n"):
        assert whole[k] == sum(p[k] for p in parts), k
    assert list(whole["hist_range"]) == list(parts[0]["hist_range"] + parts[1]["hist_range"])


def test_cluster_levels(engine_lib):
    """A cluster sample with the universal potential runs the FP32 variants without
    the other potentials' code ("clusters", "clusters+events"), with the tallies of
    each other; FP64 runs it in the geometry variant."""
    sim = SimSpec(**{**CASES["xe_uo2_clusters"][0].__dict__, "n_primaries": 300})
    out = []
    for prec, events, want in (("fp32", False, "clusters"), ("fp32", True, "clusters+events"),
                               ("fp64", False, "geometry")):
        e = Engine(precision=prec, seed=4)
        if events:
            e.set_event_log([F.EV_VACANCY], 1 << 20)
        out.append(e.run([sim])[0])
        assert F.KERNEL_LEVELS[e.stats()["kernel_level"]] == want, (prec, events)
        e.close()
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials"):
        assert out[0][k] == out[1][k], k


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_overflow_drain_gives_identical_results(engine_lib, prec):
    """A recoil stack of 4 entries per warp forces spills to the overflow list and
    drain passes; the integer tallies are unchanged."""
    sim = W.cu_self_ion(n_primaries=300, E=20e3)
    e = Engine(precision=prec, seed=4)
    ref = e.run([sim])[0]
    e.configure(precision=prec, seed=4, stack_capacity=4)
    small = e.run([sim])[0]
    st = e.stats()
    e.close()
    assert st["overflowed"] > 0
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials"):
        assert ref[k] == small[k], k


def test_exhausted_overflow_list_is_retried(engine_lib):
    """8192 Cu 100 keV cascades (about 1.5e7 members) on 4-entry recoil stacks spill
    millions of members in one pass, more than the 2^20-entry overflow list holds:
    the run is made again with larger lists and gives the tallies of the
    default-stack run exactly."""
    sim = W.cu_self_ion(n_primaries=8192)
    e = Engine(precision="fp32", seed=8)
    ref = e.run([sim])[0]
    assert e.stats()["overflow_retries"] == 0
    e.configure(precision="fp32", seed=8, stack_capacity=4)
    small = e.run([sim])[0]
    st = e.stats()
    again = e.run([sim])[0]  # the enlarged lists are kept for later runs
    st2 = e.stats()
    e.close()
    assert st["overflow_retries"] >= 1 and st2["overflow_retries"] == 0, (st, st2)
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials"):
        assert ref[k] == small[k] == again[k], k


def test_collision_budget_returns_timeout(engine_lib):
    """A per-member collision budget that is too small ends the run with an
    error status (no hang, context stays usable)."""
    sim = W.cu_self_ion(n_primaries=50, E=20e3)
    e = Engine(precision="fp64", seed=1, max_collisions=3)
    with pytest.raises(F.EngineError) as ei:
        e.run([sim])
    assert ei.value.status == 5
    e.configure(precision="fp64", seed=1)
    t = e.run([sim])[0]
    e.close()
    assert t["members"] > 50


def test_bad_input_is_rejected(engine_lib):
    e = Engine(precision="fp64")
    bad = SimSpec(layers=[LayerSpec(1.0, -1.0, [ElementSpec(29, 63.5, 1.0)])], Z=29, m=63.5, E=1e3, n_primaries=1)
    with pytest.raises(F.EngineError) as ei:
        e.run([bad])
    assert ei.value.status == 1
    e.close()


def test_multi_simulation_run(engine_lib):
    """Simulation 0 of a batch replays its standalone run exactly; the others are
    independent and statistically consistent."""
    a = W.cu_self_ion(n_primaries=400, E=5e3)
    b = W.boron_implant(n_primaries=400)
    e = Engine(precision="fp64", seed=2)
    alone = e.run([a])[0]
    both = e.run([a, b, b])
    e.close()
    for k in ("members", "collisions", "vacancies"):
        assert both[0][k] == alone[k]
    s1, s2 = summarize(both[1]), summarize(both[2])
    assert both[1]["vacancies"] != both[2]["vacancies"]
    assert _z(s1, s2, "vac_per_ion") < 4.0


def test_sputter_and_voxels_match_oracle(oracle_built, engine_lib):
    """Sputter counts, backscattering and the deposition voxels of the FP64 engine
    equal the oracle on the same streams (counts exactly; voxel sums to float
    accumulation accuracy)."""
    sim = W.gold_deposition(n_primaries=40, voxels=40)
    sim.E = 100e3
    e = Engine(precision="fp64", seed=21)
    g = e.run([sim])[0]
    vox = e.voxels(0)
    e.close()
    o = oracle_built.run(sim, seed=21, philox=True)
    for k in ("sputtered", "backscattered", "lost", "members", "vacancies"):
        assert g[k] == o[k], (k, g[k], o[k])
    assert g["sputtered"] > 0
    assert math.isclose(g["Esputtered"], o["Esputtered"], rel_tol=1e-9)
    assert math.isclose(g["Evoxel"], o["Evoxel"], rel_tol=1e-5)
    depth = vox.sum(axis=(0, 1), dtype=np.float64)
    ref = np.array(o["vox_depth"])
    assert np.allclose(depth, ref, rtol=1e-4, atol=1e-3 * ref.max())


def test_fp32_voxels_conserve_energy(engine_lib):
    """FP32: the deposited energy inside a box that contains the whole cascade equals
    electronic + nuclear loss."""
    sim = W.gold_deposition(n_primaries=300, voxels=64)
    sim.E = 50e3
    sim.voxel_origin = (-2000.0, -4000.0, -4000.0)
    sim.voxel_size = (10000.0, 8000.0, 8000.0)
    e = Engine(precision="fp32", seed=22)
    t = e.run([sim])[0]
    vox = e.voxels(0)
    e.close()
    inside = float(vox.sum(dtype=np.float64))
    assert math.isclose(inside, t["Evoxel"], rel_tol=1e-6)
    assert math.isclose(t["Evoxel"], t["Eel"] + t["Enuc"], rel_tol=2e-4)


def test_lateral_histogram(engine_lib):
    """The lateral (y, z) histogram of stopping points holds every stopped primary that
    lands inside it, and its first moments equal the range tallies'."""
    sim = W.arsenic_implant(n_primaries=4000)
    e = Engine(precision="fp32", seed=12)
    t = e.run([sim])[0]
    e.close()
    h = t["hist_lateral"]
    assert h.shape == (300, 300)
    assert h.sum() <= t["range_n"] and h.sum() >= 0.99 * t["range_n"]
    centres = (np.arange(300) + 0.5) * 10.0 - 1500.0
    my = (h.sum(axis=0) * centres).sum() / h.sum()
    assert abs(my - t["sy"] / t["range_n"]) < 5.0


ALL_EVENTS = [F.EV_VACANCY, F.EV_REPLACEMENT, F.EV_BRANCH, F.EV_DISSIPATE, F.EV_REST, F.EV_LOST, F.EV_HISTORY]


def _cu_sim(n=200, E=5000.0, **kw):
    return SimSpec(layers=[LayerSpec(1e5, 8.96, [ElementSpec(29, 63.546, 1.0, 25.0, 3.0)])], Z=29, m=63.546, E=E,
                   n_primaries=n, hist_vac_bin=1.0, hist_vac_n=2000, **kw)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_event_log_matches_tallies(engine_lib, prec):
    """Every hook call is logged once: counts and energies of the log add up to
    the run's tallies, and the tallies do not change when the log is on."""
    sim = _cu_sim()
    e = Engine(precision=prec, seed=5)
    t0 = e.run([sim])[0]
    e.set_event_log(ALL_EVENTS, 10_000_000)
    t = e.run([sim])[0]
    ev = e.events()
    e.close()
    for key in ("vacancies", "replacements", "collisions", "members"):
        assert t[key] == t0[key], key
    for key in ("Eel", "Enuc"):  # FP64 atomics in lane order: equal to rounding
        assert math.isclose(t[key], t0[key], rel_tol=1e-12), key
    k = ev["kind"]
    assert (k == F.EV_VACANCY).sum() == t["vacancies"]
    assert (k == F.EV_REPLACEMENT).sum() == t["replacements"]
    rest = ev[k == F.EV_REST]
    assert (rest["state"] == 3).sum() == t["interstitials"]
    assert (rest["state"] == 2).sum() == t["substitutionals"]
    assert len(rest) + (k == F.EV_LOST).sum() == t["members"]
    assert set(np.unique(ev["primary"])) == set(range(sim.n_primaries))
    # TrimHistory: one position of the moving atom per displaced recoil, raised by
    # the same atom as the branch event
    hist, br = ev[k == F.EV_HISTORY], ev[k == F.EV_BRANCH]
    assert len(hist) == len(br) > 0
    assert sorted(zip(hist["primary"], hist["key"])) == sorted(zip(br["primary"], br["key"]))
    assert streams_history(ev).shape == (len(hist), 3)
    # TrimPhononOut's split of the nuclear deposit (trim.C:504-527): binding energy of
    # every displaced recoil, dissipated recoils' energy plus binding, residual
    # energy of the members that came to rest
    enuc = (ev["aux"][k == F.EV_BRANCH].sum() + (ev["E"] + ev["aux"])[k == F.EV_DISSIPATE].sum()
            + rest["E"].sum())
    assert enuc == pytest.approx(t["Enuc"], rel=1e-9 if prec == "fp64" else 1e-5)
    if prec == "fp64":
        # the vacancy depth histogram from the logged recoil positions, int(x) bins
        x = ev["x"][k == F.EV_VACANCY]
        x = x[(x > -1.0) & (x < 2000.0)]
        assert np.array_equal(np.bincount(np.trunc(x).astype(np.int64), minlength=2000), t["hist_vac"])


def streams_history(ev):
    from mytrim_gb300 import streams
    return streams.history(ev)


def test_event_log_in_chunks_equals_exact_log(engine_lib):
    """Logs large enough for slots taken eight or sixteen at a time per lane return
    the same records as one filled a slot at a time, without the slots left unused."""
    from mytrim_gb300.streams import _sorted
    sim = _cu_sim(n=400)
    e = Engine(precision="fp32", seed=9)
    e.set_event_log(ALL_EVENTS, 2_000_000)
    e.run([sim])
    exact, n_exact = e.events(), e.event_count()
    lanes = e.stats()["grid"] * e.stats()["block"]
    a = _sorted(exact)
    for chunk in (8, 16):
        e.set_event_log(ALL_EVENTS, 16 * chunk * lanes + 1000)
        e.run([sim])
        chunked, n_chunked = e.events(), e.event_count()
        assert n_exact == n_chunked == len(exact) == len(chunked) > 0, chunk
        assert (chunked["kind"] >= 1).all()
        b = _sorted(chunked)
        for f in exact.dtype.names:
            assert np.array_equal(a[f], b[f]), (chunk, f)
    e.close()


def test_event_log_overflow_keeps_tallies(engine_lib):
    sim = _cu_sim(n=100)
    e = Engine(precision="fp32", seed=6)
    t0 = e.run([sim])[0]
    e.set_event_log([F.EV_DISSIPATE], 50)
    with pytest.raises(F.EngineError) as err:
        e.run([sim])
    assert err.value.status == F.ERR_QUEUE_FULL
    assert e.stats()["events_overflowed"] == 1
    t = e.run([sim], check=False)[0]
    assert len(e.events()) == 50
    t2 = e.run([sim], allow_event_overflow=True)[0]
    e.set_event_log([F.EV_DISSIPATE], 1 << 20)
    e.run([sim])
    assert e.stats()["events_overflowed"] == 0
    e.close()
    for key in ("vacancies", "collisions"):
        assert t[key] == t0[key] and t2[key] == t0[key]
    assert math.isclose(t["Eel"], t0["Eel"], rel_tol=1e-12) and math.isclose(t2["Eel"], t0["Eel"], rel_tol=1e-12)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_vacancy_energy_histogram(engine_lib, prec):
    """TrimVacEnergyCount rows: int(ln E) of the displaced recoil; summed over the
    rows they give the vacancy depth histogram; rows past the last count as dropped."""
    sim = SimSpec(layers=[LayerSpec(1e5, 2.33, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0)])], Z=79, m=196.967,
                  E=20000.0, n_primaries=60, hist_vac_bin=1.0, hist_vac_n=3000, hist_evac_rows=12)
    e = Engine(precision=prec, seed=8)
    e.set_event_log([F.EV_VACANCY], 10_000_000)
    t = e.run([sim])[0]
    ev = e.events()
    h = t["hist_evac"]
    assert h.shape == (12, 3000)
    assert np.array_equal(h.sum(axis=0), t["hist_vac"])
    assert t["hist_dropped"] == 0
    x, E = ev["x"], ev["E"]
    keep = (x > -1.0) & (x < 3000.0)
    rows = np.maximum(np.trunc(np.log(E[keep])).astype(np.int64), 0)
    ref = np.zeros_like(h)
    np.add.at(ref, (rows, np.trunc(x[keep]).astype(np.int64)), 1)
    if prec == "fp64":
        assert np.array_equal(ref, h)
    else:
        assert np.abs(ref - h).sum() <= 1e-3 * h.sum() + 2  # float log at row edges
    # two rows only: the higher-energy vacancies are dropped and counted
    sim.hist_evac_rows = 2
    t2 = e.run([sim])[0]
    e.close()
    assert t2["hist_evac"].sum() + t2["hist_dropped"] == t["hist_vac"].sum()
    assert t2["hist_dropped"] == h[2:].sum()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_cluster_sample_without_clusters_is_the_matrix(engine_lib, prec):
    """A cluster sample with no clusters is the matrix everywhere: the same
    trajectories, hence the same tallies, as a one-layer sample of it."""
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from golden_cases import CASES as GC
    base = GC["xe_uo2_clusters"][0]
    empty = SimSpec(**{**base.__dict__, "clusters": np.zeros((0, 4)), "n_primaries": 30})
    solid = SimSpec(**{**base.__dict__, "geometry": "layers", "layers": [base.layers[0]], "clusters": None,
                       "n_primaries": 30})
    e = Engine(precision=prec, seed=21)
    a = e.run([empty])[0]
    b = e.run([solid])[0]
    e.close()
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials", "range_n"):
        assert a[k] == b[k], k
    for k in ("Eel", "Enuc"):  # FP64 atomics in lane order: equal to rounding
        assert math.isclose(a[k], b[k], rel_tol=1e-12), k


def test_cluster_fp32_matches_fp64(engine_lib):
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from golden_cases import CASES as GC
    sim = SimSpec(**{**GC["xe_uo2_clusters"][0].__dict__, "n_primaries": N_FP32_CHECK})
    _, p64 = PS.run_primaries("fp64", sim, seed=33)
    _, p32 = PS.run_primaries("fp32", sim, seed=34)
    PS.assert_within_one_percent(p32, p64, "xe_uo2_clusters")


def test_event_streams(engine_lib):
    """TrimDefectLog / TrimPhononOut text from the event log: one V line per vacancy,
    one I/S/R line per member at rest with that state, ten fields per ion."""
    from mytrim_gb300 import streams
    sim = _cu_sim(n=50)
    e = Engine(precision="fp64", seed=19)
    e.set_event_log(set(streams.DEFECT_KINDS) | set(streams.PHONON_KINDS), 5_000_000)
    t = e.run([sim])[0]
    ev = e.events()
    e.close()
    d = list(streams.defect_log(ev))
    assert sum(l.startswith("V ") for l in d) == t["vacancies"]
    assert sum(l.startswith("I ") for l in d) == t["interstitials"]
    assert sum(l.startswith("S ") for l in d) == t["substitutionals"]
    assert all(len(l.split()) == 10 for l in d)
    p = list(streams.phonon_log(ev))
    assert all(len(l.split()) == 10 for l in p)
    assert sum(float(l.split()[0]) for l in p) == pytest.approx(t["Enuc"], rel=1e-4)  # 6-digit text


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_event_tags_name_the_cluster_of_birth(engine_lib, prec):
    """IonBase::_tag in the event log: a followed recoil created inside a cluster of a
    sampleClusters sample carries that cluster's index (trim.C:365 with
    sample_clusters.C:53), one created in the matrix -1; in a layered sample every
    tag is -1."""
    sim = SimSpec(**{**CASES["xe_uo2_clusters"][0].__dict__, "n_primaries": 300})
    e = Engine(precision=prec, seed=23)
    e.set_event_log([F.EV_VACANCY, F.EV_REST], 5_000_000)
    e.run([sim])
    ev = e.events()
    e.close()
    cl = np.asarray(sim.clusters)
    box = np.asarray(sim.size)
    vac = ev[ev["kind"] == F.EV_VACANCY]
    pos = np.stack([vac["x"], vac["y"], vac["z"]], axis=1)
    inside = vac["tag"] >= 0
    assert inside.any() and (~inside).any()
    # a tagged vacancy lies in its cluster (periodic images), an untagged one in none
    d = pos[inside] - cl[vac["tag"][inside], :3]
    d -= np.round(d / box) * box
    r = cl[vac["tag"][inside], 3]
    assert np.all(np.sqrt((d * d).sum(axis=1)) <= r * (1 + 1e-5) + 1e-3)
    for q in pos[~inside][:2000]:
        dd = q - cl[:, :3]
        dd -= np.round(dd / box) * box
        assert np.all(np.sqrt((dd * dd).sum(axis=1)) >= cl[:, 3] * (1 - 1e-5) - 1e-3)
    rest = ev[ev["kind"] == F.EV_REST]
    assert (rest["tag"] >= 0).any() and (rest["tag"] < len(cl)).all()
    # layered sample: no tags
    e = Engine(precision=prec, seed=23)
    e.set_event_log([F.EV_VACANCY, F.EV_REST], 5_000_000)
    e.run([_cu_sim(n=20)])
    ev = e.events()
    e.close()
    assert (ev["tag"] == -1).all()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_autotune_chooses_settings_that_keep_results(engine_lib, prec):
    """mtg_autotune times trial launches and keeps the fastest settings in the
    context; the integer tallies of a run do not depend on the launch settings (the
    random streams are keyed by member and collision, not by lane)."""
    sim = W.cu_self_ion(n_primaries=20_000, E=20e3)
    e = Engine(precision=prec, seed=41)
    before = e.run([sim])[0]
    tune = e.autotune([sim], trial_primaries=4096)
    after = e.run([sim])[0]
    st = e.stats()
    e.close()
    assert tune["trials"] >= 10
    assert tune["block_threads"] in (64, 128) and 0 <= tune["max_primaries_per_refill"] <= 32
    assert 1 <= tune["refill_min_idle"] <= 32 and tune["stack_capacity"] > 0
    assert tune["best_collisions_per_s"] >= tune["default_collisions_per_s"] > 0
    assert st["block"] == tune["block_threads"] and st["stack_capacity"] == tune["stack_capacity"]
    if tune["max_primaries_per_refill"] > 0:
        assert st["max_take"] == tune["max_primaries_per_refill"]
    for k in ("members", "collisions", "vacancies", "replacements", "interstitials", "range_n"):
        assert before[k] == after[k], k
