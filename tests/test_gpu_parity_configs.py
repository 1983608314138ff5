"""GPU against the oracle on the measurement configurations (GB300, C ABI).

Exact parity, same random streams.  The FP64 engine and the oracle
(oracle/mtoracle, the reference algorithm of trim.C:36-425 with runmytrim's FIFO
cascade loop, runmytrim.C:71-93) draw the same Philox streams.  The integer
tallies must be equal: cascade members, collisions, vacancies, replacements,
interstitials, substitutionals, lost atoms, primaries at rest, and the range,
vacancy and replacement histograms.  Energy sums and stopping-point moments must
agree to 1e-9.  The configurations are:

* Cu 100 keV into Cu, the full 10^4 primaries;
* B 10 keV and As 50 keV at 7 deg into 10 nm SiO2 on Si, 10^5 and 2*10^4 primaries;
* Ag 200 keV into Si, the benchmark workload, 4000 primaries;
* eight simulations of the 4096-simulation batch (largest Z1, highest energy,
  thickest stack, ...), each against the oracle run on its own;
* the event log (vacancies, replacements, followed and dissipated recoils, rest
  states, losses, history, with IonMDTag's _md) against the oracle's records of the
  same hook calls, and the TrimDefectLog / TrimPhononOut / IonMDTag text streams
  written from them, line for line.

Per primary, the first 400 primaries of each must match: collisions and vacancies
exactly; electronic and nuclear loss and the stopping point to 1e-9.
The two sides use different libm implementations (the engine has its own exp and
log), so results agree to rounding, not bit for bit.

Statistical parity against the reference's own random streams, at 10^6 ions.
The oracle is seeded as runmytrim seeds the reference: a 16-bit mt19937 seed per
primary, drawn from the master stream (runmytrim.C:287-304).  The GPU FP64 plain
path is compared on B 10 keV into SiO2/Si and Cu 10 keV into Cu.  Mean projected
range, straggle, lateral spread, vacancies per ion, and electronic and nuclear
loss per ion must each agree within 3 combined standard errors AND within 1 %.
The FP32 and surrogate paths must be within 1 % of the FP64 plain path on the
same 10^6 primaries, measured with a combined standard error of at most 1/3 %,
so that a 1 % error would show at 3 sigma.
"""
import math

import numpy as np
import pytest

from mytrim_gb300 import workloads as W
from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec

import parity_stats as PS

pytestmark = pytest.mark.gpu

INT_KEYS = ("primaries", "members", "collisions", "vacancies", "replacements", "interstitials", "substitutionals",
            "lost", "range_n")
HISTS = ("hist_range", "hist_vac", "hist_repl")
N_RECORDS = 400


def _configs():
    return {
        "c1_cu100k_cu": W.cu_self_ion(n_primaries=10_000),
        "c2_b10k_sio2_si": W.boron_implant(n_primaries=100_000),
        "c2_as50k_sio2_si": W.arsenic_implant(n_primaries=20_000),
        "c4_ag200k_si": W.silver_into_silicon(n_primaries=4_000),
    }


@pytest.mark.parametrize("name", sorted(_configs()))
def test_fp64_equals_oracle_on_same_streams(oracle_built, engine_lib, name):
    sim = _configs()[name]
    seed = 1
    g, p = PS.run_primaries("fp64", sim, seed)
    o = oracle_built.run_parallel(sim, seed=seed, philox=True)
    for k in INT_KEYS:
        assert g[k] == o[k], (name, k, g[k], o[k])
    for h in HISTS:
        assert list(g[h]) == list(o[h]), (name, h)
    for k in ("Eel", "Enuc", "Elost", "Eunfollowed", "sx", "sxx", "sy", "syy", "sz", "szz"):
        assert math.isclose(g[k], o[k], rel_tol=1e-9, abs_tol=1e-6), (name, k, g[k], o[k])
    # per-ion: the first primaries one by one
    r = oracle_built.run(sim, seed=seed, philox=True, n=N_RECORDS, records=N_RECORDS)["records"]
    assert len(r) == N_RECORDS
    n_rest = 0
    for rec in r:
        i = rec["index"]
        assert (p["collisions"][i], p["vacancies"][i]) == (rec["collisions"], rec["vacancies"]), (name, i)
        # the oracle's record holds the stopping point of the last primary that came
        # to rest, so positions are compared for primaries at rest only
        keys = ("eel", "enuc") + (("x", "y", "z") if p["state"][i] in PS.AT_REST else ())
        n_rest += p["state"][i] in PS.AT_REST
        for k in keys:
            assert math.isclose(p[k][i], rec[k], rel_tol=1e-9, abs_tol=1e-6), (name, i, k, p[k][i], rec[k])
    assert n_rest > N_RECORDS // 2


def _pick_c3(sims):
    """eight simulations of the batch that stress it differently"""
    idx = {
        "largest Z1": max(range(len(sims)), key=lambda i: (sims[i].Z, sims[i].E)),
        "highest E0": max(range(len(sims)), key=lambda i: sims[i].E),
        "thickest stack": max(range(len(sims)), key=lambda i: sum(l.thickness for l in sims[i].layers[:-1])),
        "most layers, steepest": max(range(len(sims)), key=lambda i: (len(sims[i].layers), -sims[i].dir[0])),
        "lightest ion": min(range(len(sims)), key=lambda i: (sims[i].Z, -sims[i].n_primaries)),
        "most primaries": max(range(len(sims)), key=lambda i: sims[i].n_primaries),
        "lowest E0": min(range(len(sims)), key=lambda i: sims[i].E),
        "last": len(sims) - 1,
    }
    return idx


def test_c3_simulations_of_the_batch_equal_oracle(oracle_built, engine_lib):
    """C3: 4096 uneven simulations in one FP64 launch (a thousandth of the
    configuration's primaries: about 6e4); eight of them, each run by the oracle on
    its own with that simulation's keys, give the same integer tallies and range
    histogram exactly and the same energy sums to 1e-9."""
    sims = W.batched_uneven(n_sims=4096, seed=1, scale_primaries=1e-3)
    from mytrim_gb300 import Engine
    e = Engine(precision="fp64", seed=7)
    out = e.run(sims)
    e.close()
    for label, i in _pick_c3(sims).items():
        o = oracle_built.run_parallel(sims[i], seed=7, philox=True, sim_index=i)
        g = out[i]
        for k in INT_KEYS:
            assert g[k] == o[k], (label, i, k, g[k], o[k])
        assert list(g["hist_range"]) == list(o["hist_range"]), (label, i)
        for k in ("Eel", "Enuc", "Elost", "sx", "sxx"):
            assert math.isclose(g[k], o[k], rel_tol=1e-9, abs_tol=1e-6), (label, i, k, g[k], o[k])


ALL_EVENTS = (1, 2, 3, 4, 5, 6, 7)  # vacancy, replacement, branch, dissipate, rest, lost, history


def _as_event_array(records, like):
    """oracle event records as the GPU's structured event array"""
    out = np.zeros(len(records), dtype=like.dtype)
    for k in ("kind", "key", "primary", "gen", "Z", "state", "md", "x", "y", "z", "E", "aux", "m"):
        out[k] = [r[k] for r in records]
    out["sim"] = 0
    out["tag"] = -1
    return out


@pytest.mark.parametrize("name", ["cu5k_cu", "as20k_sio2_si_cut", "xe20k_xe_mdtag"])
def test_event_streams_equal_oracle(oracle_built, engine_lib, name):
    """The event log -- the hook calls TrimDefectLog, TrimPhononOut and TrimHistory
    stream (trim.C:467-527, trim.h:139-153) -- against the oracle's records of the
    same hook calls on the same streams: the same events, integer fields exactly,
    positions and energies to 1e-9, and the TrimDefectLog and TrimPhononOut text
    (mytrim_gb300.streams) line for line."""
    from mytrim_gb300 import Engine, streams
    from mytrim_gb300 import _ffi as F
    if name == "cu5k_cu":
        sim = W.cu_self_ion(n_primaries=300, E=5e3)
    elif name == "xe20k_xe_mdtag":
        # IonMDTag: Xe members that start inside the MD gap (200 eV - 12 keV) carry _md 1
        sim = SimSpec(layers=[LayerSpec(1e5, 3.5, [ElementSpec(54, 131.29, 1.0, 25.0, 3.0)])], Z=54, m=131.29,
                      E=20e3, n_primaries=40, md_tag_Z=54, md_tag_E=(200.0, 12000.0))
    else:
        sim = W.arsenic_implant(n_primaries=300)
        sim.E = 20e3
    e = Engine(precision="fp64", seed=31)
    e.set_event_log(ALL_EVENTS, 10_000_000)
    t = e.run([sim])[0]
    ev = e.events()
    e.close()
    o = oracle_built.run_parallel(sim, seed=31, philox=True, event_mask=sum(1 << k for k in ALL_EVENTS))
    oe = _as_event_array(o["events"], ev)
    assert len(ev) == len(oe) > 1000
    assert (ev["kind"] == F.EV_VACANCY).sum() == t["vacancies"]
    if name == "as20k_sio2_si_cut":
        assert (ev["kind"] == F.EV_LOST).sum() == t["lost"] > 0
    a, b = streams._sorted(ev), streams._sorted(oe)
    for k in ("kind", "key", "primary", "gen", "Z", "state", "tag", "md"):
        assert np.array_equal(a[k], b[k]), (name, k)
    for k in ("x", "y", "z", "E", "aux", "m"):
        assert np.allclose(a[k], b[k], rtol=1e-9, atol=1e-6), (name, k)
    assert list(streams.defect_log(ev)) == list(streams.defect_log(oe))
    assert list(streams.phonon_log(ev)) == list(streams.phonon_log(oe))
    assert list(streams.md_tag_log(ev)) == list(streams.md_tag_log(oe))
    tagged = ev[ev["md"] == 1]
    if name == "xe20k_xe_mdtag":
        assert len(tagged) > 0 and (tagged["gen"] > 0).all()  # recoils born in the gap; the primaries are not
        assert np.isin(tagged["kind"], (F.EV_REST, F.EV_LOST, F.EV_HISTORY)).all()
    else:
        assert len(tagged) == 0


def _copper_10k(n):
    return SimSpec(layers=[LayerSpec(1e7, 8.96, [ElementSpec(29, 63.546, 1.0, 25.0, 3.0)])], Z=29, m=63.546,
                   E=10e3, Ef=5.0, n_primaries=n)


STAT_CASES = {
    "b10k_sio2_si": lambda n: W.boron_implant(n_primaries=n),
    "cu10k_cu": _copper_10k,
}
N_STAT = 1_000_000


@pytest.fixture(scope="module")
def reference_stream_runs(oracle_built, engine_lib):
    """Each case once: the oracle on the reference's seeding, and the GPU FP64 path."""
    out = {}
    for name, mk in STAT_CASES.items():
        sim = mk(N_STAT)
        o = oracle_built.run_parallel(sim, seed=20260101, philox=False)
        assert o["primaries"] == N_STAT
        _, p = PS.run_primaries("fp64", sim, seed=20260102)
        out[name] = (sim, o, p)
    return out


@pytest.mark.parametrize("name", sorted(STAT_CASES))
def test_fp64_statistics_vs_reference_streams(reference_stream_runs, name):
    """the plain method's criterion: 3 sigma AND 1 % at 10^6 ions"""
    sim, o, p = reference_stream_runs[name]
    res = PS.compare(p, o)
    for q, (rel, sig, a, b) in res.items():
        assert abs(rel) < 3.0 * sig and abs(rel) < 0.01, (name, q, PS.report(res))


@pytest.mark.parametrize("prec", ["fp32", "surrogate"])
@pytest.mark.parametrize("name", sorted(STAT_CASES))
def test_fast_paths_within_one_percent_of_fp64(reference_stream_runs, prec, name):
    """FP32 and surrogate paths within 1 % of the FP64 plain path, resolved at 3 sigma"""
    sim, _, p64 = reference_stream_runs[name]
    params = None
    if prec == "surrogate":
        from mytrim_gb300.train_surrogate import PARAMS
        params = np.load(PARAMS)
    _, p = PS.run_primaries(prec, sim, seed=20260103, params=params)
    PS.assert_within_one_percent(p, p64, f"{prec} {name}")
