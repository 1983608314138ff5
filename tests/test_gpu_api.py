"""The reference-shaped Python classes (mytrim_gb300/api.py): a run set up the way a
reference user builds SimconfType, MaterialBase, SampleLayers / sampleClusters,
IonBase and a TrimBase gives the same tallies as the engine run of the equivalent
SimSpec, with the same seed (GB300)."""
import numpy as np
import pytest

import mytrim_gb300 as M
from mytrim_gb300 import Engine
from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec

pytestmark = pytest.mark.gpu

KEYS = ("members", "collisions", "vacancies", "replacements", "interstitials", "range_n")


def _si(sc):
    m = M.MaterialBase(sc, 2.33)
    m._element = [M.Element(14, 28.086, 1.0, 15.0, 3.0)]
    m.prepare()
    return m


def test_layers_mode_potential_and_batch(engine_lib):
    sc = M.SimconfType(seed=7)
    sample = M.SampleLayers(1e7, 100.0, 100.0)
    sio2 = M.MaterialBase(sc, 2.2)
    sio2._element = [M.Element(14, 28.086, 1.0, 15.0, 3.0), M.Element(8, 15.999, 2.0, 28.0, 3.0)]
    sample.material = [sio2, _si(sc)]
    sample.layerThickness = [100.0, 1e7]
    pka = M.IonBase(33, 74.922, 20e3)
    pka._pos = [0.0, 50.0, 50.0]
    trim = M.TrimGPU(sc, sample, precision="fp64", output="primaries", max_generation=2)
    trim._potential = M.TrimGPU.MOLIERE
    got = trim.runPrimaries(pka, 200, hist_range=(10.0, 100))
    assert sc.vacancies_created == got["vacancies"] > 0
    spec = SimSpec(layers=[LayerSpec(100.0, 2.2, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0),
                                                  ElementSpec(8, 15.999, 2.0, 28.0, 3.0)]),
                           LayerSpec(1e7, 2.33, [ElementSpec(14, 28.086, 1.0, 15.0, 3.0)])],
                   Z=33, m=74.922, E=20e3, n_primaries=200, pos=(0.0, 50.0, 50.0), size=(1e7, 100.0, 100.0),
                   mode="primaries", max_generation=2, potential="moliere", hist_range_bin=10.0, hist_range_n=100)
    e = Engine(precision="fp64", seed=7)
    want = e.run([spec])[0]
    e.close()
    for k in KEYS:
        assert got[k] == want[k], k
    # runBatch: the first job of a batch replays the single run
    two = trim.runBatch([(sample, pka, 200), (sample, pka, 50)], hist_range=(10.0, 100))
    for k in KEYS:
        assert two[0][k] == want[k], k
    assert two[1]["primaries"] == 50


def test_cluster_sample(engine_lib):
    sc = M.SimconfType(seed=3)
    sample = M.sampleClusters(400.0, 400.0, 400.0)
    sample.initSpatialhash(19, 19, 19)
    uo2 = M.MaterialBase(sc, 10.0)
    uo2._element = [M.Element(92, 235.0, 1.0), M.Element(8, 16.0, 2.0)]
    xe = M.MaterialBase(sc, 3.5)
    xe._element = [M.Element(54, 132.0, 1.0)]
    sample.material = [uo2, xe]
    rng = np.random.default_rng(5)
    cl = []
    for _ in range(30):
        c = rng.uniform(0, 400, 3)
        sample.addCluster(c[0], c[1], c[2], 20.0)
        cl.append([c[0], c[1], c[2], 20.0])
    pka = M.IonBase(54, 132.0, 30e3)
    pka._pos = [0.0, 200.0, 200.0]
    trim = M.TrimGPU(sc, sample, precision="fp32")
    got = trim.runPrimaries(pka, 300)
    spec = SimSpec(layers=[LayerSpec(400.0, 10.0, [ElementSpec(92, 235.0, 1.0), ElementSpec(8, 16.0, 2.0)]),
                           LayerSpec(400.0, 3.5, [ElementSpec(54, 132.0, 1.0)])],
                   Z=54, m=132.0, E=30e3, n_primaries=300, pos=(0.0, 200.0, 200.0), size=(400.0, 400.0, 400.0),
                   geometry="clusters", clusters=np.array(cl), cluster_hash=(19, 19, 19))
    e = Engine(precision="fp32", seed=3)
    want = e.run([spec])[0]
    e.close()
    for k in KEYS:
        assert got[k] == want[k], k
