"""The Python front's host structures (no GPU): the column-wise conversion of a batch
of simulations (engine.sims_to_array) writes the same bytes as converting each
SimSpec on its own (SimSpec.to_c), and the reference-shaped classes (api.py) build
the SimSpec a reference user's objects describe."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))

import mytrim_gb300 as M  # noqa: E402
from mytrim_gb300 import _ffi as F  # noqa: E402
from mytrim_gb300 import engine as E  # noqa: E402
from mytrim_gb300 import workloads as W  # noqa: E402
from golden_cases import CASES  # noqa: E402


def test_batch_conversion_equals_per_simulation_conversion():
    sims = W.batched_uneven(n_sims=300, seed=3, scale_primaries=0.01) + [c[0] for c in CASES.values()]
    sims += [W.gold_deposition(100), W.boron_implant(10), W.xenon_bubbles(10)]
    sims[5].potential = "ckr"
    sims[6].mode = "primaries"
    sims[6].max_generation = 2
    arr, keep = E.sims_to_array(sims)
    raw = arr.tobytes()
    size = C.sizeof(F.Sim)
    ptr_off = F.Sim.sample.offset + F.Sample.clusters.offset
    assert len(raw) == size * len(sims)
    for k, s in enumerate(sims):
        one = bytes(s.to_c())
        mine = raw[k * size:(k + 1) * size]
        if s.geometry == "clusters":  # the cluster pointers point at different copies
            one, mine = one[:ptr_off] + one[ptr_off + 8:], mine[:ptr_off] + mine[ptr_off + 8:]
        assert one == mine, k
    assert len(keep) == sum(s.geometry == "clusters" for s in sims)


def test_reference_shaped_objects_build_the_simspec():
    sc = M.SimconfType(seed=3)
    sample = M.sampleClusters(400.0, 300.0, 200.0)
    sample.initSpatialhash(10, 8, 6)
    uo2 = M.MaterialBase(sc, 10.0)
    uo2._element = [M.Element(92, 235.0, 1.0), M.Element(8, 16.0, 2.0)]
    xe = M.MaterialBase(sc, 3.5)
    xe._element = [M.Element(54, 132.0, 1.0)]
    sample.material = [uo2, xe]
    sample.addCluster(10.0, 20.0, 30.0, 5.0)
    sample.addCluster(100.0, 200.0, 150.0, 7.5)
    pka = M.IonBase(54, 132.0, 30e3)
    pka._pos = [0.0, 150.0, 100.0]
    trim = M.TrimGPU.__new__(M.TrimGPU)  # no engine: the host-side spec only
    trim._potential, trim._output, trim._primaries_only, trim._max_generation = M.TrimGPU.CKR, "primaries", False, 2
    spec = trim._spec(sample, pka, 100, (10.0, 50), (1.0, 0))
    assert spec.geometry == "clusters" and spec.cluster_hash == (10, 8, 6)
    assert np.array_equal(spec.clusters, [[10.0, 20.0, 30.0, 5.0], [100.0, 200.0, 150.0, 7.5]])
    assert spec.size == (400.0, 300.0, 200.0) and spec.pos == (0.0, 150.0, 100.0)
    assert spec.potential == "ckr" and spec.mode == "primaries" and spec.max_generation == 2
    assert [e.Z for e in spec.layers[0].elements] == [92, 8] and spec.layers[1].rho == 3.5
    s = spec.to_c()
    assert s.sample.geometry == F.GEOM_CLUSTERS and s.sample.n_clusters == 2 and s.potential == F.POT_CKR
