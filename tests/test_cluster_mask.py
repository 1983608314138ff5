"""The cluster lookup's candidate lists (mytrim_gb300/csrc/mtg_geometry.cuh, built by
mtg_setup.cpp): with them the lookup answers exactly as the hash search of
sampleClusters::lookupCluster (sample_clusters.C:60-130) without them, in double
and in float, at random points inside the box, far out on periodic axes and on
cluster surfaces (host build of the same code, oracle/_build/replay_host
--lookupcheck), for separate, overlapping and box-spanning clusters."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _spec(box, bc, clusters, kn):
    lines = ["seed 1", "ion 54 132 30000 10", f"size {box[0]!r} {box[1]!r} {box[2]!r}",
             f"bc {bc[0]} {bc[1]} {bc[2]}", "layer 400 10", "element 92 235 1", "element 8 16 2",
             "layer 400 3.5", "element 54 132 1", f"clusters {kn[0]} {kn[1]} {kn[2]}"]
    lines += ["cluster " + " ".join(repr(float(v)) for v in c) for c in clusters]
    return "\n".join(lines) + "\n"


def _clusters(n, rmin, rmax, box, seed, inside=True):
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 4))
    for i in range(n):
        lo = 0.0 if inside else -0.2
        out[i, :3] = rng.uniform(lo, 1.0 - lo, 3) * np.asarray(box)
        out[i, 3] = rng.uniform(rmin, rmax)
    return out


CASES = {
    "periodic": ((400.0, 400.0, 400.0), (0, 0, 0), _clusters(40, 15, 20, (400, 400, 400), 1), (19, 19, 19)),
    "cut_inf_mix": ((300.0, 500.0, 200.0), (2, 1, 0), _clusters(60, 5, 25, (300, 500, 200), 2, inside=False),
                    (8, 12, 5)),
    "spanning_spheres": ((100.0, 100.0, 100.0), (0, 0, 0), _clusters(5, 40, 70, (100, 100, 100), 3), (4, 4, 4)),
    "many_small": ((200.0, 200.0, 200.0), (0, 1, 0), _clusters(1500, 1.0, 3.0, (200, 200, 200), 4), (40, 40, 40)),
    # most cells hold overlapping candidates and take the search
    "overlapping": ((200.0, 200.0, 200.0), (0, 0, 2), _clusters(400, 10.0, 30.0, (200, 200, 200), 5), (10, 10, 10)),
    # separate bubbles, as the xenon workload places them: nearly every cell answers
    # from its list
    "separate": ((400.0, 400.0, 400.0), (0, 0, 0), None, (19, 19, 19)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_mask_answers_as_the_search(oracle_built, case):
    box, bc, cl, kn = CASES[case]
    if cl is None:
        from mytrim_gb300.workloads import _bubbles
        cl = _bubbles(200, 15.0, 400.0, 3)
    exe = ROOT / "oracle" / "_build" / "replay_host"
    tables = ROOT / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    r = subprocess.run([str(exe), str(tables), "--lookupcheck", "200000"], input=_spec(box, bc, cl, kn),
                       capture_output=True, text=True)
    checked, bad = (int(v) for v in r.stdout.split()[-2:])
    assert checked == 200000
    assert bad == 0, r.stdout
    listed, marked = (int(v) for v in r.stdout.split("cells")[1].split()[:2])
    if case == "separate":  # the lists, not the search, answer near separate bubbles
        assert marked < 0.02 * (listed + marked), (listed, marked)


@pytest.mark.parametrize("case", ["periodic", "many_small", "separate"])
def test_cells_without_lists_answer_as_the_search(oracle_built, case):
    """Where the candidate lists would pass their size cap (here 4096 entries, in a
    build for this test), the cells only mark where a cluster reaches: the lookup
    still answers exactly as the search."""
    box, bc, cl, kn = CASES[case]
    if cl is None:
        from mytrim_gb300.workloads import _bubbles
        cl = _bubbles(200, 15.0, 400.0, 3)
    exe = ROOT / "oracle" / "_build" / "replay_host_smallcap"
    tables = ROOT / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    r = subprocess.run([str(exe), str(tables), "--lookupcheck", "100000"], input=_spec(box, bc, cl, kn),
                       capture_output=True, text=True)
    checked, bad = (int(v) for v in r.stdout.split()[-2:])
    assert checked == 100000
    assert bad == 0, r.stdout
    listed, marked = (int(v) for v in r.stdout.split("cells")[1].split()[:2])
    assert listed == 0 and marked > 0, (listed, marked)
