"""The numpy restatement of the FP32 scattering (tests/fp32_scatter_model.py) that
the GPU test of the FP32 service is pinned to: started from the reference's guess
it reproduces the reference's iterates (the FP64 host build of trim.C:180-271), and
from the tabulated start it lands within the stopping test's slack of the
converged root, closer than the reference does."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import fp32_scatter_model as M

ROOT = Path(__file__).resolve().parent.parent
POT_INDEX = {"universal": 0, "moliere": 1, "ckr": 2}


def _sample(n, seed):
    rng = np.random.default_rng(seed)
    return 10 ** rng.uniform(-4, 1.0, n), rng.uniform(0, 1, n) ** 0.5 * 30 + 1e-4


@pytest.mark.parametrize("pot", sorted(POT_INDEX))
def test_reference_start_matches_host_build(oracle_built, pot):
    eps, b = _sample(4000, 11)
    exe = ROOT / "oracle" / "_build" / "replay_host"
    tables = ROOT / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    r = subprocess.run([str(exe), str(tables), "--scatter", str(POT_INDEX[pot])],
                       input="\n".join(f"{float(x)!r} {float(y)!r}" for x, y in zip(eps, b)) + "\n",
                       capture_output=True, text=True, check=True)
    host = np.array([float.fromhex(v) for v in r.stdout.split()])
    model = M.s2(pot, eps, b, start="reference")
    rel = np.abs(model - host) / host
    # the same iterates in another arrangement of the arithmetic: rounding only
    assert np.quantile(rel, 0.99) < 1e-9 and rel.max() < 1e-6, (np.quantile(rel, 0.99), rel.max())


@pytest.mark.parametrize("pot", ["universal", "moliere"])
def test_table_start_is_near_the_converged_root(pot):
    eps, b = _sample(20000, 12)
    exact = M.converged_s2(pot, eps, b)
    big = exact > 1e-3
    tab = np.abs(M.s2(pot, eps, b) / exact - 1)[big]
    ref = np.abs(M.s2(pot, eps, b, start="reference") / exact - 1)[big]
    assert np.quantile(tab, 0.99) < 2e-3, np.quantile(tab, 0.99)
    assert np.quantile(tab, 0.99) < np.quantile(ref, 0.99)
