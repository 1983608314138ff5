"""The engine's FP64 exp and log (mytrim_gb300/csrc/mtg_common.cuh), host build:
the short routes that keep compares, conversions and scaling off the FP64 unit
(exp64, log64) equal the full-range forms (exp64_wide, log64_wide) bit for bit,
on random bit patterns, values of every magnitude and the edges of the short
routes.  The device build of the same code is checked against this host build by
the scattering and stopping tests in test_gpu_engine.py."""
import subprocess

from oracle_io import ORACLE_DIR  # noqa: F401  (path setup via conftest)


def test_short_routes_equal_full_range_forms(oracle_built):
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    exe = root / "oracle" / "_build" / "replay_host"
    tables = root / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    r = subprocess.run([str(exe), str(tables), "--mathcheck", "500000"], capture_output=True, text=True)
    checked, bad = (int(v) for v in r.stdout.split()[-2:])
    assert checked > 1_900_000
    assert bad == 0, r.stdout
    assert r.returncode == 0
