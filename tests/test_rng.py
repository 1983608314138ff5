"""The engine's counter-based generators (mytrim_gb300/csrc/mtg_common.cuh, host
build): Philox4x32-10 and Philox2x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011) against
a Python restatement of the published round function, and the uniformity of the
24-bit variates the FP32 engine draws from them."""
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
M = 0xFFFFFFFF


def philox4(c, k0, k1):
    x, y, z, w = c
    for _ in range(10):
        p0, p1 = 0xD2511F53 * x, 0xCD9E8D57 * z
        x, y, z, w = ((p1 >> 32) ^ y ^ k0) & M, p1 & M, ((p0 >> 32) ^ w ^ k1) & M, p0 & M
        k0, k1 = (k0 + 0x9E3779B9) & M, (k1 + 0xBB67AE85) & M
    return x, y, z, w


def philox2(c, k):
    x, y = c
    for _ in range(10):
        p = 0xD256D193 * x
        x, y = ((p >> 32) ^ k ^ y) & M, p & M
        k = (k + 0x9E3779B9) & M
    return x, y


def _host(lines):
    exe = ROOT / "oracle" / "_build" / "replay_host"
    tables = ROOT / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    r = subprocess.run([str(exe), str(tables), "--philox"], input="".join(lines), capture_output=True, text=True,
                       check=True)
    return [tuple(int(v, 16) for v in l.split()) for l in r.stdout.splitlines()]


def test_philox_rounds_match_the_published_function(oracle_built):
    rng = np.random.default_rng(7)
    words = rng.integers(0, 1 << 32, size=(200, 6), dtype=np.uint64).tolist()
    words += [[0] * 6, [M] * 6]
    got = _host(["%x %x %x %x %x %x\n" % tuple(w) for w in words])
    for w, g in zip(words, got):
        assert g[:4] == philox4(w[:4], w[4], w[5])
        assert g[4:] == philox2(w[:2], w[4])


def test_24_bit_variates_are_uniform(oracle_built):
    # 2^16 counters through both generators; every output word's top 24 bits in 64 bins
    n = 1 << 16
    lines = ["%x %x %x %x %x %x\n" % (i, i >> 7, 3, 0, 0x1234, 0x5678) for i in range(n)]
    out = np.array(_host(lines), dtype=np.uint64)
    for col in range(6):
        h = np.bincount((out[:, col] >> np.uint64(26)).astype(np.int64), minlength=64)
        chi2 = float(((h - n / 64) ** 2 / (n / 64)).sum())
        assert chi2 < 130.0, (col, chi2)  # 63 degrees of freedom: p about 1e-6
