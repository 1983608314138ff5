"""The engine's FP64 exp and log (mytrim_gb300/csrc/mtg_common.cuh), host build:
the short routes that keep compares, conversions and scaling off the FP64 unit
(exp64, log64) equal the full-range forms (exp64_wide, log64_wide) bit for bit,
on random bit patterns, values of every magnitude and the edges of the short
routes; and their accuracy in ulps against 50-digit evaluations.  The device
build of the same code is checked against this host build by the scattering and
stopping tests in test_gpu_engine.py."""
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


def _engine_eval(fn, rows):
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    exe = root / "oracle" / "_build" / "replay_host"
    tables = root / "mytrim_gb300" / "data" / "stopping_tables.tsv"
    txt = "\n".join(" ".join(float(v).hex() for v in r) for r in rows) + "\n"
    r = subprocess.run([str(exe), str(tables), "--eval", fn], input=txt, capture_output=True, text=True, check=True)
    return [float.fromhex(v) for v in r.stdout.split()]


def _ulp_errors(got, exact):
    import math
    import mpmath
    out = []
    for g, e in zip(got, exact):
        u = math.ulp(abs(float(e)))
        out.append(float(abs(mpmath.mpf(g) - e) / u))
    return out


def test_exp_log_pow_accuracy_in_ulps(oracle_built):
    """exp64, log64 and pow64 against 50-digit evaluations (mpmath): exp within 0.6
    ulp and log within 0.7 ulp of the exact value (Tang's table-driven methods give
    about half an ulp), pow = exp(y log x) within 0.6 + 2 |y ln x| ulp, on the
    argument ranges the collision code uses and across the whole double range."""
    import random
    mpmath = __import__("pytest").importorskip("mpmath")
    mpmath.mp.dps = 50
    rnd = random.Random(20261204)
    xs = [rnd.uniform(-50.0, 50.0) for _ in range(6000)] + [rnd.uniform(-700.0, 700.0) for _ in range(2000)]
    got = _engine_eval("exp", [(x,) for x in xs])
    err = _ulp_errors(got, [mpmath.exp(mpmath.mpf(x)) for x in xs])
    assert max(err) < 0.6, max(err)
    ls = [rnd.uniform(0.5, 2.0) * 2.0 ** rnd.randint(-1000, 1000) for _ in range(5000)]
    ls += [1.0 + rnd.uniform(-1e-3, 1e-3) for _ in range(2000)] + [rnd.uniform(1e-6, 1e6) for _ in range(2000)]
    got = _engine_eval("log", [(x,) for x in ls])
    err = _ulp_errors(got, [mpmath.log(mpmath.mpf(x)) for x in ls])
    assert max(err) < 0.7, max(err)
    # pow = exp(t), t = y log x: the rounding of t (log's and the product's, about 1.2
    # ulp of t) becomes |t| times that in the result, plus exp's own half ulp
    import math
    ps = [(10 ** rnd.uniform(-4, 4), rnd.uniform(-3.0, 3.0)) for _ in range(4000)]
    got = _engine_eval("pow", ps)
    err = _ulp_errors(got, [mpmath.power(mpmath.mpf(x), mpmath.mpf(y)) for x, y in ps])
    bound = [0.6 + 2.0 * abs(y * math.log(x)) for x, y in ps]
    assert all(e < b for e, b in zip(err, bound)), max(e / b for e, b in zip(err, bound))
