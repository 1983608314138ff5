"""Statistics for comparing cascade runs (test helper, not a test module).

The quantities the cascade path is judged on: mean projected range, straggle
and lateral spread of the primaries that came to rest, vacancies per ion, and
the split of the beam energy into electronic and nuclear loss per ion.

Standard errors come from each statistic's influence function evaluated on the
GPU's per-primary results (mtg_get_primaries): for a mean the deviations
themselves, for the straggle s = sd(x) the values ((x - mean)^2 - s^2) / 2s,
for the lateral spread L = sqrt(var y + var z) the values
((y - my)^2 + (z - mz)^2 - L^2) / 2L.  This takes the fourth moments of the
range distribution into account instead of assuming it is normal.

The oracle's tallies are sums only.  Under the hypothesis being tested (the two
runs sample the same distribution) its per-primary spread is the GPU's, so its
standard error is the GPU's per-primary spread over the square root of its own
effective sample size.  With the reference's seeding (runmytrim.C:287-304: a
16-bit seed per primary drawn from the master mt19937, simconf.C:66-71) several
primaries share a seed and repeat one cascade exactly; the variance of a mean
over N primaries is then sum_s n_s^2 / N^2 times the per-cascade variance
(n_s: primaries that drew seed s), which the oracle reports as seed_sq.
"""
import math

import numpy as np

QUANTITIES = ("range_mean", "straggle", "lateral", "vac_per_ion", "eel_per_ion", "enuc_per_ion")
AT_REST = (1, 2, 3)  # final states of a primary that came to rest inside the sample


def per_primary_stats(p):
    """Values and per-primary influence spreads from GPU per-primary arrays."""
    rest = np.isin(p["state"], AT_REST)
    x, y, z = p["x"][rest], p["y"][rest], p["z"][rest]
    out = {"n_all": len(p["state"]), "n_rest": int(rest.sum())}

    def mean(v, key, n_key):
        v = np.asarray(v, dtype=np.float64)
        out[key] = float(v.mean())
        out[key + "_sd"] = float(v.std())
        out[key + "_n"] = n_key

    mean(p["vacancies"], "vac_per_ion", "n_all")
    mean(p["eel"], "eel_per_ion", "n_all")
    mean(p["enuc"], "enuc_per_ion", "n_all")
    mean(x, "range_mean", "n_rest")
    dx = x - x.mean()
    s2 = float(np.mean(dx * dx))
    s = math.sqrt(s2)
    out["straggle"] = s
    out["straggle_sd"] = float(np.std((dx * dx - s2) / (2.0 * s)))
    out["straggle_n"] = "n_rest"
    r2 = (y - y.mean()) ** 2 + (z - z.mean()) ** 2
    L2 = float(r2.mean())
    L = math.sqrt(L2)
    out["lateral"] = L
    out["lateral_sd"] = float(np.std((r2 - L2) / (2.0 * L)))
    out["lateral_n"] = "n_rest"
    return out


def totals_stats(t):
    """Values of the same statistics from summed tallies (oracle or GPU totals)."""
    n = t["primaries"]
    rn = t["range_n"]
    mx, my, mz = t["sx"] / rn, t["sy"] / rn, t["sz"] / rn
    vx = t["sxx"] / rn - mx * mx
    vy = t["syy"] / rn - my * my
    vz = t["szz"] / rn - mz * mz
    return {"n_all": n, "n_rest": rn, "range_mean": mx, "straggle": math.sqrt(vx), "lateral": math.sqrt(vy + vz),
            "vac_per_ion": t["vacancies"] / n, "eel_per_ion": t["Eel"] / n, "enuc_per_ion": t["Enuc"] / n}


def design_effect(t):
    """Variance inflation of a run-wide mean from repeated seeds (1 without)."""
    sq = t.get("seed_sq")
    if not sq:
        return 1.0
    return float(sq) / float(t["primaries"])


def compare(gpu_primaries, other, other_is_gpu=None):
    """Relative differences and their combined standard errors, per quantity.

    gpu_primaries: per-primary arrays of a GPU run (the run under test);
    other: the comparison run, either summed oracle tallies (with seed_sq for
    the reference's seeding) or, with other_is_gpu, another GPU run's
    per-primary arrays.  Returns {quantity: (rel, rel_sigma, value, other_value)}.
    """
    g = per_primary_stats(gpu_primaries)
    if other_is_gpu:
        o = per_primary_stats(other)
        D = 1.0
    else:
        o = totals_stats(other)
        D = design_effect(other)
    out = {}
    for q in QUANTITIES:
        nk = g[q + "_n"]
        se_g = g[q + "_sd"] / math.sqrt(g[nk])
        sd_o = o[q + "_sd"] if other_is_gpu else g[q + "_sd"]
        se_o = sd_o * math.sqrt(D / o[nk])
        ref = o[q]
        out[q] = ((g[q] - ref) / ref, math.hypot(se_g, se_o) / abs(ref), g[q], ref)
    return out


def report(res):
    return "; ".join(f"{q} {v[2]:.6g} vs {v[3]:.6g}: {100 * v[0]:+.3f}% (sigma {100 * v[1]:.3f}%)"
                     for q, v in res.items())


def run_primaries(prec, sim, seed, params=None):
    """One GPU run: (totals, per-primary arrays)."""
    from mytrim_gb300 import Engine
    e = Engine(precision="fp32" if prec == "surrogate" else prec, seed=seed)
    try:
        if prec == "surrogate":
            e.set_surrogate_params(params)
            e.configure(precision="surrogate", seed=seed)
        t = e.run([sim])[0]
        return t, e.primaries(0, sim.n_primaries)
    finally:
        e.close()


def assert_within_one_percent(p_fast, p_ref, label, quantities=QUANTITIES):
    """The fast path's statistics within 1 % of the reference run's, with a combined
    standard error of at most 1/3 %, so that a 1 % error would show at 3 sigma."""
    res = compare(p_fast, p_ref, other_is_gpu=True)
    for q in quantities:
        rel, sig, _, _ = res[q]
        assert sig < 0.01 / 3.0, (label, q, "sample too small to resolve 1 %", report(res))
        assert abs(rel) < 0.01, (label, q, report(res))
    return res
