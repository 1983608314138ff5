"""Sharding a simulation over processes (one per GPU) and summing the tallies.

Primaries are independent and their random streams depend only on (simulation,
primary index), so rank r of `world` runs the contiguous primary range
`shard_range(n, r, world)` of the same simulation and the element-wise sum of the
ranks' additive tallies equals the unsharded run (integers exactly).  The sum is a
host-side all-reduce through torch.distributed (gloo or NCCL); the cascade data
itself is never exchanged.
"""
import copy

ADDITIVE = ("primaries", "members", "collisions", "vacancies", "replacements", "interstitials",
            "substitutionals", "lost", "Eel", "Enuc", "Elost", "Eunfollowed", "range_n", "sx", "sxx", "sy", "syy",
            "sz", "szz", "vac_s2", "eel_s2", "enuc_s2", "coll_s2", "newton_iterations", "rejection_passes",
            "surrogate_fallbacks")
INTEGER = {"primaries", "members", "collisions", "vacancies", "replacements", "interstitials", "substitutionals",
           "lost", "range_n", "newton_iterations", "rejection_passes", "surrogate_fallbacks"}
HISTS = ("hist_range", "hist_vac", "hist_repl")


def shard_range(n, rank, world):
    """(first, count) of rank's contiguous share of n primaries."""
    lo = (n * rank) // world
    hi = (n * (rank + 1)) // world
    return lo, hi - lo


def shard_sim(sim, rank, world):
    first, count = shard_range(sim.n_primaries, rank, world)
    s = copy.deepcopy(sim)
    s.first_primary = sim.first_primary + first
    s.n_primaries = count
    return s


def reduce_totals(t, dist, device="cpu"):
    """All-reduce (sum) the additive tallies and histograms of one simulation."""
    import torch
    ints = torch.tensor([int(t.get(k, 0)) for k in ADDITIVE if k in INTEGER], dtype=torch.int64, device=device)
    flts = torch.tensor([float(t.get(k, 0.0)) for k in ADDITIVE if k not in INTEGER], dtype=torch.float64, device=device)
    dist.all_reduce(ints)
    dist.all_reduce(flts)
    out = dict(t)
    ii = iter(ints.tolist())
    ff = iter(flts.tolist())
    for k in ADDITIVE:
        out[k] = next(ii) if k in INTEGER else next(ff)
    for h in HISTS:
        if h in t and len(t[h]):
            v = torch.as_tensor(list(t[h]), dtype=torch.int64, device=device)
            dist.all_reduce(v)
            out[h] = v.cpu().numpy()
    return out


def run_sharded(run, sim, rank, world, dist, device="cpu"):
    """Run rank's shard with `run(sim) -> totals` and return the global totals."""
    return reduce_totals(run(shard_sim(sim, rank, world)), dist, device)
