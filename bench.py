#!/usr/bin/env python
"""Benchmark: primary ions per second, full cascade, on one GB300.

Workload: Ag 200 keV into bulk Si (2.33 g/cm3, Edisp 15 eV, Ebind 3 eV), full
recoil cascade -- the surrogate workload of the benchmark suite.  One step is the
configuration's 10^7 fresh primaries through the whole cascade on the FP32 path
(exact scattering); the surrogate path (2^20 primaries per step) and the FP64
path are timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Before the warm-up the autotuner (mtg_autotune) picks the launch settings from
trial launches of 2^18 primaries (untimed; --no-autotune skips it); the line reports
them in config.launch_settings.

Printed JSON line (rank 0):
  value        primaries/s over the K timed steps, device-timed with CUDA events on
               the launching stream, inputs resident in HBM, L2 flushed (256 MiB
               write) before every timed step; a step whose collect() launched
               further drain passes, or made the run again with larger overflow
               lists, is timed to the end of that work
  e2e          the same metric through the public call (host structs in, host
               totals out, uploads and read-back inside the timed region)
  paths        each path on the same workload: fp32 (the headline), surrogate (2^20
               primaries per step), fp64 -- the plain FP64 exact-scattering path,
               2^16 primaries per step, timed like the headline (L2 flushed, CUDA
               events, 3 timed steps) with its own e2e and its ratio over the CPU
               baseline; the fast paths' relative differences from FP64 in mean
               range, straggle and vacancies per ion, with their standard errors
  roofline     the cascade kernel: 391 algorithmic operations per collision (300 + 91
               per target element) against the FP32 issue rate, SMs x 128 lanes x
               the measured SM clock; paths.*.roofline_frac the same for each path
               against its own unit (FP64: 2 lanes per SM)
  cpu_baseline the CPU oracle (reference algorithm and RNG) on the host cores
--impl reference times the reference's CPU implementation of the path (the
reference library itself where it was built from source, else the oracle port
pinned bit-identical to it) on every host core.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "primary ions/sec full cascade on 1 GB300: surrogate vs exact FP64, range err <1%"
UNIT = "primary ions/s"
WORKLOAD = "Ag 200 keV into bulk Si (2.33 g/cm3, Edisp 15 eV, Ebind 3 eV), full cascade"
W_COLL = 300 + 91 * 1  # algorithmic ops per collision (one-element target)
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) per collision of the FP32 cascade kernel on this workload:
# ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of 65,536 primaries
# (1.76e9 collisions), divided by its collisions; the traffic grows with the
# collisions a launch processes, so the figure scales to the 10^7-primary launch
DRAM_BYTES_PER_COLLISION_FP32 = 2.09

# name -> (description, builder(n_primaries)); builders from mytrim_gb300.workloads
WORKLOADS = {
    "ag200k_si": (WORKLOAD, "silver_into_silicon"),
    "cu100k_cu": ("Cu 100 keV into bulk Cu (8.96 g/cm3), full cascade", "cu_self_ion"),
    "b10k_sio2_si": ("B 10 keV at 7 deg into 10 nm SiO2 on Si, full cascade", "boron_implant"),
    "as50k_sio2_si": ("As 50 keV at 7 deg into 10 nm SiO2 on Si, full cascade", "arsenic_implant"),
    "au1m_agcusi": ("Au 1 MeV into 50 nm Ag / 200 nm Cu / Si, full cascade, sputter counting (E_surf 3 eV), "
                    "256^3 energy-deposition voxels over 300 x 100 x 100 nm", "gold_deposition"),
    "xe30k_uo2_bubbles": ("Xe 30 keV into UO2 with 200 solid-Xe bubbles of 1.5 nm radius in a periodic 40 nm box "
                          "(sampleClusters geometry), full cascade", "xenon_bubbles"),
    "batched4096": ("4096 independent simulations in one launch (Z1 1-83, E0 1 keV-1 MeV log-uniform, 0-60 deg, "
                    "1-4 layers of Si/Cu/Ag/Au/SiO2/Al2O3 5-500 nm over Si); primaries per simulation "
                    "log-uniform 1e2-1e5 scaled so that one step holds about the batch size", "batched_uneven"),
}


def make_sims(name, n, first=0):
    """the simulations of one step: n primaries (the batched workload: about n, over 4096 simulations)"""
    from mytrim_gb300 import workloads as W
    if name == "batched4096":
        sims = W.batched_uneven(n_sims=4096, seed=1, scale_primaries=n / 5.9e7)
        step = first // max(n, 1)  # fresh primaries of every simulation at each step
        for s in sims:
            s.first_primary = step * s.n_primaries
        return sims
    s = getattr(W, WORKLOADS[name][1])(n_primaries=n)
    s.first_primary = first
    return [s]


def make_sim(name, n):
    return make_sims(name, n)[0]


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--batch", type=int, default=10_000_000,
                   help="primaries per step (default: the 10^7 primaries of the Ag 200 keV configuration)")
    p.add_argument("--surrogate-batch", type=int, default=1 << 20, help="primaries per step of the surrogate leg")
    p.add_argument("--precision", default="auto", choices=["auto", "fp32", "surrogate", "fp64"])
    p.add_argument("--fp64-batch", type=int, default=1 << 16, help="primaries per step of the FP64 leg")
    p.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the FP64 leg")
    p.add_argument("--cpu-per-core", type=int, default=0, help="primaries per core in the CPU sample")
    p.add_argument("--events", default="", help="log these event kinds in every step (comma list of "
                   "vacancy, replacement, branch, dissipate, rest, lost) and report their rate")
    p.add_argument("--event-capacity", type=int, default=1 << 26)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-autotune", action="store_true",
                   help="skip the launch-settings autotuner (mtg_autotune) before the warm-up")
    p.add_argument("--workload", default="ag200k_si", choices=sorted(WORKLOADS),
                   help="ag200k_si is the benchmark; the others are for profiling and checks")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        self.f.flush()
        rows = [l.split(", ") for l in Path(self.f.name).read_text().splitlines() if l.strip()]
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_sample(sim, per_core, seed, reference):
    """Time the CPU oracle on nproc independent processes of `per_core` primaries."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_io
    cores = os.cpu_count() or 1
    s = type(sim)(**{**sim.__dict__, "n_primaries": per_core * cores})
    t0 = time.time()
    r = oracle_io.run_parallel(s, seed=seed, philox=False, procs=cores, reference=reference)
    wall = time.time() - t0
    return r, wall, cores


def have_reference_build():
    ref = ROOT / "oracle" / "_ref" / "ref_driver"
    if not ref.exists():
        return False
    try:
        subprocess.run([str(ref)], input="ion 1 1.0 1.0 0\nlayer 1 1\nelement 1 1 1\n", capture_output=True,
                       text=True, timeout=30, check=True)
        return True
    except Exception:
        return False


def run_reference(a):
    """The reference arm: the reference's CPU implementation on all host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_io
    from mytrim_gb300 import workloads as W
    oracle_io.build(None)
    reference = have_reference_build()
    per_core = a.cpu_per_core or 96
    sim = make_sim(a.workload, 1)
    rates = []
    cores = os.cpu_count() or 1
    for i in range(a.warmup + a.steps):
        r, wall, cores = cpu_sample(sim, per_core, seed=1000 + i, reference=reference)
        if i >= a.warmup:
            rates.append(r["primaries"] / wall)
    value = sum(rates) / len(rates)
    kind = "reference" if reference else "port"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * per_core * cores / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[a.workload][0], "primaries_per_step": per_core * cores,
                   "path": "CPU, FP64, mt19937"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{per_core} primaries per core x {cores} independent processes per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def hbm_line(traffic, kernel_ms):
    """The cascade kernel against the measured HBM copy bandwidth: the DRAM bytes of
    one launch (ncu, profiles/cascade_fp32_agsi.md) over its CUDA-event time."""
    peaks = ROOT / "MEASURED_PEAKS.json"
    if traffic is None or not peaks.exists() or not kernel_ms:
        return None
    peak = json.loads(peaks.read_text()).get("hbm_gbs")
    if not peak:
        return None
    achieved = traffic / (kernel_ms / 1e3) / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}


def dist_setup(a):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        return dist, world, rank, local
    return None, 1, 0, local


def main():
    a = args_parse()
    if a.impl == "reference":
        run_reference(a)
        return
    import torch
    from mytrim_gb300 import build
    build.build()
    from mytrim_gb300 import Engine, summarize
    from mytrim_gb300 import workloads as W

    dist, world, rank, local = dist_setup(a)
    torch.cuda.set_device(local)
    prec = a.precision
    if prec == "auto":
        prec = "fp32"
    eng = Engine(device=local, precision="fp32" if prec == "surrogate" else prec, seed=20261203)
    if prec == "surrogate":
        import numpy as np
        from mytrim_gb300.train_surrogate import PARAMS
        eng.set_surrogate_params(np.load(PARAMS))
        eng.configure(precision="surrogate", seed=20261203)
    stream = torch.cuda.Stream(device=local)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    ev_kinds = [k for k in a.events.split(",") if k]
    if ev_kinds:
        from mytrim_gb300 import _ffi as F
        names = {"vacancy": F.EV_VACANCY, "replacement": F.EV_REPLACEMENT, "branch": F.EV_BRANCH,
                 "dissipate": F.EV_DISSIPATE, "rest": F.EV_REST, "lost": F.EV_LOST}
        eng.set_event_log([names[k] for k in ev_kinds], a.event_capacity)
    n_events = []

    def sims_for(step, batch=None):
        b = batch or a.batch
        return make_sims(a.workload, b, (step * world + rank) * b)

    # launch settings (refill size and threshold, block shape, stack depth) chosen by
    # the autotuner from trial launches of this workload, untimed
    tuning = None
    if not a.no_autotune:
        tuning = eng.autotune(sims_for(0), trial_primaries=1 << 18)

    # warm-up steps (untimed)
    for i in range(a.warmup):
        eng.prepare(sims_for(i))
        eng.launch(stream.cuda_stream)
        eng.collect(allow_event_overflow=True)

    # timed steps: inputs resident, L2 flushed before each step, CUDA events on the
    # launching stream
    times, colls, launches, kernel_ms, prims = [], 0, 0, [], 0
    results = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(a.steps):
            eng.prepare(sims_for(a.warmup + k))
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.launch(stream.cuda_stream)
            e1.record(stream)
            rr = eng.collect(allow_event_overflow=True)
            r = {kk: sum(x[kk] for x in rr) for kk in rr[0] if not kk.startswith("hist") and kk != "status"}
            st = eng.stats()
            if st["drains"] > 1 or st["overflow_retries"] > 0:
                # the extra drain passes (or the run made again with larger overflow
                # lists) were launched by collect(), after e1: time to their end
                e2 = torch.cuda.Event(enable_timing=True)
                e2.record(stream)
                e2.synchronize()
                times.append(e0.elapsed_time(e2) / 1e3)
            else:
                times.append(e0.elapsed_time(e1) / 1e3)
            kernel_ms.append(st["kernel_ms"])
            launches += st["launches"]
            colls += r["collisions"]
            prims += r["primaries"]
            results.append(r)
            if ev_kinds:
                n_events.append(eng.event_count())
    torch.cuda.synchronize()
    clocks = clk.summary()
    total = sum(times)
    if dist:
        t = torch.tensor([total], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
        dist.barrier()
    value = world * prims / total
    coll_rate = colls * world / total

    # end to end through the public call: host structs in, host totals out
    e2e_times = []
    h2d = d2h = 0
    n_step = 0
    for k in range(2):
        ss = sims_for(a.warmup + a.steps + k)
        n_step = sum(x.n_primaries for x in ss)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.run(ss, allow_event_overflow=True)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
        st = eng.stats()
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
    e2e = n_step / statistics.mean(e2e_times) * world

    if rank != 0:
        return
    agg = {k: sum(r[k] for r in results) for k in ("primaries", "collisions", "vacancies", "Eel", "Enuc",
                                                    "range_n", "sx", "sxx", "sy", "syy", "sz", "szz",
                                                    "vac_s2", "eel_s2", "enuc_s2", "coll_s2")}
    fast = summarize(agg)

    def time_path(path, steps, base, batch):
        """device-timed steps of another path on fresh primaries (same workload)"""
        e2 = Engine(device=local, precision="fp64" if path == "fp64" else "fp32", seed=20261203)
        if path == "surrogate":
            import numpy as np
            from mytrim_gb300.train_surrogate import PARAMS
            e2.set_surrogate_params(np.load(PARAMS))
        e2.configure(precision=path, seed=20261203)
        rs, ts = [], []
        for k in range(steps + 1):
            e2.prepare(sims_for(base + k, batch))
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            e2.launch(stream.cuda_stream)
            e1.record(stream)
            rr = e2.collect()
            r = {kk: sum(x[kk] for x in rr) for kk in rr[0] if not kk.startswith("hist") and kk != "status"}
            if k > 0:  # first one is a warm-up
                rs.append(r)
                ts.append(e0.elapsed_time(e1) / 1e3)
        e2.close()
        agg2 = {kk: sum(r[kk] for r in rs) for kk in agg}
        agg2["surrogate_fallbacks"] = sum(r.get("surrogate_fallbacks", 0) for r in rs)
        return summarize(agg2), agg2["primaries"] / sum(ts), agg2

    paths = {prec: {"value": value, "unit": UNIT, "collisions_per_s": coll_rate}}
    if prec != "surrogate" and not a.no_fp64:
        from mytrim_gb300.train_surrogate import PARAMS
        if PARAMS.exists():
            sg, sg_rate, sg_agg = time_path("surrogate", 2, 1000, a.surrogate_batch)
            paths["surrogate"] = {"value": sg_rate, "unit": UNIT, "summary": sg,
                                  "collisions_per_s": sg_rate * sg_agg["collisions"] / max(sg_agg["primaries"], 1),
                                  "fallback_fraction": sg_agg["surrogate_fallbacks"] / max(sg_agg["collisions"], 1)}
    fp64 = None
    if not a.no_fp64 and prec != "fp64":
        # the plain FP64 exact-scattering path, timed like the headline: fresh
        # primaries each step, L2 flushed, CUDA events on the launching stream, one
        # untimed warm-up step; then one step end to end through the public call
        r64, rate64, agg64 = time_path("fp64", a.fp64_steps, 2000, a.fp64_batch)
        e64 = Engine(device=local, precision="fp64", seed=20261203)
        ss = sims_for(3000, a.fp64_batch)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e64.run(ss)
        torch.cuda.synchronize()
        e2e64 = sum(x.n_primaries for x in ss) / (time.perf_counter() - t0)
        st64 = e64.stats()
        e64.close()
        fp64 = {"value": rate64, "unit": UNIT, "primaries_per_step": a.fp64_batch, "steps": a.fp64_steps,
                "l2": "flushed before each timed step",
                "collisions_per_s": rate64 * agg64["collisions"] / max(agg64["primaries"], 1),
                "e2e": {"value": e2e64, "unit": UNIT, "h2d_bytes_per_step": st64["h2d_bytes"],
                        "d2h_bytes_per_step": st64["d2h_bytes"]},
                "range_mean_A": r64["range_mean"], "straggle_A": r64["straggle"], "vac_per_ion": r64["vac_per_ion"]}

        def rel_errors(f):
            d = f["range_mean"] - r64["range_mean"]
            return {"range_mean_A": f["range_mean"],
                    "range_rel_err": d / r64["range_mean"],
                    "range_rel_err_sigma": math.hypot(f["range_mean_err"], r64["range_mean_err"]) / r64["range_mean"],
                    "straggle_rel_err": (f["straggle"] - r64["straggle"]) / r64["straggle"],
                    "straggle_rel_err_sigma": math.hypot(f["straggle_err"], r64["straggle_err"]) / r64["straggle"],
                    "vac_rel_err": (f["vac_per_ion"] - r64["vac_per_ion"]) / r64["vac_per_ion"],
                    "vac_rel_err_sigma": math.hypot(f["vac_per_ion_err"], r64["vac_per_ion_err"]) / r64["vac_per_ion"],
                    "speedup_over_fp64": None}

        paths[prec].update(rel_errors(fast))
        paths[prec]["speedup_over_fp64"] = value / fp64["value"]
        if "surrogate" in paths:
            sgp = paths["surrogate"]
            sgp.update(rel_errors(sgp.pop("summary")))
            sgp["speedup_over_fp64"] = sgp["value"] / fp64["value"]
        paths["fp64"] = fp64
    for v in paths.values():
        v.pop("summary", None)

    # roofline of the cascade kernel: algorithmic ops / kernel time against the FP32
    # issue rate (SMs x 128 lanes x SM clock, one op per lane per cycle)
    props = torch.cuda.get_device_properties(local)
    sm_mhz = clocks.get("sm_mhz") or 1920.0
    peak = props.multi_processor_count * 128 * sm_mhz * 1e6 / 1e12
    # every path against the issue rate of the unit its arithmetic runs on (FP32
    # lanes for the FP32 and surrogate paths, the 2 FP64 lanes per SM for the plain
    # path), with the same algorithmic operations per collision
    lanes = {"fp32": 128, "surrogate": 128, "fp64": 2}
    for name, v in paths.items():
        if v.get("collisions_per_s") and name in lanes:
            unit_peak = props.multi_processor_count * lanes[name] * sm_mhz * 1e6
            v["roofline_frac"] = v["collisions_per_s"] * W_COLL / unit_peak
    per_launch_coll = colls / a.steps
    kms = statistics.mean(kernel_ms)
    achieved = per_launch_coll * W_COLL / (kms / 1e3) / 1e12
    traffic = None
    # the captured figure belongs to the FP32 kernel on the default workload
    if a.workload == "ag200k_si" and prec == "fp32" and not ev_kinds:
        traffic = DRAM_BYTES_PER_COLLISION_FP32 * per_launch_coll
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * total / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec != "fp64" else "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[a.workload][0], "primaries_per_step": a.batch * world, "path": prec,
                   "l2": "flushed before each timed step (256 MiB write)", "seeded": True,
                   "launch_settings": tuning},
        "collisions_per_s": coll_rate,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
        "physics": {"vac_per_ion": fast["vac_per_ion"], "range_mean_A": fast["range_mean"],
                    "straggle_A": fast["straggle"], "lateral_A": fast["lateral"],
                    "collisions_per_ion": fast["coll_per_ion"]},
        "paths": paths,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"derived: {props.multi_processor_count} SMs x 128 FP32 lanes x "
                                    f"{sm_mhz:.0f} MHz measured (MEASURED_PEAKS.json has no FP32 figure)",
                     "work": f"{W_COLL} ops per collision x {per_launch_coll:.4g} collisions per launch",
                     "kernel_ms": kms,
                     "hbm": hbm_line(traffic, kms)},
    }
    if ev_kinds:
        line["events"] = {"kinds": ev_kinds, "capacity": a.event_capacity,
                          "per_step": statistics.mean(n_events), "per_s": sum(n_events) / total,
                          "overflowed": any(n > a.event_capacity for n in n_events)}
    if not a.no_cpu and world == 1:
        cores = os.cpu_count() or 1
        per_core = a.cpu_per_core or 600
        reference = have_reference_build()
        r, wall, cores = cpu_sample(make_sim(a.workload, 1), per_core, seed=7, reference=reference)
        line["cpu_baseline"] = {"value": r["primaries"] / wall, "unit": UNIT, "cores": cores,
                                "kind": "reference" if reference else "port",
                                "sample": f"{per_core} primaries per core x {cores} independent processes "
                                          f"({r['primaries']} primaries, {wall:.1f} s)"}
        # the same-precision comparison: the GPU's FP64 plain path, end to end, over
        # the CPU's FP64 reference algorithm on all host cores
        if "fp64" in paths:
            cpu = line["cpu_baseline"]["value"]
            paths["fp64"]["e2e_over_cpu_baseline"] = paths["fp64"]["e2e"]["value"] / cpu
            paths["fp64"]["over_cpu_baseline"] = paths["fp64"]["value"] / cpu
    print(json.dumps(line), flush=True)
    eng.close()


if __name__ == "__main__":
    main()
