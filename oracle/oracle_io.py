"""Run the CPU oracles from Python (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module.  It writes a run spec (format in oracle/runspec.h) for a
``mytrim_gb300.SimSpec``, runs ``oracle/_build/mtoracle`` (the C++ restatement)
or ``oracle/_ref/ref_driver`` (the reference library itself, only where the
reference sources were available to build it), and parses the tallies.
Large runs are split over processes by primary subsets and summed.
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REPO = ORACLE_DIR.parent
MTORACLE = ORACLE_DIR / "_build" / "mtoracle"
REF_DRIVER = ORACLE_DIR / "_ref" / "ref_driver"
REF_RUNMYTRIM = ORACLE_DIR / "_ref" / "ref_runmytrim"
REF_RUNSTOPPING = ORACLE_DIR / "_ref" / "ref_runstopping"
TABLES = REPO / "mytrim_gb300" / "data" / "stopping_tables.tsv"

SUM_KEYS = ("primaries", "members", "collisions", "vacancies", "replacements", "interstitials",
            "substitutionals", "lost", "Eel", "Enuc", "Elost", "Eunfollowed", "range_n", "sx", "sxx",
            "sy", "syy", "sz", "szz", "vac_s2", "eel_s2", "enuc_s2", "coll_s2", "sputtered", "backscattered",
            "Esputtered", "Evoxel")


def reference_dir():
    """The reference checkout: $MYTRIM_REFERENCE, else the build recipe's default
    (oracle/Makefile REF); None where it is not present (e.g. on the GPU machine)."""
    ref = os.environ.get("MYTRIM_REFERENCE")
    if not ref:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", str(ORACLE_DIR), "print-ref"],
                           capture_output=True, text=True)
        ref = r.stdout.strip() if r.returncode == 0 else ""
    p = Path(ref) if ref else None
    return p if p is not None and (p / "trim.C").exists() else None


def build(reference_dir=None):
    """Compile the restatement, and the reference driver where the reference's
    sources are present (the argument, else reference_dir())."""
    env = dict(os.environ)
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "all"], check=True, env=env)
    ref = Path(reference_dir) if reference_dir else globals()["reference_dir"]()
    if ref is not None and (ref / "trim.C").exists():
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "ref", f"REF={ref}"], check=True, env=env)


POTENTIALS = {"universal": 0, "moliere": 1, "ckr": 2}  # TrimBase::Potential (trim.h:63-69)


def spec_text(sim, seed=1, philox=True, first=0, n=None, records=0, tmin=None, output=None, scale=1.0,
              sim_index=0, event_mask=0):
    w = sim.box()
    p = sim.start()
    lines = [f"seed {seed}", f"seeding {'philox' if philox else 'compat'}",
             f"ion {sim.Z} {sim.m!r} {sim.E!r} {sim.n_primaries} {sim.Ef!r}",
             f"dir {sim.dir[0]!r} {sim.dir[1]!r} {sim.dir[2]!r}",
             f"pos {p[0]!r} {p[1]!r} {p[2]!r}",
             f"size {w[0]!r} {w[1]!r} {w[2]!r}",
             f"bc {sim.bc[0]} {sim.bc[1]} {sim.bc[2]}",
             f"mode {sim.mode}" + (f" {sim.max_generation}" if sim.mode == "primaries" else ""),
             f"primaries_only {int(sim.primaries_only)}",
             f"potential {POTENTIALS[getattr(sim, 'potential', 'universal')]}",
             f"hist_range {sim.hist_range_bin!r} {sim.hist_range_n}",
             f"hist_vac {sim.hist_vac_bin!r} {sim.hist_vac_n}"]
    for l in sim.layers:
        lines.append(f"layer {l.thickness!r} {l.rho!r}")
        for e in l.elements:
            lines.append(f"element {e.Z} {e.m!r} {e.t!r} {e.Edisp!r} {e.Elbind!r}")
    if n is not None or first:
        lines.append(f"subset {first} {n if n is not None else sim.n_primaries - first}")
    if records:
        lines.append(f"records {records}")
    if sim_index:
        lines.append(f"sim {int(sim_index)}")
    if event_mask:
        lines.append(f"events {int(event_mask)}")
    if getattr(sim, "md_tag_Z", 0):
        lines.append(f"mdtag {int(sim.md_tag_Z)} {sim.md_tag_E[0]!r} {sim.md_tag_E[1]!r}")
    if output is not None:
        lines.append(f"output {output[0]} {output[1]}")
    if getattr(sim, "geometry", "layers") == "clusters":
        k = sim.cluster_hash
        lines.append(f"clusters {k[0]} {k[1]} {k[2]}")
        for c in sim.clusters:
            lines.append("cluster " + " ".join(repr(float(v)) for v in c))
    if scale != 1.0:
        lines.append(f"scale {scale!r}")
    if getattr(sim, "surface_binding", 0.0) > 0.0:
        lines.append(f"sputter {sim.surface_binding!r}")
    vn = getattr(sim, "voxel_n", (0, 0, 0))
    if vn[0] > 0:
        o, z = sim.voxel_origin, sim.voxel_size
        lines.append(f"voxels {vn[0]} {vn[1]} {vn[2]} {o[0]!r} {o[1]!r} {o[2]!r} {z[0]!r} {z[1]!r} {z[2]!r}")
    return "\n".join(lines) + "\n"


EVENT_FIELDS = ("kind", "key", "primary", "gen", "Z", "state", "md", "x", "y", "z", "E", "aux", "m")


def parse(text):
    out = {"records": [], "events": []}
    for line in text.splitlines():
        parts = line.split()
        if not parts:
            continue
        k = parts[0]
        if k == "ev":
            vals = [int(v) for v in parts[1:8]] + [float.fromhex(v) for v in parts[8:14]]
            out["events"].append(dict(zip(EVENT_FIELDS, vals)))
        elif k == "rec":
            idx, mem, coll, vac = (int(v) for v in parts[1:5])
            eel, enuc, x, y, z = (float(v) for v in parts[5:10])
            out["records"].append(dict(index=idx, members=mem, collisions=coll, vacancies=vac, eel=eel,
                                       enuc=enuc, x=x, y=y, z=z, state=int(parts[10])))
        elif k.startswith("hist_"):
            out[k] = [int(v) for v in parts[1:]]
        elif k == "vox_depth":
            out[k] = [float(v) for v in parts[1:]]
        elif len(parts) == 2:
            v = parts[1]
            out[k] = float(v) if any(c in v for c in ".en") else int(v)
    return out


def run(sim, seed=1, philox=True, first=0, n=None, records=0, reference=False, timeout=None, scale=1.0,
        sim_index=0, event_mask=0):
    """Run one oracle process on primaries [first, first + n); scale is the
    sample's length unit in Angstrom (SimconfType::setLengthScale); sim_index
    selects the member keys of that simulation of a GPU batch (philox seeding)."""
    exe = REF_DRIVER if reference else MTORACLE
    if not exe.exists():
        raise RuntimeError(f"{exe} is not built")
    args = [str(exe)] if reference else [str(exe), str(TABLES)]
    txt = spec_text(sim, seed=seed, philox=philox, first=first, n=n, records=records, scale=scale,
                    sim_index=sim_index, event_mask=event_mask)
    r = subprocess.run(args, input=txt, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"oracle failed: {r.stderr}")
    return parse(r.stdout)


def write_outputs(sim, output_type, base, seed=1, philox=True, reference=False, cwd=None, timeout=None,
                  scale=1.0):
    """Run one oracle process that writes runmytrim's output file <base>_*.dat in
    `cwd`: the restatement (mtoracle) or, with reference=True, the reference's own
    plugins (oracle/_ref/ref_runmytrim, compat seeding only).  Returns the parsed
    tallies (mtoracle only, else {}) and the stderr text (ref_runmytrim prints
    runmytrim's summary lines there)."""
    if reference:
        args = [str(REF_RUNMYTRIM)]
        exe = REF_RUNMYTRIM
    else:
        args = [str(MTORACLE), str(TABLES)]
        exe = MTORACLE
    if not exe.exists():
        raise RuntimeError(f"{exe} is not built")
    txt = spec_text(sim, seed=seed, philox=philox, output=(output_type, base), scale=scale)
    r = subprocess.run(args, input=txt, capture_output=True, text=True, timeout=timeout, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(f"oracle failed: {r.stderr}")
    return (parse(r.stdout) if not reference else {}), r.stderr


def merge(parts):
    out = {k: 0 for k in SUM_KEYS}
    for p in parts:
        for k in SUM_KEYS:
            out[k] += p.get(k, 0)
    for h in ("hist_range", "hist_vac", "hist_repl", "vox_depth"):
        hs = [p.get(h, []) for p in parts]
        if hs and hs[0] is not None:
            out[h] = [sum(v) for v in zip(*hs)] if hs[0] else []
    out["records"] = sum((p.get("records", []) for p in parts), [])
    out["events"] = sum((p.get("events", []) for p in parts), [])
    out["wall_s"] = max(p.get("wall_s", 0.0) for p in parts) if parts else 0.0
    if parts and "seed_sq" in parts[0]:
        out["seed_sq"] = parts[0]["seed_sq"]  # a property of the whole run, the same in every part
    return out


def run_parallel(sim, seed=1, philox=True, procs=None, reference=False, first=0, n=None, timeout=None,
                 sim_index=0, event_mask=0):
    """Split primaries [first, first + n) over `procs` processes and sum the tallies."""
    total = sim.n_primaries - first if n is None else n
    procs = max(1, min(procs or os.cpu_count() or 1, total))
    bounds = [first + (total * i) // procs for i in range(procs + 1)]
    jobs = [(bounds[i], bounds[i + 1] - bounds[i]) for i in range(procs) if bounds[i + 1] > bounds[i]]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        parts = list(ex.map(lambda j: run(sim, seed=seed, philox=philox, first=j[0], n=j[1],
                                          reference=reference, timeout=timeout, sim_index=sim_index,
                                          event_mask=event_mask), jobs))
    return merge(parts)


def stopping(Z1, m1, layer, energies):
    """Oracle electronic stopping [eV/Angstrom] of (Z1, m1) in `layer` at each energy."""
    # MaterialBase::getrstop = sum_i rstop(Z2_i) t_i * atomic density (material.C:114-121)
    tt = sum(max(e.t, 0.0) for e in layer.elements)
    t = [max(e.t, 0.0) / tt for e in layer.elements]
    am = 0.0
    for e, ti in zip(layer.elements, t):
        am += e.m * ti
    arho = layer.rho * 0.6022 / am
    lines = []
    for E in energies:
        for e in layer.elements:
            lines.append(f"{Z1} {m1!r} {float(E)!r} {e.Z}")
    r = subprocess.run([str(MTORACLE), str(TABLES), "--stopping"], input="\n".join(lines) + "\n",
                       capture_output=True, text=True, check=True)
    vals = [float(v) for v in r.stdout.split()]
    out = []
    k = 0
    for _ in energies:
        se = 0.0
        for ti in t:
            se += vals[k] * ti
            k += 1
        out.append(se * arho)
    return out


def runstopping_reference(Z1, m1, layer, energies):
    """What runstopping prints for the request, computed by the reference library
    (oracle/_ref/ref_runstopping; needs the reference build)."""
    lines = [f"ion {Z1} {m1!r}", f"rho {layer.rho!r}"]
    lines += [f"element {e.Z} {e.m!r} {e.t!r}" for e in layer.elements]
    lines.append("energies " + " ".join(repr(float(E)) for E in energies))
    r = subprocess.run([str(REF_RUNSTOPPING)], input="\n".join(lines) + "\n", capture_output=True, text=True,
                       check=True)
    return r.stdout
