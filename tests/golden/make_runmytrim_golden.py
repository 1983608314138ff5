"""Regenerate the runmytrim fixtures of tests/golden/runmytrim from the reference.

Each case is a runmytrim input (JSON, written here or read from the reference's
tests/json with fewer ions) and the output file the
reference's own plugin wrote for it: TrimVacCount (_vac.dat), TrimVacEnergyCount
(_evac.dat) or TrimRange (_ranges.dat), compiled from the reference sources
with oracle/Makefile ("make ref") and driven by oracle/_ref/ref_runmytrim with
runmytrim's seeding (master seed -> 16-bit per-primary mt19937 seeds).  The
summary lines runmytrim prints on stderr are kept in <case>.summary.

Needs the reference checkout ($MYTRIM_REFERENCE, else oracle/Makefile's REF).

Usage: python tests/golden/make_runmytrim_golden.py
"""
import json
import re
import shutil
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "runmytrim"
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle_io  # noqa: E402
from mytrim_gb300 import runmytrim  # noqa: E402

REF = oracle_io.reference_dir()
if REF is None:
    sys.exit("the reference checkout is needed: set MYTRIM_REFERENCE")


def doc(ion, layers, otype, seed, extra_opts=None, extra_out=None):
    opts = {"seed": seed, "threads": 4}
    opts.update(extra_opts or {})
    out = {"base": None, "type": otype}
    out.update(extra_out or {})
    return {"mytrim": {"options": opts, "ion": ion, "sample": {"layers": layers}, "output": out}}


def elem(Z, mass, fraction, **kw):
    d = {"Z": Z, "mass": mass, "fraction": fraction}
    d.update(kw)
    return d


# name -> (input document, optional text transform)
CASES = {
    # the reference's validation runs (validation/vacancy_count), 1 keV, fewer ions
    "cu_on_cu_vac": doc({"Z": 29, "mass": 63.546, "energy": 1000, "number": 2000},
                        [{"thickness": 100000, "rho": 8.92, "elements": [elem(29, 63.546, 1)]}], "vaccount", 2344),
    "si_on_c_evac": doc({"Z": 14, "mass": 27.977, "energy": 1000, "number": 1000},
                        [{"thickness": 100000, "rho": 2.253, "elements": [elem(6, 12.01, 1)]}], "vacenergycount",
                        2344),
    "xe_on_u_range": doc({"Z": 54, "mass": 131.904, "energy": 1000, "number": 1000},
                         [{"thickness": 100000, "rho": 19.043, "elements": [elem(92, 238.0, 1)]}], "range", 2344),
    # two layers; edisp / elbind given on the first element only (later elements
    # inherit them), final energy, length scale 10 (nm units)
    "ar_sio2_si_vac": doc({"Z": 18, "mass": 39.948, "energy": 10000, "number": 150, "final_energy": 5},
                          [{"thickness": 10, "rho": 2.2,
                            "elements": [elem(14, 28.086, 1, edisp=15, elbind=2), elem(8, 15.999, 2)]},
                           {"thickness": 10000, "rho": 2.33, "elements": [elem(14, 28.086, 1)]}],
                          "vaccount", 77, extra_opts={"scale": 10}),
    "cu_on_cu_range_10k": doc({"Z": 29, "mass": 63.546, "energy": 10000, "number": 300},
                              [{"thickness": 100000, "rho": 8.96, "elements": [elem(29, 63.546, 1)]}], "range", 5),
    "he_fe_primaries_only": doc({"Z": 2, "mass": 4.0026, "energy": 5000, "number": 400},
                                [{"thickness": 100000, "rho": 7.8658, "elements": [elem(26, 55.847, 1)]}],
                                "vaccount", 9, extra_out={"primaries_only": True}),
    "au_on_si_evac": doc({"Z": 79, "mass": 196.967, "energy": 20000, "number": 40},
                         [{"thickness": 100000, "rho": 2.33, "elements": [elem(14, 28.086, 1, edisp=15)]}],
                         "vacenergycount", 31),
}


# the reference's own runmytrim tests (tests/json: 150 keV Cu on a Cu film, 10 MeV Xe
# into UO2 at length scale 1 and 10), read from the reference checkout with their
# comments kept, renamed json_<name> and run with a tenth of the ions
JSON_TESTS = {"cu_on_cu": 100, "xe_on_uo2": 10, "xe_on_uo2_scale10": 10}


def reference_json_cases():
    out = {}
    for stem, number in JSON_TESTS.items():
        text = (REF / "tests" / "json" / f"{stem}.json").read_text()
        text, n_base = re.subn(r'("base"\s*:\s*")' + stem + '"', r'\g<1>json_' + stem + '"', text)
        text, n_num = re.subn(r'("number"\s*:\s*)\d+', r'\g<1>' + str(number), text)
        assert n_base == 1 and n_num == 1, stem
        out[f"json_{stem}"] = text
    return out


def render(name, d):
    d = json.loads(json.dumps(d))
    d["mytrim"]["output"]["base"] = name
    text = json.dumps(d, indent=2)
    if name == "ar_sio2_si_vac":
        # jsoncpp syntax runmytrim accepts: comments and a trailing comma
        text = "// two-layer target\n" + text.replace('"sample": {', '"sample": { /* SiO2 on Si */', 1)
        text = text.replace('"scale": 10\n', '"scale": 10,\n', 1)
    return text + "\n"


def main():
    oracle_io.build(REF)
    OUT.mkdir(exist_ok=True)
    texts = {name: render(name, d) for name, d in CASES.items()}
    texts.update(reference_json_cases())
    for name, text in texts.items():
        (OUT / f"{name}.json").write_text(text)
        inp = runmytrim.load(text)
        with tempfile.TemporaryDirectory() as tmp:
            _, err = oracle_io.write_outputs(inp.sim, inp.output_type, inp.base, seed=inp.seed, philox=False,
                                          reference=True, cwd=tmp, scale=inp.scale)
            shutil.copy(Path(tmp) / inp.output_file, OUT / inp.output_file)
        (OUT / f"{name}.summary").write_text(err)
        print(name, inp.output_file, (OUT / inp.output_file).stat().st_size, err.strip().replace("\n", " | "))


if __name__ == "__main__":
    main()
