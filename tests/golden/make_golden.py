"""Regenerate the golden fixtures of tests/golden from the reference checkout.

Needs the reference sources ($MYTRIM_REFERENCE, else oracle/Makefile's REF): it
builds the reference library with oracle/Makefile ("make ref"), runs it through
oracle/_ref/ref_driver and copies the reference's own validation data.

  ref_records.json    per-primary results and totals of the reference library on
                      fixed seeds (runmytrim seeding) for four small runs
  vacancy_table.json  the published vacancies/ion table
                      (validation/vacancy_count/vacancy_count_comparison.dat)
  srim_stopping.json  SRIM electronic stopping tables the reference validates against
                      (validation/{h_on_fe,he_on_fe,c_on_w}/srim_stopping.dat)

Usage: python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle_io  # noqa: E402
from golden_cases import CASES  # noqa: E402

REF = oracle_io.reference_dir()
if REF is None:
    sys.exit("the reference checkout is needed: set MYTRIM_REFERENCE")


def main():
    oracle_io.build(REF)
    runs = {}
    for name, (sim, seed, nrec) in CASES.items():
        r = oracle_io.run(sim, seed=seed, philox=False, records=nrec, reference=True)
        r.pop("wall_s", None)
        runs[name] = r
    (HERE / "ref_records.json").write_text(json.dumps(runs, indent=1, sort_keys=True))

    rows = []
    lines = (REF / "validation/vacancy_count/vacancy_count_comparison.dat").read_text().splitlines()
    cols = [c.strip() for c in lines[1].split(",")]
    for line in lines[2:]:
        rows.append([float(v) for v in line.split(",")])
    pairs = ["Si - C"] * 4 + ["Xe - U"] * 4 + ["Cu - Cu"] * 4
    table = {"columns": cols, "pairs": pairs, "rows": rows}
    (HERE / "vacancy_table.json").write_text(json.dumps(table, indent=1))

    srim = {}
    for case, ion, mat in [("h_on_fe", (1, 1.008), (7.8658, [(26, 55.847, 1.0)])),
                           ("he_on_fe", (2, 4.003), (7.8658, [(26, 55.847, 1.0)])),
                           ("c_on_w", (6, 12.0), (19.35, [(74, 183.85, 1.0)]))]:
        data = [[float(v) for v in l.split()] for l in
                (REF / "validation" / case / "srim_stopping.dat").read_text().splitlines() if l.strip()]
        srim[case] = {"Z1": ion[0], "m1": ion[1], "rho": mat[0], "elements": mat[1],
                      "E_eV": [d[0] for d in data], "dEdx_eV_per_A": [d[1] for d in data]}
    (HERE / "srim_stopping.json").write_text(json.dumps(srim, indent=1))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
