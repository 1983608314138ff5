"""Regenerate ``stopping_tables.tsv`` from MyTRIM's data directory.

The cascade engine needs, per element Z = 1..92, the SRIM-95 electronic-stopping
fit columns that the reference reads at start-up (simconf.C:82-137,
ScoefLine::read95A simconf.C:150-162 and readSlfctr simconf.C:177-182):

    mm1 (MAI mass number), m1 (MAI weight), mnat, rho, atrho, vfermi, heat,
    pcoef[0..7] (proton stopping coefficients)  -- from SCOEF.95A
    lfctr (screening length factor)               -- from SLFCTR.dat
    symbol                                        -- from ELNAME.dat

SCOEF.95B and SNUC03.dat are read by the reference but never used by its physics,
so they are not carried over.  The values are copied verbatim (as text tokens) so
that the parsed doubles are bit-identical to what the reference parses.

Usage:  python make_stopping_tables.py <mytrim data dir>  > stopping_tables.tsv
"""
import os
import sys
from pathlib import Path

ROWS = 92


def tokens(path, skip_lines):
    text = Path(path).read_text().splitlines()[skip_lines:]
    out = []
    for line in text:
        out.extend(line.split())
    return out


def main(datadir):
    d = Path(datadir)
    a = tokens(d / "SCOEF.95A", 2)
    s = tokens(d / "SLFCTR.dat", 1)
    e = tokens(d / "ELNAME.dat", 0)
    print("# Z\tsym\tmm1\tm1\tmnat\trho\tatrho\tvfermi\theat\tlfctr\t"
          "p0\tp1\tp2\tp3\tp4\tp5\tp6\tp7")
    for i in range(ROWS):
        row = a[16 * i: 16 * (i + 1)]
        assert int(row[0]) == i + 1, row
        z_s, lfctr = s[2 * i], s[2 * i + 1]
        assert int(z_s) == i + 1
        z_e, sym = e[3 * i], e[3 * i + 1]
        assert int(z_e) == i + 1
        cols = [row[0], sym] + row[1:8] + [lfctr] + row[8:16]
        print("\t".join(cols))


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    elif os.environ.get("MYTRIM_REFERENCE"):
        main(os.path.join(os.environ["MYTRIM_REFERENCE"], "data"))
    else:
        sys.exit("usage: make_stopping_tables.py <reference data directory> (or set MYTRIM_REFERENCE)")
