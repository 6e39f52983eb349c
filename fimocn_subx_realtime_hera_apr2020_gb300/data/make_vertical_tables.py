"""Regenerate vertical_tables.json from the reference's run-configuration data.

The hybgen target potential temperatures (theta_coor<nvl>.txt) and minimum
layer thicknesses (dpsig<nvl>.txt) are inputs the reference reads at start-up
(FIMsrc/fim/horizontal/dyn_init.F90:789-816).  Each file lists the nvl values
first and alternative choices after a separator line; only the first nvl
numbers are taken.  Usage: python make_vertical_tables.py REF, with REF the
root of the reference tree; the JSON is committed so nothing reads the
reference at run time.
"""
import json
import os
import sys


def first_numbers(path, n):
    vals = []
    with open(path) as fh:
        for line in fh:
            for tok in line.split():
                try:
                    vals.append(float(tok))
                except ValueError:
                    return vals[:n]
                if len(vals) == n:
                    return vals
    return vals[:n]


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: python make_vertical_tables.py REF  (REF: root of the reference tree)")
    REF = sys.argv[1]
    out = {}
    for nvl in (38, 64):
        th = first_numbers(os.path.join(REF, "FIMrun", f"theta_coor{nvl}.txt"), nvl)
        dp = first_numbers(os.path.join(REF, "FIMrun", f"dpsig{nvl}.txt"), nvl)
        assert len(th) == nvl and len(dp) == nvl, (nvl, len(th), len(dp))
        out[str(nvl)] = {"thetac": th, "dpsig": dp,
                         "source": [f"FIMrun/theta_coor{nvl}.txt", f"FIMrun/dpsig{nvl}.txt"]}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "vertical_tables.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
