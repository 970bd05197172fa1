"""Extract the reference's published Hunt-duct outputs used to pin the oracle.

Reads the summary CSVs shipped with GridapMHD.jl (analysis/gadi/results/2023_04/)
and writes published_hunt.json.  Run in a checkout that has the reference:

    python tests/golden/make_published.py /path/to/GridapMHD.jl
"""
import csv
import json
import os
import sys

ROWS = [  # (commit folder, experiment, csv line number (1-based, header = 1), why)
    ("eaab9d1460625f2c15ce0fd314528b0a81a3e9ba", "hconv_ha00050ns500", 7, "nc=10, Ha=50"),
    ("eaab9d1460625f2c15ce0fd314528b0a81a3e9ba", "hconv_ha00050ns500", 8, "nc=18, Ha=50"),
    ("eaab9d1460625f2c15ce0fd314528b0a81a3e9ba", "hconv_ha00500ns100", 3, "nc=15, Ha=500"),
    ("eaab9d1460625f2c15ce0fd314528b0a81a3e9ba", "hconv_ha00500ns100", 7, "nc=30, Ha=500"),
    ("daccedff6aad4c0aba4cc48b1cedb5a886a1bde9", "weak_ls16ns200", 2, "nc=32, Ha=50"),
]
KEYS = ["nc", "Ha", "Re", "ncells", "ndofs", "ndofs_u", "ndofs_p", "ndofs_j", "ndofs_φ", "uh_l2", "uh_h1",
        "jh_l2", "eu_ref_l2", "ej_ref_l2", "eu_ref_h1", "nsums", "kmap", "np", "time_solve", "time_jacobian",
        "time_residual"]


def main(ref):
    out = []
    for commit, exp, line, why in ROWS:
        rel = f"analysis/gadi/results/2023_04/{commit}/{exp}/summary.csv"
        with open(os.path.join(ref, rel)) as fh:
            rows = list(csv.DictReader(fh))
        row = rows[line - 2]
        rec = {k: row[k] for k in KEYS if k in row}
        rec["source"] = f"{rel}:{line}"
        rec["case"] = why
        out.append(rec)
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "published_hunt.json"), "w") as fh:
        json.dump(out, fh, indent=1, ensure_ascii=False)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_published.py <path to the GridapMHD.jl checkout>")
    main(sys.argv[1])
