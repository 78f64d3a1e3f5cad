"""Writes pretty_tables.json: the text blocks of the reference's own output
files (tests/spectra/*.out: the search header, the results table and the
header details), which pin the table layout of include/hfx_report.h.
Run with the reference checkout as the argument or in HFX_REFERENCE."""
import glob
import json
import os
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HFX_REFERENCE", "")
if not REF:
    sys.exit("usage: make_tables.py <reference checkout> (or set HFX_REFERENCE)")
out = {}
for path in sorted(glob.glob(os.path.join(REF, "tests", "spectra", "*.out"))):
    lines = open(path).read().split("\n")
    blocks, cur = [], []
    for l in lines:
        if l == "":
            if cur:
                blocks.append(cur)
            cur = []
        else:
            cur.append(l)
    if cur:
        blocks.append(cur)
    out[os.path.basename(path)] = {"config": blocks[0], "results": blocks[1], "detail": blocks[2],
                                   "text": "\n".join(lines)}
json.dump(out, open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "pretty_tables.json"), "w"),
          indent=1)
print(len(out), "files")
