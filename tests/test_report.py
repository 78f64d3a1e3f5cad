"""The text output of libhfx_gpu.so (include/hfx_report.h) against the
reference's own output files (tests/golden/pretty_tables.json, made by
tests/golden/make_tables.py from the reference's tests/spectra/*.out: their
search header, results table and protein details, an older column set) and
against the formats oracle's restatement of GHC's number printing."""
import json
import os

import numpy as np
import pytest

from hfx_gb300 import report as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pretty_tables.json")


@pytest.fixture(scope="module")
def F():
    import formats as F
    return F


@pytest.fixture(scope="module")
def tables():
    return json.load(open(GOLDEN))


def test_results_layout_pinned(tables):
    """The results block of every output file: the same cells laid out by
    ppAsRows 1 give the same text, trailing blanks included, and the numbers
    print as the file shows them."""
    for name, t in tables.items():
        head = [[" # ", " (M+H)+  ", "deltCn", "XCorr", "Reference", "Peptide"],
                ["---", "---------", "------", "-----", "---------", "-------"]]
        rows = []
        for line in t["results"][2:]:
            tok = line.split()
            rows.append([" " + tok[0]] + tok[1:])
            assert R.format_number(np.float32(tok[1]), 1) == tok[1], name       # (M+H)+, a Float
            assert R.format_number(float(np.float32(tok[3])), 2) == tok[3], name  # XCorr, Float shown as Double
        assert R.format_rows(head + rows, 1) == "\n".join(t["results"]), name


def test_config_layout_pinned(tables):
    for name, t in tables.items():
        rows = [[l[:11].rstrip(), "::", l[15:].rstrip()] for l in t["config"]]
        assert R.format_rows(rows, 0) == "\n".join(t["config"]), name
        mass, _, tol = rows[3][2].split()
        assert R.format_number(np.float32(mass), 0) == mass and R.format_number(np.float32(tol), 0) == tol


def test_detail_layout_pinned(tables):
    """Files whose headers fit in 95 columns; one file predates the 95-column
    paragraph of the current source (PrettyPrint.hs:132) and shows a longer
    header unwrapped, so it cannot pin the wrapping."""
    checked = 0
    for name, t in tables.items():
        headers = [l[5:].rstrip() for l in t["detail"]]
        if max(len(h) for h in headers) + 1 > 95:
            continue
        assert R.format_detail(headers) == "\n".join(t["detail"]) + "\n\n", name
        checked += 1
    assert checked >= 5


def test_whole_file_layout(tables):
    """Blocks are separated by one empty line and the file ends with one."""
    for name, t in tables.items():
        if max(len(l) for l in t["detail"]) > 3 + 2 + 95 + 1:
            continue
        rows = [[l[:11].rstrip(), "::", l[15:].rstrip()] for l in t["config"]]
        text = (R.format_rows(rows, 0) + "\n\n" + R.format_rows(
            [[" # ", " (M+H)+  ", "deltCn", "XCorr", "Reference", "Peptide"],
             ["---", "---------", "------", "-----", "---------", "-------"]] +
            [[" " + l.split()[0]] + l.split()[1:] for l in t["results"][2:]], 1) + "\n\n" +
            R.format_detail([l[5:].rstrip() for l in t["detail"]]))
        assert text == t["text"], name


@pytest.mark.parametrize("seed", range(3))
def test_numbers_match_oracle(F, seed):
    rng = np.random.default_rng(seed)
    xs = np.concatenate([rng.uniform(0, 5, 300), rng.uniform(0, 1, 100) * 10.0 ** rng.integers(-9, 9, 100),
                         np.round(rng.uniform(0, 10, 100), 5), [0.0, 0.5, 0.00005, 0.99995, 9.99995, 1e-300]])
    for x in xs:
        assert R.format_number(x, 0) == F.show_float32(x), x
        assert R.format_number(x, 1) == F.show_ffloat(x, 4, f32=True), x
        assert R.format_number(x, 2) == F.show_ffloat(x, 4), x
        assert R.format_number(x, 3) == F.show_efloat(x, 4), x
        assert R.format_number(-x, 2) == F.show_ffloat(-x, 4), x
    assert R.format_number(float("nan"), 3) == "NaN" and R.format_number(float("inf"), 2) == "Infinity"


def test_results_table_against_oracle(F):
    rng = np.random.default_rng(5)
    ms = []
    for i in range(12):
        ms.append(R.Match(mh=float(rng.uniform(800, 3000)), xcorr=float(np.float32(rng.uniform(0.5, 5.0))),
                          ions=(int(rng.integers(0, 30)), int(rng.integers(10, 40))),
                          reference=b"sp|P%05d|N%d" % (i, i), peptide=b"K.PEPT*IDE%d.R" % i,
                          evalue=float(10.0 ** rng.uniform(-12, 1)), scan=b"scan %d" % i, file=b"run.mgf"))
    ms.sort(key=lambda m: -m.xcorr)
    for all_scans in (False, True):
        got = R.format_results(ms, all_scans)
        s0 = np.float32(ms[0].xcorr)
        rows = [[" # ", " (M+H)+  ", "deltCn", "XCorr", "Ions", "Reference", "Peptide", "E-value"],
                ["---", "---------", "------", "-----", "----", "---------", "-------", "-------"]]
        if all_scans:
            rows[0] += ["Scan details", "File"]
            rows[1] += ["------------", "----"]
        for i, m in enumerate(ms):
            sc = np.float32(m.xcorr)
            r = [f" {i + 1}.", F.show_ffloat(m.mh, 4, f32=True), F.show_ffloat(float(np.float32((s0 - sc) / s0)), 4),
                 F.show_ffloat(float(sc), 4), f"{m.ions[0]}/{m.ions[1]}", m.reference.decode(), m.peptide.decode(),
                 F.show_efloat(m.evalue, 4)]
            rows.append(r + ([m.scan.decode(), m.file.decode()] if all_scans else []))
        assert got == F.pp_as_rows(rows, 1) + "\n\n"


def test_config_and_wrapping(F):
    txt = R.format_config("scan 7", "run.mgf", "db.fasta", "  Trypsin   KR P ", 500.5, 2.0, 3.0)
    lines = txt.split("\n")
    assert lines[0].startswith("Title       :: scan 7") and lines[3].startswith("Enzyme      :: Trypsin KR P")
    f32 = np.float32
    mass = f32(f32(f32(500.5) * f32(2)) - f32(f32(f32(2) * f32(1.007276)) - f32(1)))   # PrettyPrint.hs:95
    assert lines[4] == "(M+H)+ Mass :: " + F.show_float32(mass) + " ~ 3.0 (+2)"
    assert txt.endswith("\n\n")
    long = " ".join(["word%02d" % i for i in range(40)])
    d = R.format_detail([long, "short"]).split("\n")
    assert all(len(l) == len(d[0]) for l in d[:-2]) and d[-2:] == ["", ""]
    assert d[0].startswith(" 1.  word00 ") and d[1].startswith("     word") and len(d[0]) <= 3 + 2 + 95


def test_scan_report_glue(F):
    """scan_report assembles printScanResults from a search result, Ions and
    E-values (the engine's record lookup stood in for by a table)."""
    import types
    from hfx_gb300 import synth

    class Records:
        def match(self, key, pep):
            return (f"K.PEP{pep}TIDE.R", np.float32(1000.5 + pep), pep % 3)

    headers = [b"sp|P0|A protein zero", b"sp|P1|B protein one", b"sp|P2|C protein two"]
    sp = synth.Spectra(np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(3, np.int64),
                       np.array([500.25, 600.5], np.float32), np.array([2.0, 3.0], np.float32),
                       np.array([3.0, 3.0], np.float32), [], [b"scan A", b"scan B"])
    none = np.iinfo(np.uint64).max
    res = types.SimpleNamespace(score=np.array([[52000.0, 31000.0, 0.0], [40000.0, 0.0, 0.0]], np.float32),
                                key=np.array([[7, 9, none], [4, none, none]], np.uint64),
                                pep=np.array([[3, 5, 0], [1, 0, 0]], np.uint32))
    ions = (np.array([[12, 5, 0], [8, 0, 0]], np.int32), np.array([[26, 26, 0], [20, 0, 0]], np.int32))
    ev = np.array([[1.5e-6, 0.25, np.nan], [3e-3, np.nan, np.nan]])
    txt = R.scan_report(Records(), headers, sp, 0, res, ions, ev, "run.mgf", "db.fasta", "Trypsin KR P", tol=3.0)
    blocks = txt.split("\n\n")
    assert len(blocks) == 4 and blocks[-1] == ""
    assert blocks[0].split("\n")[0].startswith("Title       :: scan A")
    rows = [l.split() for l in blocks[1].split("\n")[2:]]
    assert len(rows) == 2
    assert rows[0] == ["1.", F.show_ffloat(1003.5, 4, f32=True), "0.0000", "5.2000", "12/26", "sp|P0|A",
                       "K.PEP3TIDE.R", F.show_efloat(1.5e-6, 4)]
    assert rows[1][2] == F.show_ffloat(float(np.float32((np.float32(5.2) - np.float32(3.1)) / np.float32(5.2))), 4)
    assert rows[1][5] == "sp|P2|C" and rows[1][7] == F.show_efloat(0.25, 4)
    det = blocks[2].split("\n")
    assert det[0].startswith(" 1.  sp|P0|A protein zero") and det[1].startswith(" 2.  sp|P2|C protein two")
