"""The reference's text output (include/hfx_report.h; Util/PrettyPrint.hs),
served by libhfx_gpu.so: the search header, the results tables (per scan and
over all scans) and the protein details."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import load_library


class ResultRow(C.Structure):
    _fields_ = [("mh", C.c_float), ("xcorr", C.c_float), ("ions_matched", C.c_int32), ("ions_total", C.c_int32),
                ("reference", C.c_char_p), ("peptide", C.c_char_p), ("evalue", C.c_double),
                ("scan", C.c_char_p), ("file", C.c_char_p)]


_sigs_set = False


def _lib():
    global _sigs_set
    L = load_library()
    if not _sigs_set:
        i32, i64 = C.c_int32, C.c_int64
        sig = {
            "hfx_format_results": (i64, [C.POINTER(ResultRow), i32, i32, C.c_char_p, i64]),
            "hfx_format_config": (i64, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_float, C.c_float,
                                        C.c_float, C.c_char_p, i64]),
            "hfx_format_detail": (i64, [C.POINTER(C.c_char_p), i32, C.c_char_p, i64]),
            "hfx_format_rows": (i64, [C.POINTER(C.c_char_p), i32, i32, i32, C.c_char_p, i64]),
            "hfx_format_number": (i64, [C.c_double, i32, C.c_char_p, i64]),
        }
        for k, (res, args) in sig.items():
            f = getattr(L, k)
            f.restype = res
            f.argtypes = args
        _sigs_set = True
    return L


def _text(fn, *args) -> str:
    n = fn(*args, None, 0)
    if n < 0:
        raise ValueError("bad arguments")
    buf = C.create_string_buffer(n + 1)
    fn(*args, buf, n + 1)
    return buf.raw[:n].decode(errors="replace")


def _b(s):
    return s if isinstance(s, bytes) else str(s).encode()


@dataclass
class Match:
    mh: float
    xcorr: float
    ions: tuple
    reference: bytes
    peptide: bytes
    evalue: float
    scan: bytes = b""
    file: bytes = b""


def format_results(matches, all_scans: bool = False) -> str:
    """printResults (all_scans: printAllResults) of matches in order."""
    rows = (ResultRow * max(1, len(matches)))()
    keep = []
    for i, m in enumerate(matches):
        keep += [_b(m.reference), _b(m.peptide), _b(m.scan), _b(m.file)]
        rows[i] = ResultRow(m.mh, m.xcorr, int(m.ions[0]), int(m.ions[1]), keep[-4], keep[-3], float(m.evalue),
                            keep[-2], keep[-1])
    return _text(_lib().hfx_format_results, rows, len(matches), int(all_scans))


def format_config(title, spectrum, database, enzyme, pcr, charge, tol) -> str:
    """printConfig: the header block of one spectrum's results."""
    return _text(_lib().hfx_format_config, _b(title), _b(spectrum), _b(database), _b(enzyme), float(pcr),
                 float(charge), float(tol))


def format_detail(headers) -> str:
    """printResultsDetail: the protein headers of the first matches."""
    hs = (C.c_char_p * max(1, len(headers)))(*[_b(h) for h in headers])
    return _text(_lib().hfx_format_detail, hs, len(headers))


def format_rows(cells, q: int) -> str:
    """ppAsRows q over a list of rows of strings (all rows the same length)."""
    nr, nc = len(cells), len(cells[0]) if cells else 0
    flat = (C.c_char_p * max(1, nr * nc))(*[_b(c) for r in cells for c in r])
    return _text(_lib().hfx_format_rows, flat, nr, nc, q)


def format_number(x: float, kind: int) -> str:
    """0 show (Float), 1 showFFloat (Just 4) Float, 2 the same of a Double,
    3 showEFloat (Just 4) Double."""
    return _text(_lib().hfx_format_number, float(x), int(kind))


def scan_report(eng, headers, spectra, i: int, result, ions=None, evalues=None, spectrum_file: str = "",
                database: str = "", enzyme: str = "", tol: float = 3.0, num_matches: int = 5,
                num_detail: int = 3) -> str:
    """printScanResults (PrettyPrint.hs:148-160) of spectrum i: the header,
    the first num_matches results and the protein details of the first
    num_detail.  result: a SearchResult (score, key, pep); ions: (matched,
    total) arrays [nspec, top_n] from Engine.match_ions; evalues [nspec,
    top_n] from Engine.search_evalues; headers: the database's protein
    headers (FASTA or index); the XCorr shown is score / 10000
    (Search.hs:121-122)."""
    none = (1 << 64) - 1
    ms, det = [], []
    for j in range(result.key.shape[1]):
        key = int(result.key[i, j])
        if key == none:
            break
        text, mh, prot = eng.match(key, int(result.pep[i, j]))
        h = headers[prot] if 0 <= prot < len(headers) else b""
        ms.append(Match(mh=mh, xcorr=float(C.c_float(float(result.score[i, j]) / 10000.0).value),
                        ions=(int(ions[0][i, j]), int(ions[1][i, j])) if ions is not None else (0, 0),
                        reference=(h.split() or [b""])[0], peptide=text.encode(),
                        evalue=float(evalues[i, j]) if evalues is not None else float("nan")))
        det.append(h)
    title = spectra.title[i] if getattr(spectra, "title", None) else b""
    return (format_config(title, spectrum_file, database, enzyme, spectra.pcr[i], spectra.z[i], tol) +
            format_results(ms[:num_matches]) + format_detail(det[:num_detail]))
