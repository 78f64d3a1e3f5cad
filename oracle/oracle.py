"""ctypes bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module.  It is the checker: it restates the reference's arithmetic on
the CPU (see hfx_oracle.h for the reference files it follows).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libhfx_oracle.so")
_lib = None


class Params(C.Structure):
    _fields_ = [
        ("bw", C.c_float), ("custom_bw", C.c_int32), ("remove_pcr", C.c_int32), ("ppm", C.c_int32),
        ("topn", C.c_int32), ("prec", C.c_int32), ("num_ma", C.c_int32), ("max_ma", C.c_int32),
        ("per_type", C.c_int32), ("plain", C.c_int32), ("ma", C.c_uint8 * 16), ("ma_mass", C.c_float * 16),
        ("ion_bw", C.c_float),
    ]


def build():
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        i32, i64, f32 = C.c_int32, C.c_int64, C.c_float
        sig = {
            "hfxo_mass_table": (None, [i32, P, P]),
            "hfxo_digest": (i64, [P, P, i32, P, i32, i32, f32, f32, i32, i32, i32, P, P, P, i64]),
            "hfxo_sort_idx": (None, [P, i64, P]),
            "hfxo_pack_ions": (None, [P, i64, P, i32, i32]),
            "hfxo_ms2_mass": (f32, [f32, f32]),
            "hfxo_spec_len": (i32, [P, i32, f32, f32, f32, i32]),
            "hfxo_preprocess": (i32, [P, P, i32, f32, f32, f32, i32, i32, P, P, i32]),
            "hfxo_windows": (None, [P, i64, P, P, i64, P, P]),
            "hfxo_ion_bins": (i32, [P, P, C.c_uint32, C.c_uint32, f32, i32, i32, P, P, P, P, i32]),
            "hfxo_ion_charges": (i32, [f32, i32]),
            "hfxo_score32": (f32, [P, P, i32, P]),
            "hfxo_score64": (C.c_double, [P, P, i32, P]),
            "hfxo_choose": (C.c_uint32, [C.c_uint32, C.c_uint32]),
            "hfxo_unrank_comb": (None, [P, C.c_uint32, C.c_uint32, C.c_uint32]),
            "hfxo_mod_combos": (i32, [i32, i32, P, P, P, P, i32]),
            "hfxo_mod_isoform": (C.c_uint32, [P, C.c_uint32, C.c_uint32, P, i32, P, C.c_uint32, i32, P, P]),
            "hfxo_search": (i32, [P, P, P, P, P, P, i64, P, P, P, P, P, P, i32, C.POINTER(Params), i32,
                                  P, P, P, P, P]),
            "hfxo_match_ions": (None, [P, i32, f32, f32, P, i32, P, f32, i32, P, P]),
            "hfxo_search_scores": (i32, [P, P, P, P, P, P, i64, P, P, P, P, P, P, i32, C.POINTER(Params), i32,
                                         P, P, P, P, P, P, P]),
        }
        for k, (res, args) in sig.items():
            f = getattr(L, k)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def mass_table(mono=True, static_add=None):
    add = np.zeros(26, np.float32) if static_add is None else np.ascontiguousarray(static_add, np.float32)
    out = np.empty(26, np.float32)
    lib().hfxo_mass_table(int(mono), _p(add), _p(out))
    return out


def digest(seq, seg, mt, rule=1, missed=2, min_mass=400.0, max_mass=7200.0, proline_rule=False, min_len=0,
           max_len=0):
    seq = np.ascontiguousarray(seq, np.uint8)
    seg = np.ascontiguousarray(seg, np.uint32)
    cap = int(len(seq) * (missed + 1) + 16)
    r = np.empty(cap, np.float32)
    tc = np.empty(cap, np.uint32)
    tn = np.empty(cap, np.uint32)
    n = lib().hfxo_digest(_p(seq), _p(seg), len(seg) - 1, _p(np.ascontiguousarray(mt, np.float32)), rule, missed,
                          min_mass, max_mass, int(proline_rule), min_len, max_len, _p(r), _p(tc), _p(tn), cap)
    assert n >= 0
    return r[:n].copy(), tc[:n].copy(), tn[:n].copy()


def sort_idx(r):
    r = np.ascontiguousarray(r, np.float32)
    idx = np.empty(len(r), np.uint32)
    lib().hfxo_sort_idx(_p(r), len(r), _p(idx))
    return idx


def pack_ions(seq, ma=b"", quirk=False):
    out = np.array(seq, np.uint8, copy=True)
    mab = np.frombuffer(ma, np.uint8).copy() if ma else np.zeros(1, np.uint8)
    lib().hfxo_pack_ions(_p(out), len(out), _p(mab), len(ma), int(quirk))
    return out


def ms2_mass(pcr, z):
    return lib().hfxo_ms2_mass(float(pcr), float(z))


def preprocess(mz, it, pcr, z, bw=1.0005079, custom_bw=False, remove_pcr=True, fp64=False):
    mz = np.ascontiguousarray(mz, np.float32)
    it = np.ascontiguousarray(it, np.float32)
    L = lib().hfxo_spec_len(_p(mz), len(mz), float(pcr), float(z), float(bw), int(custom_bw))
    if L < 0:
        return None
    o32 = np.empty(L, np.float32)
    o64 = np.empty(L, np.float64) if fp64 else None
    n = lib().hfxo_preprocess(_p(mz), _p(it), len(mz), float(pcr), float(z), float(bw), int(custom_bw),
                              int(remove_pcr), _p(o32), _p(o64), L)
    if n < 0:
        return None
    return (o32, o64) if fp64 else o32


def windows(r_sorted, lo, hi):
    r_sorted = np.ascontiguousarray(r_sorted, np.float32)
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    b = np.empty(len(lo), np.uint32)
    e = np.empty(len(lo), np.uint32)
    lib().hfxo_windows(_p(r_sorted), len(r_sorted), _p(lo), _p(hi), len(lo), _p(b), _p(e))
    return b, e


def ion_charges(z, is_mod=False):
    return lib().hfxo_ion_charges(float(z), int(is_mod))


def ion_bins(ions_packed, mt, tc, tn, residual, charges, length, res_add=None, modded=None, cap=65536):
    bins = np.empty(cap, np.uint32)
    lvl = np.empty(cap, np.uint8)
    n = lib().hfxo_ion_bins(_p(ions_packed), _p(np.ascontiguousarray(mt, np.float32)), int(tc), int(tn),
                            float(residual), int(charges), int(length), _p(res_add), _p(modded), _p(bins),
                            _p(lvl), cap)
    assert n >= 0
    return bins[:n].copy(), lvl[:n].copy()


def score32(bins, lvl, x):
    return lib().hfxo_score32(_p(bins), _p(lvl), len(bins), _p(np.ascontiguousarray(x, np.float32)))


def score64(bins, lvl, x):
    return lib().hfxo_score64(_p(bins), _p(lvl), len(bins), _p(np.ascontiguousarray(x, np.float64)))


def choose(n, k):
    return lib().hfxo_choose(n, k)


def unrank_comb(n, k, rank):
    out = np.zeros(max(k, 1), np.uint32)
    lib().hfxo_unrank_comb(_p(out), n, k, rank)
    return out[:k].copy()


def mod_combos(ma_mass, max_ma):
    ma_mass = np.ascontiguousarray(ma_mass, np.float32)
    cap = 1 << 16
    counts = np.empty(cap * max(1, len(ma_mass)), np.int32)
    sums = np.empty(cap, np.int32)
    deltas = np.empty(cap, np.float32)
    n = lib().hfxo_mod_combos(len(ma_mass), max_ma, _p(ma_mass), _p(counts), _p(sums), _p(deltas), cap)
    return counts[: n * len(ma_mass)].reshape(n, len(ma_mass)).copy(), sums[:n].copy(), deltas[:n].copy()


def mod_isoform(ions_packed, tc, tn, ma, mod_counts, rank=None, per_type=False):
    """(isoform count, unrank row, modified flags) of one (peptide, mod)."""
    mab = np.frombuffer(ma, np.uint8).copy()
    mc = np.ascontiguousarray(mod_counts, np.int32)
    if rank is None:
        n = lib().hfxo_mod_isoform(_p(ions_packed), tc, tn, _p(mab), len(ma), _p(mc), 0xFFFFFFFF, int(per_type),
                                   None, None)
        return n, None, None
    un = np.zeros(64, np.uint32)
    md = np.zeros(max(1, tn - tc), np.uint8)
    n = lib().hfxo_mod_isoform(_p(ions_packed), tc, tn, _p(mab), len(ma), _p(mc), rank, int(per_type), _p(un),
                               _p(md))
    return n, un[: int(mc.sum())].copy(), md[: tn - tc].copy()


def _params(bw, custom_bw, remove_pcr, ppm, topn, prec, ma, ma_mass, max_ma, per_type, plain, ion_bw):
    p = Params()
    p.bw, p.custom_bw, p.remove_pcr, p.ppm = bw, int(custom_bw), int(remove_pcr), int(ppm)
    p.topn, p.prec, p.num_ma, p.max_ma, p.per_type, p.plain = topn, prec, len(ma), max_ma, int(per_type), int(plain)
    p.ion_bw = float(ion_bw)
    for i, c in enumerate(ma):
        p.ma[i] = c
        p.ma_mass[i] = ma_mass[i]
    return p


def search(ions_packed, mt, r, tc, tn, idx, spectra, bw=1.0005079, custom_bw=False, remove_pcr=True, ppm=False,
           topn=10, prec=0, ma=b"", ma_mass=(), max_ma=0, per_type=False, plain=True, nthreads=0, ion_bw=0.0,
           all_scores=False):
    """Full search (Search.hs:98-124); returns (score, score64, key, pep, ncand),
    and with all_scores a sixth item: per spectrum every candidate's score
    (plain, then modified isoforms), the list the E-value fit reads."""
    mz, it, off, pcr, z, tol = spectra.arrays()
    p = _params(bw, custom_bw, remove_pcr, ppm, topn, prec, ma, ma_mass, max_ma, per_type, plain, ion_bw)
    ns = len(pcr)
    sc = np.empty((ns, topn), np.float32)
    s64 = np.empty((ns, topn), np.float64)
    key = np.empty((ns, topn), np.uint64)
    pep = np.empty((ns, topn), np.uint32)
    nc = np.empty(ns, np.int64)
    rc = lib().hfxo_search(_p(ions_packed), _p(np.ascontiguousarray(mt, np.float32)), _p(r), _p(tc), _p(tn),
                           _p(idx), len(r), _p(mz), _p(it), _p(off), _p(pcr), _p(z), _p(tol), ns, C.byref(p),
                           nthreads, _p(sc), _p(s64), _p(key), _p(pep), _p(nc))
    if rc != 0:
        raise RuntimeError(f"oracle search status {rc}")
    if not all_scores:
        return sc, s64, key, pep, nc
    soff = np.zeros(ns + 1, np.int64)
    np.cumsum(nc, out=soff[1:])
    sink = np.empty(max(1, int(soff[-1])), np.float32)
    rc = lib().hfxo_search_scores(_p(ions_packed), _p(np.ascontiguousarray(mt, np.float32)), _p(r), _p(tc),
                                  _p(tn), _p(idx), len(r), _p(mz), _p(it), _p(off), _p(pcr), _p(z), _p(tol), ns,
                                  C.byref(p), nthreads, _p(sc), _p(s64), _p(key), _p(pep), _p(nc), _p(soff),
                                  _p(sink))
    if rc != 0:
        raise RuntimeError(f"oracle search status {rc}")
    return sc, s64, key, pep, nc, [sink[soff[i]:soff[i + 1]].copy() for i in range(ns)]


def match_ions(x, z, pep, mt, mh, nstar=0, bw=1.0005079):
    """The "Ions" column (matched, total) of one match (Match.hs:36-44 over
    IonSeries.hs:87-147); pep: the unmodified peptide's letters (bytes)."""
    x = np.ascontiguousarray(x, np.float32)
    pb = np.frombuffer(bytes(pep), np.uint8).copy()
    m = C.c_int32()
    t = C.c_int32()
    lib().hfxo_match_ions(_p(x), len(x), float(z), float(bw), _p(pb), len(pb),
                          _p(np.ascontiguousarray(mt, np.float32)), float(mh), int(nstar), C.byref(m), C.byref(t))
    return m.value, t.value


def evalue_fit(scores, bin_width=350, cutoff_perc=3.0):
    """Util/Statistics.hs:37-100 for one spectrum's candidate scores (FP32
    raw XCorrs): (alpha, beta, histogram points) of the least-squares line
    log10(count / w) = alpha + beta * (bin centre / 10000) over the ranks
    round(0.3 n) .. round((1 - p/100) n) of the ascending scores shifted by
    1 - min and kept above 4000.  round halves to even; the cut-off product is
    single precision (evalueCutOffPerc is a Float), the 30 % one double.
    linearRegression (statistics-linreg, not in the reference tree) is
    restated as OLS with sequential sums."""
    import math
    sc = np.sort(np.asarray(scores, np.float32)).astype(np.float64)
    n = len(sc)
    if n == 0:
        return float("nan"), float("nan"), 0
    keep = np.float32(np.float32(1.0) - np.float32(np.float32(cutoff_perc) / np.float32(100.0)))
    cut_end = int(np.rint(np.float32(keep * np.float32(n))))
    cut_beg = int(np.rint(0.3 * n))
    hi = min(max(cut_end, 0), n)
    lo = min(max(cut_beg, 0), hi)
    head = float(sc[0])
    w = float(bin_width)
    pts = []
    cur, cnt = None, 0
    for v in sc[lo:hi]:
        t = (float(v) + 1.0) + (-head)
        if not t > 4000.0:
            continue
        b = math.ceil(t / w)
        if b != cur:
            if cnt:
                pts.append(((cur * w - w / 2.0) / 10000.0, math.log(cnt / w) / math.log(10.0)))
            cur, cnt = b, 0
        cnt += 1
    if cnt:
        pts.append(((cur * w - w / 2.0) / 10000.0, math.log(cnt / w) / math.log(10.0)))
    m = float(len(pts))
    if not pts:
        return float("nan"), float("nan"), 0
    sx = sy = 0.0
    for x, y in pts:
        sx += x
        sy += y
    mx, my = sx / m, sy / m
    sxy = sxx = 0.0
    for x, y in pts:
        sxy += (x - mx) * (y - my)
        sxx += (x - mx) * (x - mx)
    beta = sxy / sxx if sxx != 0.0 else float("nan")
    return my - beta * mx, beta, len(pts)


def evalue(alpha, beta, score):
    """E-value of a raw score (Statistics.hs:40): 10 ** (alpha + beta * s / 10000)."""
    import math
    return math.pow(10.0, alpha + beta * (float(score) / 10000.0))

