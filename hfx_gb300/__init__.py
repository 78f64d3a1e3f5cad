"""hfx_gb300: GB300-native SEQUEST search engine (Python host mirror).

Thin ctypes layer over libhfx_gpu.so (include/hfx_gpu.h).  The compute runs
in the CUDA library only; this module marshals arguments.  If the shared
library is missing it raises -- there is no CPU fallback.

The reference's host is Haskell: `searchForMatches` (Sequence/Search.hs:98)
over a `SequenceDB` built by `makeSeqDB` (Sequence/Fragment.hs:197) and
configured by `ConfigParams` (Config.hs:55).  `Engine` mirrors that flow:
`build_db` / `upload_db`, `set_mods`, `search`.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhfx_gpu.so")

HFX_OK, HFX_ERR_ARG, HFX_ERR_OOM, HFX_ERR_CUDA, HFX_ERR_TIMEOUT, HFX_ERR_UNSUPPORTED = range(6)

# Correlation.hs:29-30 bin widths (Crux): monoisotopic / average.
BIN_WIDTH_MONO = 1.0005079
BIN_WIDTH_AVG = 1.0011413

EXPORTED = [
    "hfx_default_params", "hfx_ctx_create", "hfx_ctx_destroy", "hfx_set_stream",
    "hfx_last_error", "hfx_build_db", "hfx_upload_db", "hfx_db_info", "hfx_db_export", "hfx_autotune", "hfx_match_peptide",
    "hfx_set_protein_segments", "hfx_match_ions", "hfx_mass_table",
    "hfx_set_mods", "hfx_mod_table", "hfx_search_host", "hfx_search_device", "hfx_search_evalues",
    "hfx_preprocess", "hfx_find_windows", "hfx_ion_bins", "hfx_mod_isoforms", "hfx_digest", "hfx_pack_ions",
    "hfx_set_profiling", "hfx_stage_stats", "hfx_search_counters", "hfx_mod_counters", "hfx_set_workspace_limit",
    "hfx_digest_gpu",
]
STAGES = ["layout", "preprocess", "windows", "score", "topn", "rescore", "mods", "lists", "pack", "mod_lists"]


class HfxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hfx error {code}: {msg}")
        self.code = code


class SearchParams(C.Structure):
    """hfx_search_params (include/hfx_gpu.h)."""
    _fields_ = [
        ("bin_width", C.c_float),
        ("custom_bin_width", C.c_int32),
        ("remove_precursor_peak", C.c_int32),
        ("tol_ppm", C.c_int32),
        ("top_n", C.c_int32),
        ("precision", C.c_int32),
        ("rescore_k", C.c_int32),
        ("batch_mode", C.c_int32),
        ("fastdiv", C.c_int32),
        ("search_plain", C.c_int32),
        ("search_mods", C.c_int32),
        ("group_size", C.c_int32),
        ("chunk", C.c_int32),
        ("max_len", C.c_int32),
        ("ion_bins_custom", C.c_int32),
        ("use_graph", C.c_int32),
    ]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libhfx_gpu.so; raise if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} not built: run `python -m hfx_gb300.build` (CUDA extension required)")
    lib = C.CDLL(path)
    P = C.c_void_p
    i32, u64, f32 = C.c_int32, C.c_uint64, C.c_float
    sig = {
        "hfx_default_params": (None, [C.POINTER(SearchParams)]),
        "hfx_ctx_create": (i32, [i32, C.POINTER(P)]),
        "hfx_ctx_destroy": (i32, [P]),
        "hfx_set_stream": (i32, [P, P]),
        "hfx_last_error": (C.c_char_p, [P]),
        "hfx_build_db": (i32, [P, P, P, i32, P, i32, i32, i32, f32, f32, i32, i32, i32]),
        "hfx_upload_db": (i32, [P, P, u64, P, P, P, u64, P]),
        "hfx_db_info": (i32, [P, C.POINTER(u64), C.POINTER(u64)]),
        "hfx_db_export": (i32, [P, P, P, P, P, P]),
        "hfx_set_mods": (i32, [P, i32, P, P, i32, i32]),
        "hfx_mod_table": (i32, [P, C.POINTER(i32), P, P, i32]),
        "hfx_search_host": (i32, [P, C.POINTER(SearchParams), P, P, P, P, P, P, i32, P, P, P, P]),
        "hfx_search_device": (i32, [P, C.POINTER(SearchParams), P, P, P, P, P, P, i32, P, P, P, P]),
        "hfx_search_evalues": (i32, [P, C.POINTER(SearchParams), P, P, P, P, P, P, i32, i32, C.c_float, P, P, P, P,
                                     P, P]),
        "hfx_match_ions": (i32, [P, C.POINTER(SearchParams), P, i32, P, i32, P, P]),
        "hfx_mass_table": (i32, [i32, P, P]),
        "hfx_autotune": (i32, [P, C.POINTER(SearchParams), P, P, P, P, P, P, i32, P, P, P, P, i32,
                               C.POINTER(C.c_float)]),
        "hfx_match_peptide": (i32, [P, u64, C.c_uint32, C.c_char_p, i32, C.POINTER(C.c_float),
                                    C.POINTER(i32)]),
        "hfx_set_protein_segments": (i32, [P, P, i32]),
        "hfx_preprocess": (i32, [P, C.POINTER(SearchParams), P, P, P, P, P, i32, C.c_int64, P, P, P, P, P]),
        "hfx_find_windows": (i32, [P, C.POINTER(SearchParams), P, P, P, P, P, i32, P, P]),
        "hfx_ion_bins": (i32, [P, P, P, P, i32, i32, i32, P, P, P]),
        "hfx_mod_isoforms": (i32, [P, P, P, P, i32, i32, P, P, P]),
        "hfx_digest": (C.c_int64, [P, P, i32, P, i32, i32, f32, f32, i32, i32, i32, P, P, P, C.c_int64]),
        "hfx_pack_ions": (i32, [P, u64, P, i32, P]),
        "hfx_set_profiling": (i32, [P, i32]),
        "hfx_stage_stats": (i32, [P, P, P, P, i32]),
        "hfx_search_counters": (i32, [P, P, i32]),
        "hfx_mod_counters": (i32, [P, P, i32]),
        "hfx_set_workspace_limit": (i32, [P, u64, C.POINTER(u64)]),
        "hfx_digest_gpu": (C.c_int64, [P, P, P, i32, P, i32, i32, f32, f32, i32, i32, i32, P, P, P, C.c_int64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def default_params(**kw) -> SearchParams:
    lib = load_library()
    p = SearchParams()
    lib.hfx_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    return a.data_ptr()  # torch tensor on the device


def mass_table(mono: bool = True, static_add=None) -> np.ndarray:
    """hfx_mass_table: residue masses A..Z (Config.hs:266-272) plus static
    additions."""
    lib = load_library()
    add = np.zeros(26, np.float32) if static_add is None else np.ascontiguousarray(static_add, np.float32)
    out = np.empty(26, np.float32)
    lib.hfx_mass_table(int(mono), _ptr(add), _ptr(out))
    return out


def digest(seq, seg, mass_table, rule=1, missed=2, min_mass=400.0, max_mass=7200.0, proline_rule=False,
           min_len=0, max_len=0):
    """Host digest of the database build (hfx_digest; Fragment.hs:363-405)."""
    lib = load_library()
    seq = np.ascontiguousarray(seq, np.uint8)
    seg = np.ascontiguousarray(seg, np.uint32)
    mt = np.ascontiguousarray(mass_table, np.float32)
    args = (_ptr(seq), _ptr(seg), len(seg) - 1, _ptr(mt), rule, missed, min_mass, max_mass, int(proline_rule),
            min_len, max_len)
    n = lib.hfx_digest(*args, None, None, None, 0)
    if n < 0:
        raise HfxError(HFX_ERR_ARG, "hfx_digest failed")
    r = np.empty(n, np.float32)
    tc = np.empty(n, np.uint32)
    tn = np.empty(n, np.uint32)
    lib.hfx_digest(*args, _ptr(r), _ptr(tc), _ptr(tn), n)
    return r, tc, tn


def pack_ions(ascii, ma: bytes = b""):
    lib = load_library()
    a = np.ascontiguousarray(ascii, np.uint8)
    out = np.empty_like(a)
    mab = np.frombuffer(ma, np.uint8).copy() if ma else np.zeros(1, np.uint8)
    rc = lib.hfx_pack_ions(_ptr(a), len(a), _ptr(mab), len(ma), _ptr(out))
    if rc != HFX_OK:
        raise HfxError(rc, "hfx_pack_ions failed")
    return out


@dataclass
class SearchResult:
    score: np.ndarray   # [nspec, top_n] raw XCorr (display = /10000)
    key: np.ndarray     # [nspec, top_n] ordering key
    pep: np.ndarray     # [nspec, top_n] fragment index
    ncand: np.ndarray   # [nspec]


class SearchCancelled(RuntimeError):
    """Raised by Engine.search_batches when cancelled between batches;
    `partial` holds the rows of the spectra searched before, `done` their
    count."""

    def __init__(self, partial: "SearchResult", done: int):
        super().__init__(f"search cancelled after {done} spectra")
        self.partial = partial
        self.done = done


def _concat(parts, params) -> "SearchResult":
    tn = (params or default_params()).top_n
    if not parts:
        return SearchResult(np.zeros((0, tn), np.float32), np.zeros((0, tn), np.uint64),
                            np.zeros((0, tn), np.uint32), np.zeros(0, np.int64))
    return SearchResult(*(np.concatenate([getattr(r, f) for r in parts]) for f in ("score", "key", "pep", "ncand")))


class Engine:
    """One CUDA context with a search database (Fragment.hs DeviceSeqDB)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.hfx_ctx_create(device, C.byref(h))
        if rc != HFX_OK:
            raise HfxError(rc, f"hfx_ctx_create(device={device}) failed")
        self.h = h

    def close(self):
        if self.h:
            self.lib.hfx_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != HFX_OK:
            raise HfxError(rc, self.lib.hfx_last_error(self.h).decode())

    def set_profiling(self, on: bool = True):
        self._check(self.lib.hfx_set_profiling(self.h, int(on)))

    def stage_stats(self, reset: bool = True):
        """{stage: (milliseconds, launches, units)} accumulated since the last reset."""
        n = len(STAGES)
        ms = np.zeros(n, np.float64)
        nl = np.zeros(n, np.int64)
        nu = np.zeros(n, np.int64)
        self._check(self.lib.hfx_stage_stats(self.h, _ptr(ms), _ptr(nl), _ptr(nu), int(reset)))
        return {STAGES[i]: (float(ms[i]), int(nl[i]), int(nu[i])) for i in range(n)}

    def counters(self, reset: bool = True):
        """Work counters of the batched list path (see hfx_search_counters)."""
        c = np.zeros(8, np.uint64)
        self._check(self.lib.hfx_search_counters(self.h, _ptr(c), int(reset)))
        names = ["lists", "list_entries", "candidates", "entries_streamed", "pairs", "positions_claimed",
                 "residues_read", "tile_bytes"]
        return {n: int(c[i]) for i, n in enumerate(names)}

    def mod_counters(self, reset: bool = True):
        """Work counters of the modification search over isoform lists (see
        hfx_mod_counters)."""
        c = np.zeros(8, np.uint64)
        self._check(self.lib.hfx_mod_counters(self.h, _ptr(c), int(reset)))
        names = ["lists", "list_entries", "candidates", "entries_streamed", "pairs", "isoforms", "residues_read",
                 "tile_bytes"]
        return {n: int(c[i]) for i, n in enumerate(names)}

    def set_workspace_limit(self, nbytes: int) -> int:
        """hfx_set_workspace_limit: cap the context's workspace bytes (0 = no
        cap); returns the bytes held now.  A search that would need more
        raises HfxError with code HFX_ERR_OOM."""
        used = C.c_uint64()
        self._check(self.lib.hfx_set_workspace_limit(self.h, int(nbytes), C.byref(used)))
        return used.value

    def digest(self, seq, seg, mass_table, rule=1, missed=2, min_mass=400.0, max_mass=7200.0, proline_rule=False,
               min_len=0, max_len=0):
        """hfx_digest_gpu: the database digest on this context's GPU; the same
        (r, tc, tn) as the host `digest`."""
        seq = np.ascontiguousarray(seq, np.uint8)
        seg = np.ascontiguousarray(seg, np.uint32)
        mt = np.ascontiguousarray(mass_table, np.float32)
        args = (_ptr(seq), _ptr(seg), len(seg) - 1, _ptr(mt), rule, missed, min_mass, max_mass, int(proline_rule),
                min_len, max_len)
        n = self.lib.hfx_digest_gpu(self.h, *args, None, None, None, 0)
        if n < 0:
            raise HfxError(HFX_ERR_ARG, self.lib.hfx_last_error(self.h).decode())
        r = np.empty(n, np.float32)
        tc = np.empty(n, np.uint32)
        tn = np.empty(n, np.uint32)
        m = self.lib.hfx_digest_gpu(self.h, *args, _ptr(r), _ptr(tc), _ptr(tn), n)
        if m != n:
            raise HfxError(HFX_ERR_CUDA, self.lib.hfx_last_error(self.h).decode())
        return r, tc, tn

    def search_batches(self, spectra, params: SearchParams | None = None, batch: int = 4096, cancel=None,
                       on_batch=None) -> SearchResult:
        """Search `spectra` in batches of `batch` spectra (one hfx_search_host
        call each, as the reference searches its scans in groups,
        Main.hs:122-151).  `cancel` (a threading.Event or anything with
        is_set()) is checked between batches: once set, no further batch is
        started and SearchCancelled is raised carrying the rows of the batches
        already searched.  on_batch(i, lo, hi) runs after batch i."""
        import numpy as np
        n = len(spectra)
        parts = []
        for i, lo in enumerate(range(0, n, batch)):
            if cancel is not None and cancel.is_set():
                raise SearchCancelled(_concat(parts, params), lo)
            hi = min(n, lo + batch)
            parts.append(self.search(spectra.subset(np.arange(lo, hi)), params))
            if on_batch is not None:
                on_batch(i, lo, hi)
        return _concat(parts, params)

    def set_stream(self, stream_ptr: int):
        self._check(self.lib.hfx_set_stream(self.h, stream_ptr))

    # -- database ---------------------------------------------------------
    def build_db(self, seq: np.ndarray, seg: np.ndarray, static_add=None, mono=True, rule=1,
                 missed=2, min_mass=400.0, max_mass=7200.0, proline_rule=False, min_len=0,
                 max_len=0):
        seq = np.ascontiguousarray(seq, dtype=np.uint8)
        seg = np.ascontiguousarray(seg, dtype=np.uint32)
        add = np.zeros(26, np.float32) if static_add is None else np.ascontiguousarray(static_add, np.float32)
        self._check(self.lib.hfx_build_db(self.h, _ptr(seq), _ptr(seg), len(seg) - 1, _ptr(add), int(mono),
                                          rule, missed, min_mass, max_mass, int(proline_rule), min_len,
                                          max_len))

    def upload_db(self, ions_ascii, r, tc, tn, mass_table):
        ions_ascii = np.ascontiguousarray(ions_ascii, np.uint8)
        r = np.ascontiguousarray(r, np.float32)
        tc = np.ascontiguousarray(tc, np.uint32)
        tn = np.ascontiguousarray(tn, np.uint32)
        mt = np.ascontiguousarray(mass_table, np.float32)
        self._check(self.lib.hfx_upload_db(self.h, _ptr(ions_ascii), len(ions_ascii), _ptr(r), _ptr(tc),
                                           _ptr(tn), len(r), _ptr(mt)))

    def db_info(self):
        a, b = C.c_uint64(), C.c_uint64()
        self._check(self.lib.hfx_db_info(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def db_export(self):
        _, n = self.db_info()
        r = np.empty(n, np.float32)
        tc = np.empty(n, np.uint32)
        tn = np.empty(n, np.uint32)
        idx = np.empty(n, np.uint32)
        mt = np.empty(26, np.float32)
        self._check(self.lib.hfx_db_export(self.h, _ptr(r), _ptr(tc), _ptr(tn), _ptr(idx), _ptr(mt)))
        return r, tc, tn, idx, mt

    def set_mods(self, ma: str, ma_mass, max_ma: int, per_type: bool = False):
        ma_b = np.frombuffer(ma.encode(), np.uint8).copy() if ma else np.zeros(1, np.uint8)
        mm = np.ascontiguousarray(ma_mass if len(ma) else [0.0], np.float32)
        self._check(self.lib.hfx_set_mods(self.h, len(ma), _ptr(ma_b), _ptr(mm), max_ma, int(per_type)))

    def mod_table(self):
        n = C.c_int32()
        self._check(self.lib.hfx_mod_table(self.h, C.byref(n), None, None, 1 << 20))
        counts = np.empty(max(1, n.value * 8), np.int32)
        deltas = np.empty(max(1, n.value), np.float32)
        self._check(self.lib.hfx_mod_table(self.h, C.byref(n), _ptr(counts), _ptr(deltas), 1 << 20))
        return n.value, counts, deltas

    # -- search -----------------------------------------------------------
    def search(self, spectra, params: SearchParams | None = None) -> SearchResult:
        """Host-buffer search (hfx_search_host): copies in and out included."""
        p = params or default_params()
        mz, it, off, pcr, z, tol = spectra.arrays()
        ns = len(pcr)
        tn = p.top_n
        out_s = np.empty((ns, tn), np.float32)
        out_k = np.empty((ns, tn), np.uint64)
        out_p = np.empty((ns, tn), np.uint32)
        out_n = np.empty(ns, np.int64)
        self._check(self.lib.hfx_search_host(self.h, C.byref(p), _ptr(mz), _ptr(it), _ptr(off), _ptr(pcr),
                                             _ptr(z), _ptr(tol), ns, _ptr(out_s), _ptr(out_k), _ptr(out_p),
                                             _ptr(out_n)))
        return SearchResult(out_s, out_k, out_p, out_n)

    def search_device(self, dev, params: SearchParams, out):
        """Device-buffer search (hfx_search_device); dev/out hold torch tensors."""
        self._check(self.lib.hfx_search_device(
            self.h, C.byref(params), _ptr(dev["mz"]), _ptr(dev["it"]), _ptr(dev["off"]), _ptr(dev["pcr"]),
            _ptr(dev["z"]), _ptr(dev["tol"]), int(dev["pcr"].numel()), _ptr(out["score"]), _ptr(out["key"]),
            _ptr(out["pep"]), _ptr(out.get("ncand"))))

    def search_evalues(self, dev, params: SearchParams, out, bin_width: int = 350, cutoff_perc: float = 3.0):
        """hfx_search_evalues: the device-buffer search plus E-values; out
        also holds "ev" [nspec, top_n] and "fit" [nspec, 3] float64 tensors."""
        self._check(self.lib.hfx_search_evalues(
            self.h, C.byref(params), _ptr(dev["mz"]), _ptr(dev["it"]), _ptr(dev["off"]), _ptr(dev["pcr"]),
            _ptr(dev["z"]), _ptr(dev["tol"]), int(dev["pcr"].numel()), int(bin_width), float(cutoff_perc),
            _ptr(out["score"]), _ptr(out["key"]), _ptr(out["pep"]), _ptr(out.get("ncand")), _ptr(out["ev"]),
            _ptr(out["fit"])))

    def match_ions(self, dev, params: SearchParams, out):
        """hfx_match_ions: the "Ions" column (matched, total) of every result
        of the last search on these spectra; out gains "ions_matched" and
        "ions_total" [nspec, top_n] int32 tensors."""
        import torch
        n, k = out["key"].shape
        if "ions_matched" not in out:
            out["ions_matched"] = torch.empty((n, k), dtype=torch.int32, device=out["key"].device)
            out["ions_total"] = torch.empty((n, k), dtype=torch.int32, device=out["key"].device)
        self._check(self.lib.hfx_match_ions(self.h, C.byref(params), _ptr(dev["z"]), n, _ptr(out["key"]), k,
                                            _ptr(out["ions_matched"]), _ptr(out["ions_total"])))
        return out

    def match(self, key: int, pep: int):
        """hfx_match_peptide: (peptide text "X.PEPTIDE.Y" with '*' after
        modified residues, (M+H)+, protein index) of one result entry."""
        buf = C.create_string_buffer(512)
        mh = C.c_float()
        prot = C.c_int32()
        self._check(self.lib.hfx_match_peptide(self.h, int(key), int(pep), buf, 512, C.byref(mh), C.byref(prot)))
        return buf.value.decode(), mh.value, prot.value

    def autotune(self, dev, params: SearchParams, out, reps: int = 2):
        """hfx_autotune: picks group_size and chunk for this batch (in place);
        returns the best milliseconds per search."""
        ms = C.c_float()
        self._check(self.lib.hfx_autotune(
            self.h, C.byref(params), _ptr(dev["mz"]), _ptr(dev["it"]), _ptr(dev["off"]), _ptr(dev["pcr"]),
            _ptr(dev["z"]), _ptr(dev["tol"]), int(dev["pcr"].numel()), _ptr(out["score"]), _ptr(out["key"]),
            _ptr(out["pep"]), _ptr(out.get("ncand")), reps, C.byref(ms)))
        return ms.value

    def preprocess(self, dev, params: SearchParams, stride: int, rows, rows_bf16=None, rows_fp16=None,
                   lens=None, masses=None):
        self._check(self.lib.hfx_preprocess(
            self.h, C.byref(params), _ptr(dev["mz"]), _ptr(dev["it"]), _ptr(dev["off"]), _ptr(dev["pcr"]),
            _ptr(dev["z"]), int(dev["pcr"].numel()), stride, _ptr(rows), _ptr(rows_bf16), _ptr(rows_fp16),
            _ptr(lens), _ptr(masses)))

    def find_windows(self, dev, params: SearchParams, begin, end):
        self._check(self.lib.hfx_find_windows(
            self.h, C.byref(params), _ptr(dev["mz"]), _ptr(dev["off"]), _ptr(dev["pcr"]), _ptr(dev["z"]),
            _ptr(dev["tol"]), int(dev["pcr"].numel()), _ptr(begin), _ptr(end)))

    def ion_bins(self, pos, charges, lens, cap, bins, levels, count, fastdiv=False):
        self._check(self.lib.hfx_ion_bins(self.h, _ptr(pos), _ptr(charges), _ptr(lens), int(pos.numel()), cap,
                                          int(fastdiv), _ptr(bins), _ptr(levels), _ptr(count)))

    def mod_isoforms(self, pos, mod, rank, cap, count, unrank, modded):
        """Stage (e) alone (hfx_mod_isoforms); all arguments are device tensors."""
        self._check(self.lib.hfx_mod_isoforms(self.h, _ptr(pos), _ptr(mod), _ptr(rank), int(pos.numel()), cap,
                                              _ptr(count), _ptr(unrank), _ptr(modded)))
