"""Input formats on both sides of the search (include/hfx_io.h), served by
libhfx_gpu.so: MGF / DTA spectra (Spectrum.hs readMS2Data), FASTA proteins
(Sequence/Fasta.hs readFasta, plain or .gz) and the digested-database .index
file (Sequence/Index.hs readIndex / writeIndex)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import load_library
from .synth import Spectra

_sigs_set = False


def _lib():
    global _sigs_set
    L = load_library()
    if not _sigs_set:
        P, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        PP = C.POINTER(C.c_void_p)
        sig = {
            "hfx_read_spectra": (i32, [C.c_char_p, PP, C.c_char_p, i32]),
            "hfx_parse_spectra": (i32, [C.c_char_p, i64, i32, PP, C.c_char_p, i32]),
            "hfx_spectra_count": (i64, [P]),
            "hfx_spectra_arrays": (None, [P, PP, PP, PP, PP, PP]),
            "hfx_spectra_title": (P, [P, i64, C.POINTER(i64)]),
            "hfx_spectra_free": (None, [P]),
            "hfx_read_fasta": (i32, [C.c_char_p, PP, C.c_char_p, i32]),
            "hfx_parse_fasta": (i32, [C.c_char_p, i64, i32, PP, C.c_char_p, i32]),
            "hfx_proteins_count": (i64, [P]),
            "hfx_proteins_arrays": (None, [P, PP, PP]),
            "hfx_proteins_header": (P, [P, i64, C.POINTER(i64)]),
            "hfx_proteins_free": (None, [P]),
            "hfx_read_index": (i32, [C.c_char_p, PP, C.c_char_p, i32]),
            "hfx_parse_index": (i32, [C.c_char_p, i64, PP, C.c_char_p, i32]),
            "hfx_index_options": (P, [P, C.POINTER(i64)]),
            "hfx_index_sizes": (None, [P, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]),
            "hfx_index_header": (P, [P, i64, C.POINTER(i64)]),
            "hfx_index_arrays": (None, [P, PP, PP, PP, PP, PP, PP]),
            "hfx_index_free": (None, [P]),
            "hfx_write_index": (i32, [C.c_char_p, C.c_char_p, i64, C.POINTER(C.c_char_p), P, i64, P, P, P, P,
                                      i64, P, C.c_char_p, i32]),
        }
        for k, (res, args) in sig.items():
            f = getattr(L, k)
            f.restype = res
            f.argtypes = args
        _sigs_set = True
    return L


class FormatError(ValueError):
    pass


def _f32(text: str) -> np.float32:
    """A decimal rounded once to the nearest float32 (Haskell read :: Float)."""
    from fractions import Fraction
    q = Fraction(text)
    c = np.float32(float(q))
    best = c
    for d in (np.nextafter(c, np.float32(-np.inf)), np.nextafter(c, np.float32(np.inf))):
        if np.isfinite(d):
            e0, e1 = abs(Fraction(float(best)) - q), abs(Fraction(float(d)) - q)
            if e1 < e0 or (e1 == e0 and (int(d.view(np.uint32)) & 1) == 0):
                best = d
    return best


def _call(fn, *args):
    err = C.create_string_buffer(512)
    h = C.c_void_p()
    rc = fn(*args, C.byref(h), err, 512)
    if rc != 0:
        raise FormatError(err.value.decode(errors="replace"))
    return h


def _array(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dtype))), (n,)).copy()


def _string(ptr, n):
    return C.string_at(ptr, n) if n else b""


def _spectra(h, tol: float) -> Spectra:
    L = _lib()
    try:
        n = L.hfx_spectra_count(h)
        ptrs = [C.c_void_p() for _ in range(5)]
        L.hfx_spectra_arrays(h, *[C.byref(p) for p in ptrs])
        off = _array(ptrs[2], n + 1, np.int64)
        npk = int(off[-1])
        titles = []
        for i in range(n):
            k = C.c_int64()
            t = L.hfx_spectra_title(h, i, C.byref(k))
            titles.append(_string(t, k.value))
        return Spectra(_array(ptrs[0], npk, np.float32), _array(ptrs[1], npk, np.float32), off,
                       _array(ptrs[3], n, np.float32), _array(ptrs[4], n, np.float32),
                       np.full(n, tol, np.float32), [], titles)
    finally:
        L.hfx_spectra_free(h)


def read_spectra(path: str, tol: float = 3.0) -> Spectra:
    """readMS2Data: a .mgf or .dta file; tol is the search tolerance given to
    every spectrum (massTolerance, not part of the file)."""
    L = _lib()
    return _spectra(_call(L.hfx_read_spectra, path.encode()), tol)


def parse_spectra(text: bytes, kind: str, tol: float = 3.0) -> Spectra:
    L = _lib()
    return _spectra(_call(L.hfx_parse_spectra, text, len(text), {"dta": 0, "mgf": 1}[kind]), tol)


@dataclass
class ProteinFile:
    seq: np.ndarray                      # uint8 residues, concatenated (dbIon)
    seg: np.ndarray                      # uint32 [n + 1] offsets (dbIonSeg)
    headers: list = field(default_factory=list)   # dbHeader


def _proteins(h) -> ProteinFile:
    L = _lib()
    try:
        n = L.hfx_proteins_count(h)
        ps, pg = C.c_void_p(), C.c_void_p()
        L.hfx_proteins_arrays(h, C.byref(ps), C.byref(pg))
        seg = _array(pg, n + 1, np.uint32)
        headers = []
        for i in range(n):
            k = C.c_int64()
            t = L.hfx_proteins_header(h, i, C.byref(k))
            headers.append(_string(t, k.value))
        return ProteinFile(_array(ps, int(seg[-1]), np.uint8), seg, headers)
    finally:
        L.hfx_proteins_free(h)


def read_fasta(path: str) -> ProteinFile:
    return _proteins(_call(_lib().hfx_read_fasta, path.encode()))


def parse_fasta(data: bytes, gz: bool = False) -> ProteinFile:
    return _proteins(_call(_lib().hfx_parse_fasta, data, len(data), int(gz)))


@dataclass
class IndexFile:
    options: str
    headers: list
    ions: np.ndarray       # uint8 residues
    ion_seg: np.ndarray    # uint32 [proteins + 1]
    r: np.ndarray          # float32 residual masses
    c: np.ndarray          # uint32 first residue
    n: np.ndarray          # uint32 last residue (one past the protein for its last fragment)
    frag_seg: np.ndarray   # uint32 [proteins + 1]

    def mass_table(self) -> np.ndarray:
        """The residue mass table the options describe, as readIndex's
        readConfig builds it (Index.hs:74-82, Config.hs:197-216, 266-272):
        aa-mass-type and the add_X additions."""
        from . import mass_table
        add = np.zeros(26, np.float32)
        for line in self.options.splitlines():
            k, sep, v = line.partition("=")
            k = k.strip()
            if sep and k.startswith("add_") and len(k) == 5 and "A" <= k[4] <= "Z":
                add[ord(k[4]) - ord("A")] = _f32(v.strip())
        return mass_table(self.option("aa-mass-type", "Mono") != "Average", add)

    def option(self, key: str, default=None):
        """The value of one `key = value` line of the options text."""
        for line in self.options.splitlines():
            k, sep, v = line.partition("=")
            if sep and k.strip() == key:
                return v.strip()
        return default


def _index(h) -> IndexFile:
    L = _lib()
    try:
        k = C.c_int64()
        opt = _string(L.hfx_index_options(h, C.byref(k)), k.value).decode(errors="replace")
        nh, ni, nf = C.c_int64(), C.c_int64(), C.c_int64()
        L.hfx_index_sizes(h, C.byref(nh), C.byref(ni), C.byref(nf))
        headers = []
        for i in range(nh.value):
            t = L.hfx_index_header(h, i, C.byref(k))
            headers.append(_string(t, k.value))
        ptrs = [C.c_void_p() for _ in range(6)]
        L.hfx_index_arrays(h, *[C.byref(p) for p in ptrs])
        nf, nh, ni = nf.value, nh.value, ni.value
        return IndexFile(opt, headers, _array(ptrs[0], ni, np.uint8), _array(ptrs[1], nh + 1, np.uint32),
                         _array(ptrs[2], nf, np.float32), _array(ptrs[3], nf, np.uint32),
                         _array(ptrs[4], nf, np.uint32), _array(ptrs[5], nh + 1, np.uint32))
    finally:
        L.hfx_index_free(h)


def read_index(path: str) -> IndexFile:
    return _index(_call(_lib().hfx_read_index, path.encode()))


def parse_index(data: bytes) -> IndexFile:
    return _index(_call(_lib().hfx_parse_index, data, len(data)))


def write_index(path: str, x: IndexFile) -> None:
    L = _lib()
    hs = (C.c_char_p * max(1, len(x.headers)))(*x.headers)
    arrs = [np.ascontiguousarray(a, t) for a, t in ((x.ions, np.uint8), (x.ion_seg, np.uint32),
                                                    (x.r, np.float32), (x.c, np.uint32), (x.n, np.uint32),
                                                    (x.frag_seg, np.uint32))]
    err = C.create_string_buffer(512)
    rc = L.hfx_write_index(path.encode(), x.options.encode(), len(x.headers), hs, arrs[0].ctypes.data,
                           len(arrs[0]), arrs[1].ctypes.data, arrs[2].ctypes.data, arrs[3].ctypes.data,
                           arrs[4].ctypes.data, len(arrs[2]), arrs[5].ctypes.data, err, 512)
    if rc != 0:
        raise FormatError(err.value.decode(errors="replace"))
