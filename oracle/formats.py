"""Restatement of the reference's file formats (TEST INFRASTRUCTURE ONLY).

Only tests/ import this module.  It is the checker for include/hfx_io.h:
  read_mgf     Spectrum/MGF.hs:48-75 over Util/Parsec.hs:25-85
  read_dta     Spectrum/DTA.hs:35-55
  read_fasta   Sequence/Fasta.hs:27-36 over the bio package's reader (bio 0.5,
               not in the reference tree: blank lines dropped, a record per
               '>' line, sequence lines up to the first not starting with a
               letter)
  index        Sequence/Index.hs:40-82 and the Binary SequenceDB instance
               (Sequence/Fragment.hs:165-172) under the binary 0.5 and
               vector-binary-instances 0.1 encodings (not in the tree):
               Int = big-endian Int64, Word32 big-endian, vectors = length +
               elements, Float = decodeFloat (Integer, Int), Integer = tag 0 +
               Int32 | tag 1 + sign + [Word8] little-endian; the database part
               gzip-compressed (zlib package, Codec.Compression.GZip).
Written independently of the C++ readers: regular expressions and Python's
gzip module.
"""
from __future__ import annotations

import gzip
import math
import re
import struct
from fractions import Fraction

import numpy as np

MASS_H = np.float32(1.007276)   # Mass.hs:25

# readSigned readFloat: optional '-' lexeme, then a decimal number lexeme
_NUM = re.compile(rb"\s*(-)?\s*(\d+(?:\.\d+)?(?:[eE][+-]?\d+)?)")


def _nearest_f32(q: Fraction):
    """The float32 nearest to the rational q (ties to even), as fromRational."""
    c = np.float32(float(q))
    best = c
    for d in (np.nextafter(c, np.float32(-np.inf)), np.nextafter(c, np.float32(np.inf))):
        if not np.isfinite(d):
            continue
        e0, e1 = abs(Fraction(float(best)) - q), abs(Fraction(float(d)) - q)
        if e1 < e0 or (e1 == e0 and (int(d.view(np.uint32)) & 1) == 0):
            best = d
    return best


def read_signed_float(tok: bytes):
    m = _NUM.match(tok)
    if not m:
        raise ValueError(f"no parse: {tok!r}")
    v = _nearest_f32(Fraction(m.group(2).decode()))
    return -v if m.group(1) else v


_PAIR = re.compile(rb"[ \t]*+([0-9.\-]++)[ \t]*+([0-9.\-]++)[\r\n]+")  # Parsec does not backtrack


def _pairs(text: bytes, pos: int):
    """endBy readF2 eol: pairs up to the first line that does not start a
    number; a line that starts one but is not a full pair is an error."""
    out = []
    while True:
        m = _PAIR.match(text, pos)
        if not m:
            if re.match(rb"[ \t0-9.\-]", text[pos:pos + 1]):
                raise ValueError("malformed peak line")
            return out, pos
        out.append((read_signed_float(m.group(1)), read_signed_float(m.group(2))))
        pos = m.end()


_KEYVAL = re.compile(rb"\s*([A-Za-z_][A-Za-z0-9_\-]*)\s*=\s*([^#\n\r][^#\n\r]*)(#[^\n\r]*|[\r\n]+|$)")


def read_mgf(text: bytes):
    """[(title, pepmass, charge, [(mz, it)])]"""
    pos, out = 0, []
    while pos < len(text):
        m = re.compile(rb"BEGIN IONS[\r\n]+").match(text, pos)
        if not m:
            raise ValueError("expecting BEGIN IONS")
        pos = m.end()
        kv = []
        while True:
            m = _KEYVAL.match(text, pos)
            if not m:
                break
            kv.append((m.group(1), m.group(2).rstrip()))
            pos = m.end()
        peaks, pos = _pairs(text, pos)
        m = re.compile(rb"END IONS[\r\n]*").match(text, pos)
        if not m:
            raise ValueError("expecting END IONS")
        pos = m.end()
        get = {}
        for k, v in kv:
            get.setdefault(k, v)
        charge = read_signed_float(get[b"CHARGE"]) if b"CHARGE" in get else np.float32(0)
        pepmass = read_signed_float(get[b"PEPMASS"]) if b"PEPMASS" in get else np.float32(0)
        if charge == 0 or pepmass == 0:
            raise ValueError("missing charge state or peptide mass")
        out.append((get.get(b"TITLE", b""), pepmass, charge, peaks))
    return out


def read_dta(text: bytes):
    """(pcr, charge, [(mz, it)]): pcr = (m + (c - 1) * H) / c in Float."""
    pairs, _ = _pairs(text, 0)
    if not pairs:
        raise ValueError("empty spectrum")
    m, c = pairs[0]
    if math.trunc(float(c)) != float(c):
        raise ValueError("invalid peptide charge state")
    pcr = np.float32(np.float32(m + np.float32(np.float32(c - np.float32(1)) * MASS_H)) / c)
    return pcr, c, pairs[1:]


def read_fasta(data: bytes, gz: bool = False):
    """[(header, sequence)]"""
    if gz:
        data = gzip.decompress(data)
    lines = [l[:-1] if l.endswith(b"\r") else l for l in data.split(b"\n")]
    lines = [l for l in lines if l]
    out = []
    i = 0
    while i < len(lines):
        if not lines[i].startswith(b">"):
            raise ValueError("not a FASTA header")
        head, seq, keep = lines[i][1:], [], True
        i += 1
        while i < len(lines) and not lines[i].startswith(b">"):
            keep = keep and bool(re.match(rb"[A-Za-z]", lines[i]))
            if keep:
                seq.append(lines[i])
            i += 1
        out.append((head, b"".join(seq)))
    return out


# ------------------------------------------------------------------ index

def _int(v):
    return struct.pack(">q", v)


def _bytes(b):
    return _int(len(b)) + b


def _float(x):
    x = float(np.float32(x))
    if x == 0.0:
        m, e = 0, 0
    else:
        f, k = math.frexp(x)
        m, e = int(f * (1 << 24)), k - 24
    return b"\x00" + struct.pack(">i", m) + _int(e)


def index_options(database, missed, rule, min_mass, max_mass, mono, adds):
    """Index.hs:47-57: '\\n' then one `key = value` line each (Haskell show
    of the values); adds: {letter: mass delta} of the static modifications."""
    lines = [f"database         = {database}", f"missed-cleavages = {missed}", f"digestion-rule   = {rule}",
             f"min-peptide-mass = {min_mass!r}", f"max-peptide-mass = {max_mass!r}",
             f"aa-mass-type     = {'Mono' if mono else 'Average'}"]
    lines += [f"add_{k} = {v!r}" for k, v in sorted(adds.items())]
    return "\n" + "".join(l + "\n" for l in lines)


def encode_index(options: str, headers, ions, ion_seg, r, c, n, frag_seg, level=6):
    body = _int(len(headers)) + b"".join(_bytes(h) for h in headers)
    body += _bytes(bytes(np.asarray(ions, np.uint8)))
    body += _int(len(ion_seg)) + b"".join(struct.pack(">I", int(v)) for v in ion_seg)
    body += _int(len(r)) + b"".join(_float(v) for v in r)
    for w in (c, n, frag_seg):
        body += _int(len(w)) + b"".join(struct.pack(">I", int(v)) for v in w)
    return _bytes(options.encode()) + gzip.compress(body, compresslevel=level)


def decode_index(data: bytes):
    (k,) = struct.unpack_from(">q", data, 0)
    options = data[8:8 + k].decode()
    b = gzip.decompress(data[8 + k:])
    pos = 0

    def i64():
        nonlocal pos
        (v,) = struct.unpack_from(">q", b, pos)
        pos += 8
        return v

    def raw(k):
        nonlocal pos
        v = b[pos:pos + k]
        pos += k
        return v

    headers = [raw(i64()) for _ in range(i64())]
    ions = np.frombuffer(raw(i64()), np.uint8).copy()

    def words():
        k = i64()
        return np.array(struct.unpack_from(f">{k}I", raw(4 * k)), np.uint32)

    ion_seg = words()
    r = []
    for _ in range(i64()):
        tag = raw(1)[0]
        if tag == 0:
            (m,) = struct.unpack(">i", raw(4))
        else:
            sign = raw(1)[0]
            mag = int.from_bytes(raw(i64()), "little")
            m = -mag if sign == 255 else mag
        r.append(np.float32(math.ldexp(m, i64())))
    c, n, frag_seg = words(), words(), words()
    return dict(options=options, headers=headers, ions=ions, ion_seg=ion_seg, r=np.array(r, np.float32), c=c, n=n,
                frag_seg=frag_seg)


# ------------------------------------------------------------------ text output
# GHC Numeric (base < 4.6) restated over numpy's Dragon4 shortest digits:
# floatToDigits, roundTo (halves up on the first dropped digit) and the
# formatRealFloat layouts; Util/PrettyPrint.hs:99-211 for the tables.

def float_digits(x, f32):
    if x == 0:
        return [0], 0
    s = np.format_float_scientific(np.float32(x) if f32 else np.float64(x), unique=True, trim="-")
    mant, ex = s.split("e")
    ds = [int(c) for c in mant if c.isdigit()]
    while len(ds) > 1 and ds[-1] == 0:
        ds.pop()
    return ds, int(ex) + 1


def round_to(d, ds):
    c = 1 if d < len(ds) and ds[d] >= 5 else 0
    out = []
    for k in range(d - 1, -1, -1):
        v = (ds[k] if k < len(ds) else 0) + c
        out.append(0 if v == 10 else v)
        c = 1 if v == 10 else 0
    out.reverse()
    return (1, [1] + out) if c else (0, out)


def show_ffloat(x, dec=4, f32=False):
    x = float(np.float32(x)) if f32 else float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "-Infinity" if x < 0 else "Infinity"
    if x < 0 or (x == 0 and math.copysign(1, x) < 0):
        return "-" + show_ffloat(-x, dec, f32)
    ds, e = float_digits(x, f32)
    if e >= 0:
        ei, r = round_to(dec + e, ds)
        s = "".join(map(str, r))
        ls, rs = s[:e + ei] or "0", s[e + ei:]
        return ls + ("." + rs if rs else "")
    ei, r = round_to(dec, [0] * (-e) + ds)
    r = r if ei else [0] + r
    s = "".join(map(str, r))
    return s[0] + ("." + s[1:] if len(s) > 1 else "")


def show_efloat(x, dec=4):
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "-Infinity" if x < 0 else "Infinity"
    if x < 0 or (x == 0 and math.copysign(1, x) < 0):
        return "-" + show_efloat(-x, dec)
    d = max(dec, 1)
    ds, e = float_digits(x, False)
    if ds == [0]:
        return "0." + "0" * d + "e0"
    ei, r = round_to(d + 1, ds)
    if ei:
        r = r[:-1]
    s = "".join(map(str, r))
    return s[0] + "." + s[1:] + "e" + str(e - 1 + ei)


def show_float32(x):
    x = float(np.float32(x))
    if math.isnan(x):
        return "NaN"
    if x < 0 or (x == 0 and math.copysign(1, x) < 0):
        return "-" + show_float32(-x)
    ds, e = float_digits(x, True)
    s = "".join(map(str, ds))
    if e < 0 or e > 7:
        return "0.0e0" if s == "0" else s[0] + "." + (s[1:] or "0") + "e" + str(e - 1)
    if e == 0:
        return "0." + s
    return s[:e].ljust(e, "0") + "." + (s[e:] or "0")


def pp_as_rows(rows, q):
    w = [max(len(r[c]) for r in rows) for c in range(len(rows[0]))]
    return "\n".join(" ".join(cell + " " * (w[c] - len(cell) + q) for c, cell in enumerate(r)) for r in rows)
