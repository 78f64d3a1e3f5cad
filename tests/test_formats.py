"""The file readers of libhfx_gpu.so (include/hfx_io.h: MGF, DTA, FASTA and
.gz, the .index database) against the formats oracle (oracle/formats.py),
on seeded files with the grammar's corners, and the index both ways
(deflate-compressed by Python's gzip, stored blocks written here)."""
import gzip

import numpy as np
import pytest

from hfx_gb300 import io as hio
from hfx_gb300 import synth


@pytest.fixture(scope="module")
def F():
    import formats as F
    return F


def _fmt(rng, v):
    return [f"{v:.4f}", f"{v:.1f}", f"{v:.6f}", f"{int(v)}"][int(rng.integers(0, 4))]


def _mgf(rng, nspec):
    out = []
    for s in range(nspec):
        eol = "\r\n" if rng.random() < 0.3 else "\n"
        params = [f"TITLE=scan {s} file.raw  ", f"CHARGE={int(rng.integers(1, 5))}{'+' if rng.random() < 0.7 else ''}",
                  f"PEPMASS={_fmt(rng, rng.uniform(300, 1500))}" + (f" {rng.uniform(1e3, 1e6):.1f}"
                                                                       if rng.random() < 0.5 else ""),
                  f"RTINSECONDS = {rng.uniform(0, 3000):.2f}"]
        rng.shuffle(params)
        # a comment leaves its line end to the next parameter, so it may not
        # end the last one (see test_mgf_errors)
        lines = ["BEGIN IONS", "SCANS=12 # a comment"] + params
        for _ in range(int(rng.integers(0, 60))):
            sep = [" ", "\t", "   "][int(rng.integers(0, 3))]
            lead = " " if rng.random() < 0.1 else ""
            lines.append(f"{lead}{_fmt(rng, rng.uniform(50, 2000))}{sep}{_fmt(rng, rng.uniform(0, 1e5))}")
        lines.append("END IONS")
        out.append(eol.join(lines) + eol + ("\n" if rng.random() < 0.3 else ""))
    return "".join(out).encode()


@pytest.mark.parametrize("seed", range(5))
def test_mgf_matches_oracle(F, seed):
    rng = np.random.default_rng(seed)
    text = _mgf(rng, 40)
    got = hio.parse_spectra(text, "mgf")
    ref = F.read_mgf(text)
    assert len(got) == len(ref) == 40
    for i, (title, pepmass, charge, peaks) in enumerate(ref):
        a, b = got.off[i], got.off[i + 1]
        assert got.title[i] == title
        assert got.pcr[i].view(np.uint32) == np.float32(pepmass).view(np.uint32)
        assert got.z[i] == charge
        mz = np.array([p[0] for p in peaks], np.float32)
        it = np.array([p[1] for p in peaks], np.float32)
        assert np.array_equal(got.mz[a:b].view(np.uint32), mz.view(np.uint32))
        assert np.array_equal(got.it[a:b].view(np.uint32), it.view(np.uint32))


@pytest.mark.parametrize("text", [
    b"BEGIN IONS\nTITLE=x\nPEPMASS=500\n100 2\nEND IONS\n",            # no charge
    b"BEGIN IONS\nCHARGE=2+\nPEPMASS=0\nEND IONS\n",                    # zero mass
    b"BEGIN IONS\nCHARGE=2+\nPEPMASS=500\n100 2\n",                     # no END IONS
    b"BEGIN IONS\nCHARGE=2+\nPEPMASS=500\n100 2 \nEND IONS\n",          # trailing blank on a peak line
    b"BEGIN IONS\nCHARGE=2+\nPEPMASS=500\n100 2 3\nEND IONS\n",         # three columns
    b"BEGIN IONS\nCHARGE=2+\nPEPMASS=500\n100\nEND IONS\n",             # one column
    b"\nBEGIN IONS\nCHARGE=2+\nPEPMASS=500\nEND IONS\n",                # text before BEGIN IONS
    b"BEGIN IONS\nCHARGE=+2\nPEPMASS=500\nEND IONS\n",                  # '+' before the number
    b"BEGIN IONS\nCHARGE=2\nPEPMASS=500\n10020\nEND IONS\n",            # tokens run together
    b"BEGIN IONS\nCHARGE=2\nPEPMASS=500 # c\n100 2\nEND IONS\n",       # comment on the last parameter
    b"BEGIN IONS\nCHARGE=2\nPEPMASS=500\n1e3 5\nEND IONS\n",            # no exponents in peak values
])
def test_mgf_errors(F, text):
    with pytest.raises(ValueError):
        F.read_mgf(text)
    with pytest.raises(hio.FormatError):
        hio.parse_spectra(text, "mgf")


def test_mgf_values(F):
    text = (b"BEGIN IONS\r\nTITLE = a title  # note\r\nCHARGE=3+ and 4+\r\nPEPMASS=5.0e2 77\r\n"
            b"\t100.25\t-2\r\n1-3 5\r\n100.5.7 2-3\r\nEND IONS")
    got = hio.parse_spectra(text, "mgf")
    assert got.title == [b"a title"] and got.z[0] == 3.0 and got.pcr[0] == 500.0
    assert got.mz.tolist() == [100.25, 1.0, 100.5] and got.it.tolist() == [-2.0, 5.0, 2.0]
    (t, pm, ch, peaks), = F.read_mgf(text)
    assert (t, float(pm), float(ch)) == (b"a title", 500.0, 3.0)
    assert [(float(a), float(b)) for a, b in peaks] == [(100.25, -2.0), (1.0, 5.0), (100.5, 2.0)]


@pytest.mark.parametrize("seed", range(4))
def test_dta_matches_oracle(F, seed):
    rng = np.random.default_rng(seed)
    lines = [f"{rng.uniform(800, 3000):.4f} {int(rng.integers(1, 5))}"]
    lines += [f"{_fmt(rng, rng.uniform(50, 2000))} {_fmt(rng, rng.uniform(0, 1e4))}" for _ in range(80)]
    text = ("\n".join(lines) + "\n").encode()
    got = hio.parse_spectra(text, "dta")
    pcr, c, peaks = F.read_dta(text)
    assert got.pcr[0].view(np.uint32) == pcr.view(np.uint32) and got.z[0] == c
    assert np.array_equal(got.mz, np.array([p[0] for p in peaks], np.float32))
    assert np.array_equal(got.it, np.array([p[1] for p in peaks], np.float32))
    assert got.title == [b""]


def test_dta_errors_and_trailing_text(F):
    for bad in (b"", b"1500.2 2.5\n100 1\n", b"abc\n"):
        with pytest.raises(ValueError):
            F.read_dta(bad)
        with pytest.raises(hio.FormatError):
            hio.parse_spectra(bad, "dta")
    # the reference's parser stops at the first line that is no pair
    got = hio.parse_spectra(b"1500.2 2\n100 1\nEND\n200 3\n", "dta")
    assert got.mz.tolist() == [100.0] and F.read_dta(b"1500.2 2\n100 1\nEND\n200 3\n")[2] == [(100.0, 1.0)]


def _fasta(rng, n):
    prot = synth.proteins(n, seed=int(rng.integers(0, 1 << 30)))
    out = []
    for i in range(n):
        s = bytes(prot.seq[prot.seg[i]:prot.seg[i + 1]])
        eol = b"\r\n" if rng.random() < 0.2 else b"\n"
        out.append(b">sp|P%05d|NAME_%d Protein %d OS=Homo sapiens" % (i, i, i) + eol)
        w = int(rng.integers(40, 81))
        out += [s[k:k + w] + eol for k in range(0, len(s), w)]
        if rng.random() < 0.2:
            out.append(eol)
        if rng.random() < 0.1:
            out.append(b"*" + eol + b"IGNORED" + eol)   # a non-letter line ends the sequence
    return b"".join(out), prot


@pytest.mark.parametrize("gz", [False, True])
def test_fasta_matches_oracle(F, gz):
    rng = np.random.default_rng(7)
    data, prot = _fasta(rng, 300)
    if gz:
        data = gzip.compress(data, compresslevel=int(rng.integers(1, 10)))
    got = hio.parse_fasta(data, gz=gz)
    ref = F.read_fasta(data, gz=gz)
    assert got.headers == [h for h, _ in ref]
    assert got.seq.tobytes() == b"".join(s for _, s in ref)
    lens = np.array([len(s) for _, s in ref], np.int64)
    assert np.array_equal(got.seg, np.concatenate([[0], np.cumsum(lens)]).astype(np.uint32))
    assert got.seq.tobytes() == prot.seq.tobytes()


def test_fasta_file_and_gzip_errors(F, tmp_path):
    data, prot = _fasta(np.random.default_rng(3), 50)
    (tmp_path / "db.fasta").write_bytes(data)
    (tmp_path / "db.fasta.gz").write_bytes(gzip.compress(data))
    a = hio.read_fasta(str(tmp_path / "db.fasta"))
    b = hio.read_fasta(str(tmp_path / "db.fasta.gz"))
    assert a.seq.tobytes() == b.seq.tobytes() == prot.seq.tobytes() and a.headers == b.headers
    z = bytearray(gzip.compress(data))
    z[-8] ^= 1                                    # CRC
    with pytest.raises(hio.FormatError):
        hio.parse_fasta(bytes(z), gz=True)
    with pytest.raises(hio.FormatError):
        hio.parse_fasta(bytes(z[: len(z) // 2]), gz=True)
    with pytest.raises(hio.FormatError):
        hio.parse_fasta(b"ACDE\n>x\nK\n")            # no header first


def _digested(oracle, n=400):
    prot = synth.proteins(n, seed=11)
    mt = oracle.mass_table(True, synth.static_mods())
    dg = {k: v for k, v in synth.DIGEST.items() if k != "mono"}
    r, tc, tn = oracle.digest(prot.seq, prot.seg, mt, **dg)
    # fragments per protein (fragment segments, Fragment.hs:219-228)
    fs = np.searchsorted(tc, prot.seg[:-1], side="left").astype(np.uint32)
    fs = np.concatenate([fs, [len(r)]]).astype(np.uint32)
    headers = [b"sp|P%05d|N%d Protein %d" % (i, i, i) for i in range(n)]
    return prot, headers, r, tc, tn, fs


@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_index_read_matches_oracle(F, oracle, level):
    prot, headers, r, tc, tn, fs = _digested(oracle)
    opts = F.index_options("db.fasta", 1, 1, 400.0, 7200.0, True, {"C": 57.021})
    data = F.encode_index(opts, headers, prot.seq, prot.seg, r, tc, tn, fs, level=level)
    x = hio.parse_index(data)
    assert x.options == opts and x.headers == headers
    assert x.ions.tobytes() == prot.seq.tobytes() and np.array_equal(x.ion_seg, prot.seg)
    assert np.array_equal(x.r.view(np.uint32), r.view(np.uint32))
    assert np.array_equal(x.c, tc) and np.array_equal(x.n, tn) and np.array_equal(x.frag_seg, fs)
    assert x.option("aa-mass-type") == "Mono" and x.option("add_C") == "57.021"


def test_index_write_round_trip(F, oracle, tmp_path):
    prot, headers, r, tc, tn, fs = _digested(oracle, 150)
    opts = F.index_options("db.fasta", 2, 1, 400.0, 7200.0, False, {})
    x = hio.IndexFile(opts, headers, prot.seq, prot.seg, r, tc, tn, fs)
    path = str(tmp_path / "db.index")
    hio.write_index(path, x)
    ref = F.decode_index(open(path, "rb").read())
    assert ref["options"] == opts and ref["headers"] == headers
    assert np.array_equal(ref["r"].view(np.uint32), r.view(np.uint32))
    assert np.array_equal(ref["c"], tc) and np.array_equal(ref["n"], tn) and np.array_equal(ref["frag_seg"], fs)
    y = hio.read_index(path)
    assert np.array_equal(y.r.view(np.uint32), r.view(np.uint32)) and y.headers == headers
    with pytest.raises(hio.FormatError):
        hio.parse_index(open(path, "rb").read()[:-20])


def test_file_suffixes(tmp_path):
    (tmp_path / "a.MGF").write_bytes(b"BEGIN IONS\nCHARGE=2\nPEPMASS=500\n100 1\nEND IONS\n")
    (tmp_path / "b.dta").write_bytes(b"1000.5 2\n100 1\n")
    (tmp_path / "c.txt").write_bytes(b"")
    assert len(hio.read_spectra(str(tmp_path / "a.MGF"))) == 1
    assert len(hio.read_spectra(str(tmp_path / "b.dta"), tol=0.5)) == 1
    with pytest.raises(hio.FormatError):
        hio.read_spectra(str(tmp_path / "c.txt"))
    with pytest.raises(hio.FormatError):
        hio.read_spectra(str(tmp_path / "missing.mgf"))


def test_gzip_members_and_fasta_corners(F):
    """Concatenated gzip members read as one stream; empty and letterless
    sequence lines."""
    a = b">p1 one\nACDE\n"
    b = b">p2 two\n\n\nKKR\n>p3 empty\n>p4\nMM\n"
    data = gzip.compress(a) + gzip.compress(b)
    got = hio.parse_fasta(data, gz=True)
    ref = F.read_fasta(data, gz=True)
    assert got.headers == [h for h, _ in ref] == [b"p1 one", b"p2 two", b"p3 empty", b"p4"]
    assert got.seq.tobytes() == b"ACDEKKRMM" and got.seg.tolist() == [0, 4, 7, 7, 9]


def test_mgf_sample_without_peaks(F):
    text = b"BEGIN IONS\nPEPMASS=712.5\nCHARGE=2+\nEND IONS\n"
    got = hio.parse_spectra(text, "mgf")
    assert len(got) == 1 and got.off.tolist() == [0, 0] and got.pcr[0] == np.float32(712.5)
    assert F.read_mgf(text)[0][3] == []


def test_index_options_mass_table(F):
    """readIndex's readConfig over the options text: aa-mass-type and the
    add_X lines give the residue table (Config.hs:197-216, 266-272)."""
    import hfx_gb300
    for mono in (True, False):
        opts = F.index_options("db.fasta", 1, 1, 400.0, 7200.0, mono, {"C": 57.021, "M": 15.9949})
        x = hio.IndexFile(opts, [], np.zeros(0, np.uint8), np.zeros(1, np.uint32), np.zeros(0, np.float32),
                          np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(1, np.uint32))
        add = np.zeros(26, np.float32)
        add[ord("C") - 65], add[ord("M") - 65] = np.float32(57.021), np.float32(15.9949)
        want = hfx_gb300.mass_table(mono, add)
        assert np.array_equal(x.mass_table().view(np.uint32), want.view(np.uint32))
        assert x.option("missed-cleavages") == "1" and x.option("aa-mass-type") == ("Mono" if mono else "Average")
