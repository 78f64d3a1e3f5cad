"""End to end through the file readers: a FASTA (and .gz) database and MGF
spectra written from the seeded workload, read back by libhfx_gpu.so and
searched, give the same results as the in-memory arrays; so does a database
written to a .index file and uploaded from it (readIndex + withDeviceDB)."""
import gzip

import numpy as np
import pytest

from hfx_gb300 import io as hio
from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _fasta(prot):
    out = []
    for i in range(len(prot.seg) - 1):
        s = bytes(prot.seq[prot.seg[i]:prot.seg[i + 1]])
        out.append(b">sp|P%05d|PROT%d Protein %d" % (i, i, i))
        out += [s[k:k + 60] for k in range(0, len(s), 60)]
    return b"\n".join(out) + b"\n"


def _f(x):
    return np.format_float_positional(np.float32(x), unique=True, trim="0")


def _mgf(sp):
    out = []
    for i in range(len(sp)):
        out += ["BEGIN IONS", f"TITLE=spectrum {i}", f"PEPMASS={_f(sp.pcr[i])}", f"CHARGE={int(sp.z[i])}+"]
        a, b = sp.off[i], sp.off[i + 1]
        out += [f"{_f(m)} {_f(v)}" for m, v in zip(sp.mz[a:b], sp.it[a:b])]
        out.append("END IONS")
    return ("\n".join(out) + "\n").encode()


def _same(a, b):
    assert np.array_equal(a.key, b.key) and np.array_equal(a.pep, b.pep) and np.array_equal(a.ncand, b.ncand)
    assert np.array_equal(a.score.view(np.uint32), b.score.view(np.uint32))


@pytest.fixture(scope="module")
def direct(gpulib, tiny):
    import hfx_gb300
    prot, sp, cfg = tiny
    sub = sp.subset(np.arange(48))
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    res = eng.search(sub, hfx_gb300.default_params(top_n=10, batch_mode=1))
    yield eng, prot, sub, res
    eng.close()


@pytest.mark.parametrize("gz", [False, True])
def test_fasta_and_mgf_files(direct, tmp_path, gz):
    import hfx_gb300
    eng0, prot, sub, ref = direct
    data = _fasta(prot)
    db = tmp_path / ("db.fasta.gz" if gz else "db.fasta")
    db.write_bytes(gzip.compress(data) if gz else data)
    (tmp_path / "run.mgf").write_bytes(_mgf(sub))
    pf = hio.read_fasta(str(db))
    assert pf.seq.tobytes() == prot.seq.tobytes() and np.array_equal(pf.seg, prot.seg)
    spx = hio.read_spectra(str(tmp_path / "run.mgf"), tol=float(sub.tol[0]))
    spx.tol = sub.tol.copy()
    assert spx.title[3] == b"spectrum 3"
    assert np.array_equal(spx.mz.view(np.uint32), sub.mz.view(np.uint32))
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(pf.seq, pf.seg, static_add=synth.static_mods(), **synth.DIGEST)
        _same(eng.search(spx, hfx_gb300.default_params(top_n=10, batch_mode=1)), ref)
    finally:
        eng.close()


def test_index_file(direct, tmp_path):
    import hfx_gb300
    eng0, prot, sub, ref = direct
    r, tc, tn, idx, mt = eng0.db_export()      # fragments in digest order
    nf = len(idx)
    frag_seg = np.concatenate([np.searchsorted(tc, prot.seg[:-1]), [nf]]).astype(np.uint32)
    adds = {chr(ord("A") + i): float(v) for i, v in enumerate(synth.static_mods()) if v != 0}
    opts = "\n" + "".join(f"{k} = {v}\n" for k, v in [("database", "db.fasta"), ("missed-cleavages", 1),
                                                       ("digestion-rule", 1), ("aa-mass-type", "Mono")])
    opts += "".join(f"add_{k} = {_f(v)}\n" for k, v in adds.items())
    headers = [b"sp|P%05d" % i for i in range(len(prot.seg) - 1)]
    path = str(tmp_path / "db.index")
    hio.write_index(path, hio.IndexFile(opts, headers, prot.seq, prot.seg, r, tc, tn, frag_seg))
    x = hio.read_index(path)
    assert np.array_equal(x.mass_table().view(np.uint32), mt.view(np.uint32))
    eng = hfx_gb300.Engine(0)
    try:
        eng.upload_db(x.ions, x.r, x.c, x.n, x.mass_table())
        _same(eng.search(sub, hfx_gb300.default_params(top_n=10, batch_mode=1)), ref)
    finally:
        eng.close()


@pytest.mark.parametrize("mono,rule,missed,pr,lo,hi", [(True, 1, 1, True, 6, 50), (True, 1, 2, False, 0, 0),
                                                      (False, 2, 0, False, 0, 0), (True, 0, 0, False, 0, 0),
                                                      (True, 13, 1, True, 3, 30), (True, 6, 3, True, 0, 0),
                                                      (True, 8, 1, False, 7, 0), (True, 12, 2, False, 0, 20)])
def test_device_digest_matches_oracle(gpulib, oracle, tiny, mono, rule, missed, pr, lo, hi):
    """The database digest on the device (hfx_digest_gpu, used by
    hfx_build_db) equals the oracle's restatement of makeSeqDB's digest
    element for element: order, FP32 masses, tc and tn."""
    import hfx_gb300
    prot, _, _ = tiny
    mt = oracle.mass_table(mono, synth.static_mods())
    eng = hfx_gb300.Engine(0)
    try:
        a = eng.digest(prot.seq, prot.seg, mt, rule=rule, missed=missed, proline_rule=pr, min_len=lo, max_len=hi)
        b = oracle.digest(prot.seq, prot.seg, mt, rule=rule, missed=missed, proline_rule=pr, min_len=lo, max_len=hi)
        assert len(a[0]) == len(b[0])
        assert rule == 0 or len(a[0]) > 0  # rule 0 never cleaves: whole proteins, all above 7200 Da
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    finally:
        eng.close()


def test_device_digest_edges(gpulib, oracle):
    """Empty proteins, a protein of one residue, cleavage at the last residue
    and proline after the cleavage site."""
    import hfx_gb300
    seqs = [b"", b"K", b"PEPTIDEK", b"AKPRKRP", b"", b"MKWVTFISLLLLFSSAYSRGVFRRDTHK", b"R"]
    seq = np.frombuffer(b"".join(seqs), np.uint8).copy()
    seg = np.cumsum([0] + [len(x) for x in seqs]).astype(np.uint32)
    mt = oracle.mass_table(True, synth.static_mods())
    eng = hfx_gb300.Engine(0)
    try:
        for pr in (False, True):
            for missed in (0, 1, 2):
                a = eng.digest(seq, seg, mt, rule=1, missed=missed, proline_rule=pr, min_mass=0.0, max_mass=1e6)
                b = oracle.digest(seq, seg, mt, rule=1, missed=missed, proline_rule=pr, min_mass=0.0, max_mass=1e6)
                for x, y in zip(a, b):
                    assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (pr, missed)
    finally:
        eng.close()
