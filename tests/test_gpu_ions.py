"""GPU parity of the "Ions" column (hfx_match_ions; Match.hs:36-44 over
IonSeries.hs:87-147) against the oracle, for every result of unmodified,
modified, BF16 and 0.02 Da searches, and on spectra built so that more than
200 peaks tie at the 200th value (ties taken in index order)."""
import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MA = b"MSTY"
MA_MASS = [15.995, 79.966, 79.966, 79.966]
H = np.float32(1.007276)
H2O = np.float32(18.010565)
NONE = np.iinfo(np.uint64).max


def _dev(sp):
    d = torch.device("cuda:0")
    return dict(mz=torch.from_numpy(sp.mz).to(d), it=torch.from_numpy(sp.it).to(d),
                off=torch.from_numpy(sp.off).to(d), pcr=torch.from_numpy(sp.pcr).to(d),
                z=torch.from_numpy(sp.z).to(d), tol=torch.from_numpy(sp.tol).to(d))


def _out(n, k):
    d = torch.device("cuda:0")
    return dict(score=torch.empty((n, k), dtype=torch.float32, device=d),
                key=torch.empty((n, k), dtype=torch.int64, device=d),
                pep=torch.empty((n, k), dtype=torch.int32, device=d),
                ncand=torch.empty(n, dtype=torch.int64, device=d))


def _run(eng, sp, p):
    dev = _dev(sp)
    out = _out(len(sp), p.top_n)
    eng.search_device(dev, p, out)
    eng.match_ions(dev, p, out)
    return (out["key"].cpu().numpy().view(np.uint64), out["pep"].cpu().numpy().view(np.uint32),
            out["ions_matched"].cpu().numpy(), out["ions_total"].cpu().numpy())


def _check(oracle, eng, sp, res, bw=1.0005079, custom_bw=False):
    key, pep, got_m, got_t = res
    r = eng.db_export()[0]
    mt = eng.db_export()[4]
    n_res = 0
    for i in range(len(sp)):
        a, b = sp.off[i], sp.off[i + 1]
        x = oracle.preprocess(sp.mz[a:b], sp.it[a:b], sp.pcr[i], sp.z[i], bw=bw, custom_bw=custom_bw)
        for j in range(key.shape[1]):
            if key[i, j] == NONE:
                assert (got_m[i, j], got_t[i, j]) == (0, 0)
                continue
            text, _, _ = eng.match(int(key[i, j]), int(pep[i, j]))
            body = text[2:-2]
            mh = np.float32(np.float32(r[pep[i, j]] + H) + H2O)
            want = oracle.match_ions(x, sp.z[i], body.replace("*", "").encode(), mt, mh, body.count("*"), bw)
            assert (got_m[i, j], got_t[i, j]) == want, (i, j, text)
            n_res += 1
    return n_res


@pytest.fixture(scope="module")
def eng_tiny(gpulib, tiny):
    import hfx_gb300
    prot, sp, cfg = tiny
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    yield eng, prot, sp
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_ions_plain(eng_tiny, oracle, precision):
    import hfx_gb300
    eng, prot, sp = eng_tiny
    sub = sp.subset(np.arange(32))
    p = hfx_gb300.default_params(top_n=10, precision=precision, batch_mode=1, rescore_k=32 if precision else 0)
    res = _run(eng, sub, p)
    assert _check(oracle, eng, sub, res) > 100
    assert (res[2][:, 0] > 0).mean() > 0.5          # the best matches explain peaks


def test_ions_mods(gpulib, tiny, oracle):
    """Modified matches: ions of the unmodified fragment, total over the
    text with its '*' marks."""
    import hfx_gb300
    prot, sp, cfg = tiny
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
        eng.set_mods(MA.decode(), MA_MASS, 4, False)
        sub = sp.subset(np.arange(24))
        res = _run(eng, sub, hfx_gb300.default_params(top_n=10, batch_mode=1))
        assert (res[0][res[0] != NONE] >> np.uint64(63)).any()
        assert _check(oracle, eng, sub, res) > 100
    finally:
        eng.close()


def test_ions_highres_rows(eng_tiny, oracle):
    import hfx_gb300
    eng, prot, sp = eng_tiny
    sub = sp.subset(np.arange(12))
    p = hfx_gb300.default_params(top_n=10, bin_width=0.02, custom_bin_width=1, batch_mode=1, ion_bins_custom=1)
    res = _run(eng, sub, p)
    assert _check(oracle, eng, sub, res, bw=0.02, custom_bw=True) > 50


def _tie_spectrum(prot, r, tc, tn, mt, p_idx, fillers):
    """Equal-intensity peaks at least 3.2 Da apart (so every one becomes the
    same positive XCorr value) at the fragment's b and y ions above 1000 m/z,
    plus `fillers` peaks below 996 m/z."""
    seq = prot.seq[tc[p_idx]:tn[p_idx] + 1]
    ladder = np.cumsum([np.float32(mt[c - ord("A")]) for c in seq], dtype=np.float32)
    mh = np.float32(np.float32(r[p_idx] + H) + H2O)
    ions = sorted(set([float(m + H) for m in ladder[:-1]] + [float(mh - (m + H)) for m in ladder[:-1]]))
    planted = []
    for v in ions:
        if v > 1000.0 and (not planted or v - planted[-1] >= 3.2):
            planted.append(v)
    fill = [100.0 + 3.2 * k for k in range(fillers) if 100.0 + 3.2 * k < 996.0]
    mz = np.array(fill + planted + [planted[-1] + 25.0], np.float32)
    z = np.float32(2.0)
    pcr = np.float32((np.float32(r[p_idx]) + 2 * H + H2O) / 2)
    return mz, np.full(len(mz), 100.0, np.float32), pcr, z


def test_ions_ties_at_the_200th_peak(eng_tiny, oracle):
    """More than 200 equal positive values: the first 200 in index order are
    peaks; removing the fillers lets the planted ion peaks count."""
    import hfx_gb300
    eng, prot, sp = eng_tiny
    r, tc, tn, idx, mt = eng.db_export()
    lens = tn.astype(np.int64) - tc.astype(np.int64)
    picks = [int(i) for i in np.nonzero((lens >= 14) & (r > 1500.0) & (r < 2600.0))[0][:4]]
    assert picks
    mzs, its, offs, pcrs, zs = [], [], [0], [], []
    for fillers in (260, 0):
        for p_idx in picks:
            mz, it, pcr, z = _tie_spectrum(prot, r, tc, tn, mt, p_idx, fillers)
            mzs.append(mz)
            its.append(it)
            offs.append(offs[-1] + len(mz))
            pcrs.append(pcr)
            zs.append(z)
    n = len(pcrs)
    spx = synth.Spectra(np.concatenate(mzs), np.concatenate(its), np.array(offs, np.int64),
                        np.array(pcrs, np.float32), np.array(zs, np.float32), np.full(n, 0.05, np.float32))
    p = hfx_gb300.default_params(top_n=10, bin_width=0.02, custom_bin_width=1, batch_mode=1, ion_bins_custom=1)
    res = _run(eng, spx, p)
    _check(oracle, eng, spx, res, bw=0.02, custom_bw=True)
    key, pep, got_m, _ = res
    k = len(picks)
    for a, p_idx in enumerate(picks):
        pos = int(np.nonzero(idx == p_idx)[0][0])
        tied = np.nonzero(key[a] == pos)[0]
        free = np.nonzero(key[k + a] == pos)[0]
        assert len(tied) == 1 and len(free) == 1, (a, key[a], pos)
        assert got_m[a, tied[0]] < got_m[k + a, free[0]], (a, got_m[a], got_m[k + a])


def test_scan_report(eng_tiny):
    """printScanResults text of searched spectra: the header, the results
    table with the search's own XCorr / Ions / E-value and the details."""
    import hfx_gb300
    from hfx_gb300 import report
    eng, prot, sp = eng_tiny
    sub = sp.subset(np.arange(6))
    headers = [b"sp|P%05d|PROT%d Protein %d - Homo sapiens" % (i, i, i) for i in range(len(prot.seg) - 1)]
    dev = _dev(sub)
    out = _out(len(sub), 10)
    out["ev"] = torch.empty((len(sub), 10), dtype=torch.float64, device="cuda:0")
    out["fit"] = torch.empty((len(sub), 3), dtype=torch.float64, device="cuda:0")
    p = hfx_gb300.default_params(top_n=10, batch_mode=1)
    eng.search_evalues(dev, p, out)
    eng.match_ions(dev, p, out)
    res = hfx_gb300.SearchResult(score=out["score"].cpu().numpy(), key=out["key"].cpu().numpy().view(np.uint64),
                                 pep=out["pep"].cpu().numpy().view(np.uint32), ncand=out["ncand"].cpu().numpy())
    ions = (out["ions_matched"].cpu().numpy(), out["ions_total"].cpu().numpy())
    ev = out["ev"].cpu().numpy()
    for i in range(len(sub)):
        txt = report.scan_report(eng, headers, sub, i, res, ions, ev, "run.mgf", "db.fasta", "Trypsin KR P")
        blocks = txt.split("\n\n")
        assert len(blocks) == 4 and blocks[-1] == ""
        rows = blocks[1].split("\n")
        assert rows[0].split() == ["#", "(M+H)+", "deltCn", "XCorr", "Ions", "Reference", "Peptide", "E-value"]
        top = rows[2].split()
        text, mh, prot_i = eng.match(int(res.key[i, 0]), int(res.pep[i, 0]))
        assert top[0] == "1." and top[2] == "0.0000" and top[6] == text
        assert top[4] == f"{ions[0][i, 0]}/{ions[1][i, 0]}" and top[5] == headers[prot_i].split()[0].decode()
        assert top[3] == report.format_number(float(np.float32(res.score[i, 0] / np.float32(10000))), 2)
        assert top[7] == report.format_number(float(ev[i, 0]), 3)
        assert blocks[2].split("\n")[0].startswith(" 1.  " + headers[prot_i].decode())
