"""GPU parity of the device E-values (hfx_search_evalues) against the
oracle's restatement of Util/Statistics.hs over every candidate's FP32 score
(computed by the oracle, one candidate at a time)."""
import math

import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _oracle_all_scores(oracle, eng, prot, sp, i, bw=1.0005079, custom_bw=False):
    """FP32 XCorr of every candidate in spectrum i's window (mass order)."""
    r, tc, tn, idx, mt = eng.db_export()
    ions = oracle.pack_ions(prot.seq)
    a, b = sp.off[i], sp.off[i + 1]
    x = oracle.preprocess(sp.mz[a:b], sp.it[a:b], sp.pcr[i], sp.z[i], bw=bw, custom_bw=custom_bw)
    if x is None:
        return np.zeros(0, np.float32)
    m = np.float32(oracle.ms2_mass(sp.pcr[i], sp.z[i]))
    tol = np.float32(sp.tol[i])
    lo, hi = oracle.windows(r[idx], np.array([m - tol], np.float32), np.array([m + tol], np.float32))
    ch = oracle.ion_charges(float(sp.z[i]))
    out = []
    for q in range(int(lo[0]), int(hi[0])):
        p = idx[q]
        bins, lvl = oracle.ion_bins(ions, mt, int(tc[p]), int(tn[p]), float(r[p]), ch, len(x))
        out.append(oracle.score32(bins, lvl, x))
    return np.array(out, np.float32)


def _dev(sp):
    d = torch.device("cuda:0")
    return dict(mz=torch.from_numpy(sp.mz).to(d), it=torch.from_numpy(sp.it).to(d),
                off=torch.from_numpy(sp.off).to(d), pcr=torch.from_numpy(sp.pcr).to(d),
                z=torch.from_numpy(sp.z).to(d), tol=torch.from_numpy(sp.tol).to(d))


@pytest.fixture(scope="module")
def eng_tiny(gpulib, tiny):
    import hfx_gb300
    prot, sp, cfg = tiny
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    yield eng, prot, sp
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_evalues_match_oracle(eng_tiny, oracle, precision):
    import hfx_gb300
    eng, prot, sp = eng_tiny
    sub = sp.subset(np.arange(24))
    n = len(sub)
    d = torch.device("cuda:0")
    out = dict(score=torch.empty((n, 10), dtype=torch.float32, device=d),
               key=torch.empty((n, 10), dtype=torch.int64, device=d),
               pep=torch.empty((n, 10), dtype=torch.int32, device=d),
               ncand=torch.empty(n, dtype=torch.int64, device=d),
               ev=torch.empty((n, 10), dtype=torch.float64, device=d),
               fit=torch.empty((n, 3), dtype=torch.float64, device=d))
    p = hfx_gb300.default_params(top_n=10, precision=precision, batch_mode=1, rescore_k=32 if precision else 0)
    eng.search_evalues(_dev(sub), p, out)
    fit = out["fit"].cpu().numpy()
    ev = out["ev"].cpu().numpy()
    score = out["score"].cpu().numpy()
    key = out["key"].cpu().numpy().view(np.uint64)
    ref = eng.search(sub, hfx_gb300.default_params(top_n=10, precision=precision, batch_mode=1,
                                                   rescore_k=32 if precision else 0))
    assert np.array_equal(key, ref.key) and np.array_equal(score.view(np.uint32), ref.score.view(np.uint32))
    fitted = 0
    for i in range(n):
        all_sc = _oracle_all_scores(oracle, eng, prot, sub, i)
        a, b, m = oracle.evalue_fit(all_sc)
        assert int(fit[i, 2]) == m, i
        if m < 2:
            continue
        fitted += 1
        assert math.isclose(fit[i, 0], a, rel_tol=1e-9, abs_tol=1e-9), (i, fit[i], a, b)
        assert math.isclose(fit[i, 1], b, rel_tol=1e-9, abs_tol=1e-9), (i, fit[i], a, b)
        for j in range(10):
            if key[i, j] == np.iinfo(np.uint64).max:
                assert math.isnan(ev[i, j])
                continue
            assert math.isclose(ev[i, j], oracle.evalue(a, b, score[i, j]), rel_tol=1e-8), (i, j)
    assert fitted >= n // 2


def test_evalues_parameters(eng_tiny, oracle):
    """Another bin width and cut-off, as --evalue-bin-width and
    --evalue-high-cutoff-percentage would set them."""
    import hfx_gb300
    eng, prot, sp = eng_tiny
    sub = sp.subset(np.arange(8))
    n = len(sub)
    d = torch.device("cuda:0")
    out = dict(score=torch.empty((n, 5), dtype=torch.float32, device=d),
               key=torch.empty((n, 5), dtype=torch.int64, device=d),
               pep=torch.empty((n, 5), dtype=torch.int32, device=d),
               ncand=torch.empty(n, dtype=torch.int64, device=d),
               ev=torch.empty((n, 5), dtype=torch.float64, device=d),
               fit=torch.empty((n, 3), dtype=torch.float64, device=d))
    eng.search_evalues(_dev(sub), hfx_gb300.default_params(top_n=5), out, bin_width=200, cutoff_perc=5.0)
    fit = out["fit"].cpu().numpy()
    for i in range(n):
        a, b, m = oracle.evalue_fit(_oracle_all_scores(oracle, eng, prot, sub, i), bin_width=200, cutoff_perc=5.0)
        assert int(fit[i, 2]) == m
        if m >= 2:
            assert math.isclose(fit[i, 1], b, rel_tol=1e-9, abs_tol=1e-9)


MA = b"MSTY"
MA_MASS = [15.995, 79.966, 79.966, 79.966]   # Met oxidation, Ser/Thr/Tyr phosphorylation


@pytest.mark.parametrize("precision,plain,per_type", [(0, 1, False), (1, 1, False), (0, 0, True)])
def test_evalues_with_mods(gpulib, tiny, oracle, precision, plain, per_type):
    """A modification search fits over every match of the spectrum, modified
    isoforms included (Search.hs:116-121); the oracle hands back the same
    score list (plain candidates, then every isoform)."""
    import hfx_gb300
    prot, sp, cfg = tiny
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
        eng.set_mods(MA.decode(), MA_MASS, 4, per_type)
        sub = sp.subset(np.arange(16))
        n = len(sub)
        d = torch.device("cuda:0")
        out = dict(score=torch.empty((n, 10), dtype=torch.float32, device=d),
                   key=torch.empty((n, 10), dtype=torch.int64, device=d),
                   pep=torch.empty((n, 10), dtype=torch.int32, device=d),
                   ncand=torch.empty(n, dtype=torch.int64, device=d),
                   ev=torch.empty((n, 10), dtype=torch.float64, device=d),
                   fit=torch.empty((n, 3), dtype=torch.float64, device=d))
        p = hfx_gb300.default_params(top_n=10, precision=precision, batch_mode=1, search_plain=plain,
                                     rescore_k=32 if precision else 0)
        eng.search_evalues(_dev(sub), p, out)
        r, tc, tn, idx, mt = eng.db_export()
        sc, _, key, pep, nc, all_sc = oracle.search(oracle.pack_ions(prot.seq, MA), mt, r, tc, tn, idx, sub,
                                                    topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4, per_type=per_type,
                                                    plain=bool(plain), all_scores=True)
        assert np.array_equal(out["ncand"].cpu().numpy(), nc)
        assert np.array_equal(out["key"].cpu().numpy().view(np.uint64), key)
        assert np.array_equal(out["score"].cpu().numpy().view(np.uint32), sc.view(np.uint32))
        assert (key[key != np.iinfo(np.uint64).max] >> np.uint64(63)).any()
        fit = out["fit"].cpu().numpy()
        ev = out["ev"].cpu().numpy()
        fitted = 0
        for i in range(n):
            assert len(all_sc[i]) == nc[i]
            a, b, m = oracle.evalue_fit(all_sc[i])
            assert int(fit[i, 2]) == m, i
            if m < 2:
                continue
            fitted += 1
            assert math.isclose(fit[i, 0], a, rel_tol=1e-9, abs_tol=1e-9), (i, fit[i], a, b)
            assert math.isclose(fit[i, 1], b, rel_tol=1e-9, abs_tol=1e-9), (i, fit[i], a, b)
            for j in range(10):
                if key[i, j] != np.iinfo(np.uint64).max:
                    assert math.isclose(ev[i, j], oracle.evalue(a, b, sc[i, j]), rel_tol=1e-8), (i, j)
        assert fitted >= n // 2
    finally:
        eng.close()
