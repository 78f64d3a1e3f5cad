"""GPU parity at the benchmark database: 20,000 proteins (1.40 M peptides
after the 6-50 length filter).  The modification search (M, S, T, Y, up to
three modifications), the open +-500 Da windows of the batching workload
(~5.6e5 candidates per spectrum) next to +-10 ppm ones, and the 0.02 Da rows
(~10^5 bins), each on spectra of that workload, compared with the oracle's
keys, FP32 scores, fragment indices and candidate counts bit for bit.  The
samples are sized so that the oracle finishes each in seconds on the host
cores."""
import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def full_db(gpulib, oracle):
    import hfx_gb300
    prot = synth.proteins(20000, seed=1)
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    r, tc, tn, idx, mt = eng.db_export()
    assert len(r) > 1_000_000
    yield eng, prot, (r, tc, tn, idx, mt)
    eng.close()


def _compare(res, ref, label):
    sc, _, key, pep, nc = ref
    assert np.array_equal(res.ncand, nc), label
    assert np.array_equal(res.key, key), label
    assert np.array_equal(res.score.view(np.uint32), sc.view(np.uint32)), label
    assert np.array_equal(res.pep, pep), label


def test_mods_at_scale(full_db, oracle):
    """The modification workload: variable M+15.995, S/T/Y+79.966,
    max-modable-acids 4 (up to three modifications, 34 combinations;
    Fragment.hs:260-289), FP32 and the BF16 engine with FP32 rescoring."""
    import hfx_gb300
    eng, prot, (r, tc, tn, idx, mt) = full_db
    _, sp, cfg = synth.workload("mods", n_spectra=200)
    ma = cfg["ma"]
    ions = oracle.pack_ions(prot.seq, ma.encode())
    ref = oracle.search(ions, mt, r, tc, tn, idx, sp, topn=10, ma=ma.encode(), ma_mass=cfg["ma_mass"],
                        max_ma=cfg["max_ma"])
    assert int(ref[4].sum()) > 1_000_000  # modified isoforms and plain candidates
    eng.set_mods(ma, cfg["ma_mass"], cfg["max_ma"])
    try:
        for prec in (0, 1):
            p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=prec, rescore_k=32 if prec else 0)
            _compare(eng.search(sp, p), ref, f"mods precision {prec}")
    finally:
        eng.set_mods("", [], 0)


def test_open_windows_at_scale(full_db, oracle):
    """The batching workload: +-500 Da windows of ~5.6e5 candidates next to
    +-10 ppm ones in one batched launch (FP32, and BF16 + FP32 rescoring)."""
    import hfx_gb300
    eng, prot, (r, tc, tn, idx, mt) = full_db
    _, sp, cfg = synth.workload("batch", n_spectra=400)
    wide = np.nonzero(sp.tol > 0)[0][:24]
    narrow = np.nonzero(sp.tol < 0)[0][:40]
    sub = sp.subset(np.sort(np.concatenate([wide, narrow])))
    ions = oracle.pack_ions(prot.seq)
    ref = oracle.search(ions, mt, r, tc, tn, idx, sub, topn=10, ppm=2)
    nc = ref[4]
    assert nc[sub.tol > 0].mean() > 3e5 and nc[sub.tol < 0].max() < 2000
    for prec in (0, 1):
        p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=prec, rescore_k=32 if prec else 0,
                                     tol_ppm=2)
        _compare(eng.search(sub, p), ref, f"open windows precision {prec}")


def test_002_da_rows_at_scale(full_db, oracle):
    """The 0.02 Da workload: the batching spectra binned at 0.02 Da (custom
    ion bin width), BF16 and FP16 rows with the top 50 rescored in FP32."""
    import hfx_gb300
    eng, prot, (r, tc, tn, idx, mt) = full_db
    _, sp, cfg = synth.workload("highres", n_spectra=400)
    sub = sp.subset(np.sort(np.concatenate([np.nonzero(sp.tol < 0)[0][:48], np.nonzero(sp.tol > 0)[0][:2]])))
    ions = oracle.pack_ions(prot.seq)
    ref = oracle.search(ions, mt, r, tc, tn, idx, sub, topn=10, bw=0.02, custom_bw=True, ppm=2, ion_bw=0.02)
    assert ref[4].max() > 3e5  # the open windows
    for prec in (1, 2):
        p = hfx_gb300.default_params(top_n=10, bin_width=0.02, custom_bin_width=1, ion_bins_custom=1, tol_ppm=2,
                                     batch_mode=1, precision=prec, rescore_k=50)
        _compare(eng.search(sub, p), ref, f"0.02 Da precision {prec}")
