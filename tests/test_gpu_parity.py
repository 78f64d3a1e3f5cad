"""GPU parity tests: the CUDA path, called through the C ABI, against the
oracle on the same seeded inputs.  Integer / index / ordering results must
be bit-exact; FP32 scores and rows are bit-exact too because the kernels
follow the oracle's canonical operation order."""
import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(sp):
    d = torch.device("cuda:0")
    return dict(mz=torch.from_numpy(sp.mz).to(d), it=torch.from_numpy(sp.it).to(d),
                off=torch.from_numpy(sp.off).to(d), pcr=torch.from_numpy(sp.pcr).to(d),
                z=torch.from_numpy(sp.z).to(d), tol=torch.from_numpy(sp.tol).to(d))


def _engine(prot, digest=None):
    import hfx_gb300
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **(digest or synth.DIGEST))
    return eng


@pytest.fixture(scope="module")
def tiny_engine(gpulib, tiny):
    prot, sp, cfg = tiny
    eng = _engine(prot)
    yield eng, prot, sp
    eng.close()


@pytest.fixture(scope="module")
def full_engine(gpulib):
    prot = synth.proteins(20000, seed=1)
    sp = synth.spectra(prot, 240, seed=101, charge_p={1: 0.05, 2: 0.5, 3: 0.35, 4: 0.10}, npeaks=(50, 400))
    eng = _engine(prot)
    yield eng, prot, sp
    eng.close()


def _oracle_db(oracle, eng, prot, ma=b""):
    r, tc, tn, idx, mt = eng.db_export()
    ions = oracle.pack_ions(prot.seq, ma)
    return ions, mt, r, tc, tn, idx


def test_preprocess_bitexact(tiny_engine, oracle):
    import hfx_gb300
    eng, prot, sp = tiny_engine
    p = hfx_gb300.default_params()
    dev = _dev(sp)
    stride = 8192
    n = len(sp)
    rows = torch.empty((n, stride), dtype=torch.float32, device="cuda")
    rbf = torch.empty((n, stride), dtype=torch.bfloat16, device="cuda")
    rh = torch.empty((n, stride), dtype=torch.float16, device="cuda")
    lens = torch.empty(n, dtype=torch.int32, device="cuda")
    masses = torch.empty(n, dtype=torch.float32, device="cuda")
    eng.preprocess(dev, p, stride, rows, rbf, rh, lens, masses)
    rows, lens, masses = rows.cpu().numpy(), lens.cpu().numpy(), masses.cpu().numpy()
    rbf = rbf.float().cpu().numpy()
    rh = rh.float().cpu().numpy()
    for i in range(n):
        a, b = sp.off[i], sp.off[i + 1]
        x = oracle.preprocess(sp.mz[a:b], sp.it[a:b], sp.pcr[i], sp.z[i])
        assert lens[i] == len(x)
        assert np.array_equal(rows[i, :len(x)].view(np.uint32), x.view(np.uint32)), i
        assert not rows[i, len(x):].any()
        assert np.array_equal(rbf[i, :len(x)], torch.from_numpy(x).bfloat16().float().numpy())
        assert np.array_equal(rh[i, :len(x)], x.astype(np.float16).astype(np.float32))
        assert masses[i] == np.float32(oracle.ms2_mass(sp.pcr[i], sp.z[i]))


def test_windows_exact(full_engine, oracle):
    import hfx_gb300
    eng, prot, sp = full_engine
    r, tc, tn, idx, mt = eng.db_export()
    rs = r[idx]
    for tol in (3.0, 0.5, 0.01):
        sp.tol[:] = tol
        dev = _dev(sp)
        b = torch.empty(len(sp), dtype=torch.int32, device="cuda")
        e = torch.empty(len(sp), dtype=torch.int32, device="cuda")
        eng.find_windows(dev, hfx_gb300.default_params(), b, e)
        m = np.array([oracle.ms2_mass(p, z) for p, z in zip(sp.pcr, sp.z)], np.float32)
        ob, oe = oracle.windows(rs, (m - np.float32(tol)).astype(np.float32), (m + np.float32(tol)).astype(np.float32))
        assert np.array_equal(b.cpu().numpy().astype(np.uint32), ob)
        assert np.array_equal(e.cpu().numpy().astype(np.uint32), oe)
    sp.tol[:] = 3.0


@pytest.mark.parametrize("fastdiv", [False, True])
def test_ion_bins(full_engine, oracle, fastdiv):
    eng, prot, sp = full_engine
    ions, mt, r, tc, tn, idx = _oracle_db(oracle, eng, prot)
    rng = np.random.Generator(np.random.PCG64(21))
    n = 3000
    pos = rng.integers(0, len(r), n).astype(np.uint32)
    pos[:50] = np.argsort(tn[idx] - tc[idx])[-50:]          # the longest peptides
    ch = rng.integers(1, 5, n).astype(np.int32)
    lens = rng.integers(200, 4000, n).astype(np.int32)
    cap = 4096
    d = torch.device("cuda")
    bins = torch.zeros((n, cap), dtype=torch.int32, device=d)
    lvl = torch.zeros((n, cap), dtype=torch.uint8, device=d)
    cnt = torch.zeros(n, dtype=torch.int32, device=d)
    eng.ion_bins(torch.from_numpy(pos.astype(np.int32)).to(d), torch.from_numpy(ch).to(d),
                 torch.from_numpy(lens).to(d), cap, bins, lvl, cnt, fastdiv=fastdiv)
    bins, lvl, cnt = bins.cpu().numpy(), lvl.cpu().numpy(), cnt.cpu().numpy()
    mismatch = 0
    for i in range(n):
        p = idx[pos[i]]
        ob, ol = oracle.ion_bins(ions, mt, tc[p], tn[p], r[p], int(ch[i]), int(lens[i]))
        same = cnt[i] == len(ob) and np.array_equal(bins[i, :cnt[i]].view(np.uint32), ob) and \
            np.array_equal(lvl[i, :cnt[i]], ol)
        if not fastdiv:
            assert same, i
        mismatch += not same
    if fastdiv:
        # __fdividef moves bins that sit within ~2 ulp of a half-bin edge
        print(f"fastdiv: {mismatch}/{n} candidates differ from IEEE division")
        assert mismatch < 0.2 * n


def _compare(res, ref, label):
    sc, _, key, pep, nc = ref
    assert np.array_equal(res.ncand, nc), label
    assert np.array_equal(res.key, key), label
    assert np.array_equal(res.score.view(np.uint32), sc.view(np.uint32)), label
    assert np.array_equal(res.pep, pep), label


def test_search_plain_tiny(tiny_engine, oracle):
    import hfx_gb300
    eng, prot, sp = tiny_engine
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10))
    _compare(res, ref, "tiny")


def test_search_plain_full_subset(full_engine, oracle):
    import hfx_gb300
    eng, prot, sp = full_engine
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10))
    _compare(res, ref, "full")
    res32 = eng.search(sp, hfx_gb300.default_params(top_n=32))
    ref32 = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=32)
    _compare(res32, ref32, "full top32")


def test_search_deterministic(full_engine):
    import hfx_gb300
    eng, prot, sp = full_engine
    p = hfx_gb300.default_params(top_n=10)
    a = eng.search(sp, p)
    b = eng.search(sp, p)
    assert np.array_equal(a.score.view(np.uint32), b.score.view(np.uint32))
    assert np.array_equal(a.key, b.key)


def _edge_spectra(sp):
    """Six spectra: an empty one, an (almost) empty window, a charge without
    ions (max charge 5), a one-peak spectrum and two ordinary ones."""
    sub = sp.subset(np.arange(6))
    mz, it, off = [], [], [0]
    for i in range(6):
        a, b = sub.off[i], sub.off[i + 1]
        if i == 0:
            a = b                                   # empty spectrum
        if i == 3:
            a = b - 1                               # one peak
        mz.append(sub.mz[a:b])
        it.append(sub.it[a:b])
        off.append(off[-1] + (b - a))
    sub.mz, sub.it, sub.off = np.concatenate(mz), np.concatenate(it), np.array(off, np.int64)
    sub.tol[1] = 1e-7                               # (almost) empty window
    sub.z[2] = 6.0                                  # max charge 5: no ions
    return sub


# (batch_mode, precision, use_graph): the per-spectrum path, the list path in
# FP32 and BF16 (eager and replayed) and the fused path
EDGE_MODES = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1), (2, 0, 0)]


@pytest.mark.parametrize("mode,precision,graph", EDGE_MODES)
def test_search_edge_cases(tiny_engine, oracle, mode, precision, graph):
    """Empty spectrum, empty window, charge without ions (max charge > 4
    scores 0 in the reference's plain kernel), a one-peak spectrum, on
    every search path."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = _edge_spectra(sp)
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=10)
    p = hfx_gb300.default_params(top_n=10, batch_mode=mode, precision=precision, use_graph=graph,
                                 rescore_k=32 if precision else 0)
    for rep in range(2 if graph else 1):
        res = eng.search(sub, p)
        _compare(res, ref, f"edges mode={mode} precision={precision} graph={graph} rep={rep}")
        assert res.ncand[0] == 0
        assert (res.score[2][res.key[2] != np.iinfo(np.uint64).max] == 0).all()


@pytest.mark.parametrize("mode,precision,graph", EDGE_MODES)
def test_no_candidates_in_the_batch(tiny_engine, oracle, mode, precision, graph):
    """A batch whose windows are all empty (precursors far above the
    database): no lists, no work items, every result the empty key."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = sp.subset(np.arange(5))
    sub.z[:] = 2.0
    sub.pcr[:] = 3900.0                             # ~7,798 Da: above every peptide, rows < 8,192 bins
    sub.tol[:] = 1.0
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=10)
    assert int(ref[4].sum()) == 0
    p = hfx_gb300.default_params(top_n=10, batch_mode=mode, precision=precision, use_graph=graph,
                                 rescore_k=32 if precision else 0)
    for rep in range(2 if graph else 1):
        res = eng.search(sub, p)
        _compare(res, ref, f"no candidates mode={mode} precision={precision} graph={graph} rep={rep}")
        assert (res.key == np.iinfo(np.uint64).max).all()


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("G", [1, 2, 4, 8])
def test_batched_fp32_bitexact(full_engine, oracle, G, mode):
    import hfx_gb300
    eng, prot, sp = full_engine
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=mode, group_size=G, chunk=512))
    _compare(res, ref, f"batched mode={mode} G={G}")


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("precision", [1, 2])
def test_batched_lowp_rescore_matches_fp32(full_engine, oracle, precision, mode):
    """BF16 / FP16 rows pick the kept candidates, FP32 rescoring restores the
    exact FP32 scores: the top-10 equals the FP32 oracle's."""
    import hfx_gb300
    eng, prot, sp = full_engine
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=mode, precision=precision, rescore_k=32))
    _compare(res, ref, f"precision {precision} mode {mode}")


@pytest.mark.parametrize("chunk", [512, 4096])
@pytest.mark.parametrize("precision", [1, 2])
def test_group16_lowp_rescore(full_engine, oracle, precision, chunk):
    """16-spectrum groups (two 16-byte tile loads per bin, reduce-scatter
    over 16 slots): the FP32-rescored top-10 equals the oracle's."""
    import hfx_gb300
    eng, prot, sp = full_engine
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=1, precision=precision, rescore_k=32,
                                                  group_size=16, chunk=chunk))
    _compare(res, ref, f"G=16 precision {precision} chunk {chunk}")


def test_group16_needs_lowp_lists(full_engine):
    """group_size 16 is refused for FP32 rows and for the fused batch mode."""
    import hfx_gb300
    eng, prot, sp = full_engine
    sub = sp.subset(np.arange(8))
    for kw in (dict(precision=0, batch_mode=1), dict(precision=1, batch_mode=2)):
        with pytest.raises(hfx_gb300.HfxError):
            eng.search(sub, hfx_gb300.default_params(top_n=10, group_size=16, **kw))


def test_batched_tiny_and_edges(tiny_engine, oracle):
    import hfx_gb300
    eng, prot, sp = tiny_engine
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
    for prec in (0, 1):
        res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=1, precision=prec))
        _compare(res, ref, f"tiny batched prec={prec}")


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_mixed_tolerance_open_search(tiny_engine, oracle, mode):
    """Per-spectrum tolerance units (tol_ppm = 2: negative = ppm): narrow
    +-10 ppm windows next to open +-500 Da windows (10^4-10^5 candidates,
    cut into wide work items), bit-exact against the oracle."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = sp.subset(np.arange(40))
    sub.tol[:] = -10.0
    sub.tol[::5] = 500.0
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=10, ppm=2)
    assert ref[4][::5].min() > 10000 and ref[4][1::5].max() < 1000
    res = eng.search(sub, hfx_gb300.default_params(top_n=10, batch_mode=mode, tol_ppm=2))
    _compare(res, ref, f"mixed tolerance mode={mode}")
    if mode:
        res = eng.search(sub, hfx_gb300.default_params(top_n=10, batch_mode=mode, tol_ppm=2, precision=1))
        _compare(res, ref, f"mixed tolerance bf16 mode={mode}")


HIGHRES = 0.02   # Da per bin: ~10^5 bins per row, beyond shared memory


def _highres_subset(sp, n=16):
    sub = sp.subset(np.arange(n))
    return sub


def test_long_rows_preprocess_bitexact(tiny_engine, oracle):
    """0.02 Da rows (~10^5 bins) are built sparsely; they equal the dense
    oracle rows bit for bit, with BF16/FP16 copies."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = _highres_subset(sp, 12)
    p = hfx_gb300.default_params(bin_width=HIGHRES, custom_bin_width=1)
    xs = [oracle.preprocess(sub.mz[sub.off[i]:sub.off[i + 1]], sub.it[sub.off[i]:sub.off[i + 1]], sub.pcr[i],
                            sub.z[i], bw=HIGHRES, custom_bw=True) for i in range(len(sub))]
    stride = (max(len(x) for x in xs) + 15) // 16 * 16
    assert stride > 51200
    n = len(sub)
    rows = torch.empty((n, stride), dtype=torch.float32, device="cuda")
    rbf = torch.empty((n, stride), dtype=torch.bfloat16, device="cuda")
    rh = torch.empty((n, stride), dtype=torch.float16, device="cuda")
    lens = torch.empty(n, dtype=torch.int32, device="cuda")
    eng.preprocess(_dev(sub), p, stride, rows, rbf, rh, lens, None)
    rows, lens = rows.cpu().numpy(), lens.cpu().numpy()
    rbf, rh = rbf.float().cpu().numpy(), rh.float().cpu().numpy()
    for i, x in enumerate(xs):
        assert lens[i] == len(x)
        assert np.array_equal(rows[i, :len(x)].view(np.uint32), x.view(np.uint32)), i
        assert not rows[i, len(x):].any()
        assert np.array_equal(rbf[i, :len(x)], torch.from_numpy(x).bfloat16().float().numpy())
        assert np.array_equal(rh[i, :len(x)], x.astype(np.float16).astype(np.float32))


@pytest.mark.parametrize("ion_custom", [0, 1])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_long_rows_search(tiny_engine, oracle, precision, ion_custom):
    """Search at 0.02 Da: 32-bit sorted ion lists, tiles gathered from L2,
    list-based FP32 rescoring.  ion_custom bins the ions at 0.02 Da too (the
    new switch); 0 keeps the reference's mono-width ion bins."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = _highres_subset(sp, 16)
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=10, bw=HIGHRES, custom_bw=True,
                        ion_bw=HIGHRES if ion_custom else 0.0)
    p = hfx_gb300.default_params(top_n=10, bin_width=HIGHRES, custom_bin_width=1, batch_mode=1,
                                 precision=precision, rescore_k=32, ion_bins_custom=ion_custom)
    res = eng.search(sub, p)
    _compare(res, ref, f"0.02 Da precision={precision} ion_custom={ion_custom}")
    if precision:
        p.group_size = 16
        res = eng.search(sub, p)
        _compare(res, ref, f"0.02 Da G=16 precision={precision} ion_custom={ion_custom}")
    if ion_custom:
        assert (ref[0][:, 0] > 0).mean() > 0.9   # the source peptides score


def test_custom_ion_width_needs_long_rows(tiny_engine):
    import hfx_gb300
    eng, prot, sp = tiny_engine
    with pytest.raises(hfx_gb300.HfxError):
        eng.search(sp.subset(np.arange(4)), hfx_gb300.default_params(ion_bins_custom=1, batch_mode=1))


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_eager(full_engine, oracle, precision):
    """use_graph: the first call plans and captures, later calls replay the
    CUDA graph.  A second batch of the same shape replays the same graph (or
    re-plans if it needs more work items); every result equals the eager
    search's."""
    import hfx_gb300
    eng, prot, sp = full_engine
    a = sp.subset(np.arange(0, 120))
    b = sp.subset(np.arange(120, 240))
    pe = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=precision)
    pg = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=precision, use_graph=1)
    ra, rb = eng.search(a, pe), eng.search(b, pe)
    for rep in range(3):
        for sub, ref in ((a, ra), (b, rb)):
            res = eng.search(sub, pg)
            assert np.array_equal(res.key, ref.key), rep
            assert np.array_equal(res.score.view(np.uint32), ref.score.view(np.uint32)), rep
            assert np.array_equal(res.ncand, ref.ncand), rep
    # the graph path is still the oracle's search
    _compare(eng.search(a, pg), oracle.search(*_oracle_db(oracle, eng, prot), a, topn=10), "graph")


@pytest.mark.parametrize("mixed", [False, True])
def test_graph_replay_long_rows(tiny_engine, mixed):
    """use_graph at 0.02 Da (32-bit lists, tiles read from L2), with and
    without wide windows: replays equal the eager search."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = _highres_subset(sp, 24)
    kw = dict(top_n=10, bin_width=HIGHRES, custom_bin_width=1, batch_mode=1, precision=1, rescore_k=32,
              ion_bins_custom=1)
    if mixed:
        sub.tol[:] = -10.0
        sub.tol[::4] = 500.0
        kw["tol_ppm"] = 2
    ref = eng.search(sub, hfx_gb300.default_params(**kw))
    pg = hfx_gb300.default_params(use_graph=1, **kw)
    for rep in range(3):
        res = eng.search(sub, pg)
        assert np.array_equal(res.key, ref.key), rep
        assert np.array_equal(res.score.view(np.uint32), ref.score.view(np.uint32)), rep


def test_graph_replay_skips_rows_beyond_max_len(full_engine, oracle):
    """Spectra whose rows exceed max_len score nothing in eager searches;
    graph replays treat them the same way (no error)."""
    import hfx_gb300
    eng, prot, sp = full_engine
    sub = sp.subset(np.arange(0, 64))
    lens = [len(oracle.preprocess(sub.mz[sub.off[i]:sub.off[i + 1]], sub.it[sub.off[i]:sub.off[i + 1]], sub.pcr[i],
                                  sub.z[i])) for i in range(len(sub))]
    cut = int(np.median(lens))
    kw = dict(top_n=10, batch_mode=1, precision=1, max_len=cut)
    ref = eng.search(sub, hfx_gb300.default_params(**kw))
    assert (ref.ncand == 0).sum() > 5 and (ref.ncand > 0).sum() > 5
    pg = hfx_gb300.default_params(use_graph=1, **kw)
    for rep in range(3):
        res = eng.search(sub, pg)
        assert np.array_equal(res.key, ref.key), rep
        assert np.array_equal(res.ncand, ref.ncand), rep


def test_autotune_picks_a_valid_shape(full_engine):
    """hfx_autotune times the batched search over group and work-item sizes
    and writes the fastest into the parameters; the tuned search returns the
    same results as the default one."""
    import hfx_gb300
    eng, prot, sp = full_engine
    sub = sp.subset(np.arange(120))
    p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1)
    ref = eng.search(sub, p)
    dev = _dev(sub)
    out = dict(score=torch.empty((120, 10), dtype=torch.float32, device="cuda"),
               key=torch.empty((120, 10), dtype=torch.int64, device="cuda"),
               pep=torch.empty((120, 10), dtype=torch.int32, device="cuda"),
               ncand=torch.empty(120, dtype=torch.int64, device="cuda"))
    ms = eng.autotune(dev, p, out, reps=1)
    assert ms > 0 and p.group_size in (4, 8, 16) and p.chunk in (1024, 2048, 4096, 8192, 16384)
    res = eng.search(sub, p)
    assert np.array_equal(res.key, ref.key)
    assert np.array_equal(res.score.view(np.uint32), ref.score.view(np.uint32))


def test_autotune_choice_persisted(full_engine, tmp_path, monkeypatch):
    """With HFX_AUTOTUNE_FILE set, hfx_autotune writes its choice for the
    batch shape once and later calls read it back instead of timing: the same
    group and work-item sizes, one line in the file, the same results."""
    import hfx_gb300
    eng, prot, sp = full_engine
    path = tmp_path / "autotune.tsv"
    monkeypatch.setenv("HFX_AUTOTUNE_FILE", str(path))
    sub = sp.subset(np.arange(64))
    dev = _dev(sub)

    def out():
        return dict(score=torch.empty((64, 10), dtype=torch.float32, device="cuda"),
                    key=torch.empty((64, 10), dtype=torch.int64, device="cuda"),
                    pep=torch.empty((64, 10), dtype=torch.int32, device="cuda"),
                    ncand=torch.empty(64, dtype=torch.int64, device="cuda"))
    p1 = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1)
    o1 = out()
    ms1 = eng.autotune(dev, p1, o1, reps=1)
    lines = path.read_text().splitlines()
    assert len(lines) == 1 and lines[0].split("\t")[1:3] == [str(p1.group_size), str(p1.chunk)]
    p2 = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1)
    o2 = out()
    ms2 = eng.autotune(dev, p2, o2, reps=1)
    assert (p2.group_size, p2.chunk) == (p1.group_size, p1.chunk) and abs(ms2 - ms1) < 1e-3
    assert len(path.read_text().splitlines()) == 1
    assert torch.equal(o1["key"], o2["key"]) and torch.equal(o1["score"], o2["score"])
    # another batch shape is tuned and appended
    p3 = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=0)
    eng.autotune(dev, p3, out(), reps=1)
    assert len(path.read_text().splitlines()) == 2


@pytest.mark.parametrize("G", [4, 8])
def test_keep_64_candidates(full_engine, oracle, G):
    """Up to 64 candidates kept per spectrum for FP32 rescoring (two member
    lists of 32 per lane pair, 64-entry item merges): the top-32 after
    rescoring equals the oracle's, and so does the top-10 with 50 kept."""
    import hfx_gb300
    eng, prot, sp = full_engine
    sub = sp.subset(np.arange(96))
    for top_n, keep in ((32, 64), (10, 50)):
        ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=top_n)
        p = hfx_gb300.default_params(top_n=top_n, batch_mode=1, precision=1, rescore_k=keep, group_size=G,
                                     chunk=512)
        _compare(eng.search(sub, p), ref, f"keep {keep} top {top_n} G={G}")


def test_keep_50_at_002_da(tiny_engine, oracle):
    """The 0.02 Da configuration's top-50 rescoring (long rows, 32-bit
    lists, tiles read from L2)."""
    import hfx_gb300
    eng, prot, sp = tiny_engine
    sub = _highres_subset(sp, 16)
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=10, bw=HIGHRES, custom_bw=True, ion_bw=HIGHRES)
    for prec in (1, 2):
        p = hfx_gb300.default_params(top_n=10, bin_width=HIGHRES, custom_bin_width=1, batch_mode=1,
                                     precision=prec, rescore_k=50, ion_bins_custom=1)
        _compare(eng.search(sub, p), ref, f"0.02 Da keep 50 precision {prec}")


def test_keep_more_than_32_capped_with_mods(gpulib, tiny, oracle):
    """With modification search the kept candidates stay at most 32 (the
    modified scorer's lists hold 32): a larger rescore_k is capped, and the
    results still equal the oracle's."""
    import hfx_gb300
    prot, sp, cfg = tiny
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
        eng.set_mods("MSTY", [15.995, 79.966, 79.966, 79.966], 4, False)
        sub = sp.subset(np.arange(16))
        db = _oracle_db(oracle, eng, prot, b"MSTY")
        ref = oracle.search(*db, sub, topn=10, ma=b"MSTY", ma_mass=[15.995, 79.966, 79.966, 79.966], max_ma=4)
        p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1, rescore_k=64)
        _compare(eng.search(sub, p), ref, "mods keep capped")
    finally:
        eng.close()


def test_graph_replay_with_fallen_back_group_size(gpulib, oracle):
    """A requested group size of 16 falls back to 8 when more than 32
    candidates are kept for rescoring; the CUDA graph's tiles must be sized
    for the groups of 8 actually planned (twice as many), so a replayed
    search of a large batch still equals the oracle's."""
    import hfx_gb300
    prot, sp, _ = synth.workload("tiny", n_spectra=1000)
    eng = _engine(prot)
    try:
        ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10)
        p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1, rescore_k=50, group_size=16, use_graph=1)
        for rep in range(3):  # sizing, capture, replay
            _compare(eng.search(sp, p), ref, f"graph replay {rep}")
    finally:
        eng.close()
