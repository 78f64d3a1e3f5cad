"""GPU parity of stage (e), variable-modification search: the combination
table, the isoform enumeration (counts, unranked positions, modified
residues) and the full search with modified candidates, against the oracle
on the same seeded inputs.  Everything is bit-exact: candidate counts, keys
(combination, mass-order position, isoform rank), FP32 scores, peptides."""
import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MA = b"MSTY"
MA_MASS = [15.995, 79.966, 79.966, 79.966]   # Met oxidation, Ser/Thr/Tyr phosphorylation


def _engine(prot, max_ma=4, per_type=False):
    import hfx_gb300
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    eng.set_mods(MA.decode(), MA_MASS, max_ma, per_type)
    return eng


def _oracle_db(oracle, eng, prot):
    r, tc, tn, idx, mt = eng.db_export()
    return oracle.pack_ions(prot.seq, MA), mt, r, tc, tn, idx


def _compare(res, ref, label):
    sc, _, key, pep, nc = ref
    assert np.array_equal(res.ncand, nc), label
    assert np.array_equal(res.key, key), label
    assert np.array_equal(res.score.view(np.uint32), sc.view(np.uint32)), label
    assert np.array_equal(res.pep, pep), label


@pytest.fixture(scope="module")
def mods_full(gpulib):
    prot = synth.proteins(20000, seed=1)
    sp = synth.spectra(prot, 96, seed=101, charge_p={1: 0.05, 2: 0.5, 3: 0.35, 4: 0.10}, npeaks=(50, 400))
    eng = _engine(prot)
    yield eng, prot, sp
    eng.close()


@pytest.fixture(scope="module")
def mods_tiny(gpulib, tiny):
    prot, sp, cfg = tiny
    eng = _engine(prot)
    yield eng, prot, sp
    eng.close()


def test_mod_table_matches_oracle(mods_tiny, oracle):
    eng, prot, sp = mods_tiny
    n, counts, deltas = eng.mod_table()
    oc, _, od = oracle.mod_combos(MA_MASS, 4)
    assert n == len(oc) == 34
    assert np.array_equal(counts[: n * 4].reshape(n, 4), oc)
    assert np.array_equal(deltas[:n].view(np.uint32), od.view(np.uint32))


@pytest.mark.parametrize("per_type", [False, True])
def test_mod_isoforms_exact(gpulib, tiny, oracle, per_type):
    """Per (peptide, combination, rank): the isoform count, the unranked
    occurrence indices and the modified residues equal the oracle's."""
    prot, sp, cfg = tiny
    eng = _engine(prot, per_type=per_type)
    try:
        ions, mt, r, tc, tn, idx = _oracle_db(oracle, eng, prot)
        n, counts, _ = eng.mod_table()
        counts = counts[: n * 4].reshape(n, 4)
        rng = np.random.default_rng(7)
        pos_l, mu_l, rank_l, ref = [], [], [], []
        # candidates rich in S/T/Y and M, every combination, first/last/random ranks
        cand = rng.choice(len(r), 400, replace=False)
        for q in cand:
            pi = idx[q]
            for mu in rng.choice(n, 6, replace=False):
                niso, _, _ = oracle.mod_isoform(ions, int(tc[pi]), int(tn[pi]), MA, counts[mu], per_type=per_type)
                ranks = {0, max(0, niso - 1), int(rng.integers(0, max(1, niso)))} if niso else {0}
                for rk in sorted(ranks):
                    pos_l.append(q)
                    mu_l.append(mu)
                    rank_l.append(rk)
                    ref.append((niso,) + oracle.mod_isoform(ions, int(tc[pi]), int(tn[pi]), MA, counts[mu], rank=rk,
                                                            per_type=per_type)[1:] if niso else (0, None, None))
        d = torch.device("cuda:0")
        cap = 64
        m = len(pos_l)
        pos = torch.tensor(np.array(pos_l, np.uint32).view(np.int32), device=d)
        mu_t = torch.tensor(np.array(mu_l, np.int32), device=d)
        rank = torch.tensor(np.array(rank_l, np.uint32).view(np.int32), device=d)
        cnt = torch.zeros(m, dtype=torch.int32, device=d)
        unr = torch.full((m, 8), -1, dtype=torch.int32, device=d)
        modded = torch.zeros((m, cap), dtype=torch.uint8, device=d)
        eng.mod_isoforms(pos, mu_t, rank, cap, cnt, unr, modded)
        cnt = cnt.cpu().numpy().view(np.uint32)
        unr = unr.cpu().numpy().view(np.uint32)
        modded = modded.cpu().numpy()
        nonzero = 0
        for i, (niso, un, md) in enumerate(ref):
            assert cnt[i] == niso, i
            if niso == 0:
                continue
            nonzero += 1
            k = int(counts[mu_l[i]].sum())
            assert np.array_equal(unr[i, :k], un), (i, unr[i], un)
            L = len(md)
            assert np.array_equal(modded[i, :L], md), i
        assert nonzero > 100
    finally:
        eng.close()


def test_search_mods_tiny(mods_tiny, oracle):
    import hfx_gb300
    eng, prot, sp = mods_tiny
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    assert (ref[2] >> np.uint64(63)).any()           # modified matches reach the top-10
    for mode in (0, 1, 2):
        res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=mode))
        _compare(res, ref, f"tiny mods mode={mode}")


@pytest.mark.parametrize("G", [1, 4, 8])
@pytest.mark.parametrize("mode", [1, 2])
def test_search_mods_full(mods_full, oracle, G, mode):
    import hfx_gb300
    eng, prot, sp = mods_full
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=mode, group_size=G, chunk=512))
    _compare(res, ref, f"full mods G={G} mode={mode}")


@pytest.mark.parametrize("precision", [0, 1])
def test_search_mods_graph_replay(mods_full, oracle, precision):
    """The isoform lists under CUDA-graph replay: sizing run, capture and
    replays (record and list capacities from the sizing run) all equal the
    oracle."""
    import hfx_gb300
    eng, prot, sp = mods_full
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=precision, rescore_k=32 if precision else 0,
                                 use_graph=1)
    for rep in range(3):
        _compare(eng.search(sp, p), ref, f"mods graph replay {rep} precision {precision}")


def test_mod_counters_account_for_every_pair(mods_full, oracle):
    """With profiling on, the pairs scored by the unmodified list scorer and
    by the isoform-list scorer add up to the oracle's candidate counts; the
    isoform lists are timed as their own stage."""
    import hfx_gb300
    eng, prot, sp = mods_full
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    eng.set_profiling(True)
    try:
        eng.stage_stats(reset=True)
        eng.counters(reset=True)
        eng.mod_counters(reset=True)
        res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=1))
        st = eng.stage_stats(reset=True)
        plain, mods = eng.counters(reset=True), eng.mod_counters(reset=True)
    finally:
        eng.set_profiling(False)
    _compare(res, ref, "mods with profiling")
    assert plain["pairs"] + mods["pairs"] == int(ref[4].sum())
    assert mods["pairs"] > 0 and mods["isoforms"] > 0 and mods["list_entries"] > 0
    assert mods["entries_streamed"] > 0 and mods["tile_bytes"] > 0 and mods["residues_read"] > 0
    assert st["mod_lists"][1] > 0 and st["mods"][1] == 1


@pytest.mark.parametrize("precision", [1, 2])
def test_search_mods_lowp_rescore(mods_full, oracle, precision):
    """BF16 / FP16 rows choose the kept candidates (modified included), FP32
    rescoring restores the oracle's FP32 top-10."""
    import hfx_gb300
    eng, prot, sp = mods_full
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sp, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=1, precision=precision, rescore_k=32))
    _compare(res, ref, f"mods precision {precision}")


def test_group16_refused_with_mods(mods_tiny):
    import hfx_gb300
    eng, prot, sp = mods_tiny
    with pytest.raises(hfx_gb300.HfxError):
        eng.search(sp.subset(np.arange(8)), hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1,
                                                                     group_size=16))


def test_search_mods_only_and_per_type(gpulib, tiny, oracle):
    """Modified candidates alone (no unmodified search) and the per-acid
    i-th counter."""
    import hfx_gb300
    prot, sp, cfg = tiny
    for per_type in (False, True):
        eng = _engine(prot, max_ma=3, per_type=per_type)
        try:
            db = _oracle_db(oracle, eng, prot)
            ref = oracle.search(*db, sp, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=3, per_type=per_type, plain=False)
            res = eng.search(sp, hfx_gb300.default_params(top_n=10, batch_mode=1, search_plain=0))
            _compare(res, ref, f"mods only per_type={per_type}")
            assert (res.key[res.key != np.iinfo(np.uint64).max] >> np.uint64(63) == 1).all()
        finally:
            eng.close()


def test_search_mods_edge_charges(mods_tiny, oracle):
    """Charge 7 (no unmodified ions, 4 modified charges) and charge 12 (no
    ions either way: every candidate scores 0) next to ordinary spectra."""
    import hfx_gb300
    eng, prot, sp = mods_tiny
    sub = sp.subset(np.arange(8))
    sub.z[1] = 7.0
    sub.z[2] = 12.0
    sub.tol[3] = 1e-7
    ref = oracle.search(*_oracle_db(oracle, eng, prot), sub, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    for mode in (1, 2):
        res = eng.search(sub, hfx_gb300.default_params(top_n=10, batch_mode=mode))
        _compare(res, ref, f"mods edges mode={mode}")
    assert (res.score[2][res.key[2] != np.iinfo(np.uint64).max] == 0).all()


@pytest.mark.parametrize("precision,graph", [(0, 0), (1, 0), (1, 1), (0, 1)])
def test_search_mods_empty_and_one_peak(mods_tiny, oracle, precision, graph):
    """The isoform-list path on an empty spectrum, a one-peak spectrum and an
    (almost) empty window, eager and replayed; then a batch with no
    candidate at all (no isoform records)."""
    import hfx_gb300
    eng, prot, sp = mods_tiny
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
    sub.tol[1] = 1e-7
    db = _oracle_db(oracle, eng, prot)
    ref = oracle.search(*db, sub, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=precision, use_graph=graph,
                                 rescore_k=32 if precision else 0)
    for rep in range(2 if graph else 1):
        _compare(eng.search(sub, p), ref, f"mods empty/one-peak precision={precision} graph={graph} rep={rep}")
    none = sp.subset(np.arange(4))
    none.z[:] = 2.0
    none.pcr[:] = 3900.0                            # above every peptide and isoform mass
    none.tol[:] = 1.0
    ref = oracle.search(*db, none, topn=10, ma=MA, ma_mass=MA_MASS, max_ma=4)
    assert int(ref[4].sum()) == 0
    for rep in range(2 if graph else 1):
        res = eng.search(none, p)
        _compare(res, ref, f"mods no candidates precision={precision} graph={graph} rep={rep}")
        assert (res.key == np.iinfo(np.uint64).max).all()


def _ref_match(prot, r, tc, tn, k, ions, counts=None, rank=None, per_type=False, oracle=None):
    """Location.hs:42-58 lookup and Fragment.hs:84-106 modifyFragment,
    transcribed independently: peptide text with flanks, (M+H)+, '*' after
    the i-th occurrence of each modified acid."""
    seq = bytes(prot.seq)
    c, n = int(tc[k]), int(tn[k])
    pi = int(np.searchsorted(prot.seg, c, side="right")) - 1
    a, b = int(prot.seg[pi]), int(prot.seg[pi + 1])
    ntake = n - c + 1 if n < len(seq) else n - c
    text = (chr(seq[c - 1]) if c > a else "-") + "." + seq[c:c + ntake].decode() + "." + \
        (chr(seq[n + 1]) if n < b - 1 else "-")
    mass = np.float32(np.float32(np.float32(r[k]) + np.float32(1.007276)) + np.float32(18.010565))
    if counts is None:
        return text, float(mass), pi
    add = np.float32(0.0)
    for i, m in enumerate(MA_MASS):
        add = np.float32(add + np.float32(np.float32(counts[i]) * np.float32(m)))
    mass = np.float32(mass + add)
    _, un, _ = oracle.mod_isoform(ions, c, n, MA, counts, rank=rank, per_type=per_type)
    star, u = set(), 0
    for i, acid in enumerate(MA.decode()):
        occ = [j for j in range(2, len(text) - 2) if text[j] == acid]
        for _ in range(int(counts[i])):
            star.add(occ[int(un[u])])
            u += 1
    out = "".join(ch + ("*" if j in star else "") for j, ch in enumerate(text))
    return out, float(mass), pi


def test_match_records(mods_tiny, oracle):
    """hfx_match_peptide: the result record of plain and modified matches."""
    import hfx_gb300
    eng, prot, sp = mods_tiny
    ions, mt, r, tc, tn, idx = _oracle_db(oracle, eng, prot)
    n, counts, _ = eng.mod_table()
    counts = counts[: n * 4].reshape(n, 4)
    res = eng.search(sp.subset(np.arange(20)), hfx_gb300.default_params(top_n=10, batch_mode=1))
    pos_of = np.empty(len(idx), np.int64)
    pos_of[idx] = np.arange(len(idx))
    seen_mod = seen_plain = 0
    for key, pep in zip(res.key.ravel(), res.pep.ravel()):
        if key == np.iinfo(np.uint64).max:
            continue
        key = int(key)
        q = int(pos_of[pep])
        text, mh, pi = eng.match(key, int(pep))
        if key >> 63:
            mu, rank = (key >> 54) & 511, key & ((1 << 27) - 1)
            assert (key >> 27) & ((1 << 27) - 1) == q
            ref = _ref_match(prot, r, tc, tn, int(pep), ions, counts[mu], rank, oracle=oracle)
            seen_mod += 1
        else:
            assert key == q
            ref = _ref_match(prot, r, tc, tn, int(pep), ions)
            seen_plain += 1
        assert (text, pi) == (ref[0], ref[2]), (text, ref)
        assert np.float32(mh) == np.float32(ref[1])
    assert seen_mod > 20 and seen_plain > 20
