"""CPU checks of the oracle's E-value restatement (Util/Statistics.hs:37-100):
the slice ranks, the shift and the 4000 floor, the histogram points and the
least-squares line, on hand-built score sets; and the full score list the
fit reads (every unmodified candidate and modified isoform)."""
import math

import numpy as np
import pytest


def test_fit_recovers_a_known_line(oracle):
    # after the shift by 1 - min, bin k (width 350) holds round(2000 * 10**(-0.4 k)) scores
    w = 350
    rng = np.random.default_rng(1)
    scores = []
    for k in range(13, 25):
        c = int(round(2000 * 10 ** (-0.4 * (k - 13))))
        lo, hi = (k - 1) * w, k * w
        scores += list(rng.uniform(lo + 1, hi - 1, max(c, 1)))
    body = np.array(scores)
    # n = 10,000: 300 scores above the 97 % cut (rank 9,700), the body right
    # below it, low scores (under the 4000 floor) filling ranks 0 .. and the
    # 30 % cut; a minimum of 1 makes the shift 0
    n = 10000
    low = np.full(n - 300 - len(body), 100.0)
    low[0] = 1.0
    scores = np.concatenate([low, body, np.full(300, 1e7)]).astype(np.float32)
    assert len(low) >= 0.3 * n
    a, b, m = oracle.evalue_fit(scores)
    assert m >= 8
    # the same points fitted by numpy
    sc = np.sort(scores.astype(np.float64))
    n = len(sc)
    hi = int(np.rint(np.float32(np.float32(0.97) * np.float32(n))))
    lo = int(np.rint(0.3 * n))
    t = (sc[lo:hi] + 1.0) - sc[0]
    t = t[t > 4000.0]
    bins, counts = np.unique(np.ceil(t / w), return_counts=True)
    x = (bins * w - w / 2) / 10000.0
    y = np.log10(counts / w)
    bb, aa = np.polyfit(x, y, 1)
    assert math.isclose(b, bb, rel_tol=1e-9) and math.isclose(a, aa, rel_tol=1e-9)
    assert b < 0


def test_slice_ranks_round_half_to_even(oracle):
    # n = 50: 0.3 n = 15 exactly, 0.97 n = 48.5 in single precision -> 48 (half to even)
    w = 350
    scores = np.arange(50, dtype=np.float32) * 1000.0
    _, _, m = oracle.evalue_fit(scores, bin_width=w)
    sc = np.sort(scores.astype(np.float64))
    t = (sc[15:48] + 1.0) - sc[0]
    assert m == len(np.unique(np.ceil(t[t > 4000.0] / w)))


def test_empty_and_degenerate(oracle):
    a, b, m = oracle.evalue_fit(np.zeros(0, np.float32))
    assert m == 0 and math.isnan(a) and math.isnan(b)
    a, b, m = oracle.evalue_fit(np.full(100, 5.0, np.float32))   # nothing clears 4000
    assert m == 0 and math.isnan(a)
    assert math.isclose(oracle.evalue(1.0, -2.0, 10000.0), 0.1, rel_tol=1e-15)


@pytest.mark.parametrize("plain", [True, False])
def test_all_scores_list_matches_top(oracle, plain):
    """hfxo_search_scores hands back every candidate's score (unmodified,
    then every modified isoform): as many as the candidate count, and its
    best ten are the search's top-10 scores."""
    from hfx_gb300 import synth
    prot, sp, cfg = synth.workload("tiny")
    ma, ma_mass = b"MSTY", [15.995, 79.966, 79.966, 79.966]
    mt = oracle.mass_table(True, synth.static_mods())
    dg = {k: v for k, v in synth.DIGEST.items() if k != "mono"}
    r, tc, tn = oracle.digest(prot.seq, prot.seg, mt, **dg)
    idx = oracle.sort_idx(r)
    sub = sp.subset(np.arange(8))
    sc, _, key, _, nc, all_sc = oracle.search(oracle.pack_ions(prot.seq, ma), mt, r, tc, tn, idx, sub, topn=10,
                                              ma=ma, ma_mass=ma_mass, max_ma=4, plain=plain, all_scores=True)
    for i in range(len(sub)):
        assert len(all_sc[i]) == nc[i]
        top = np.sort(all_sc[i])[::-1][:10]
        v = sc[i][key[i] != np.iinfo(np.uint64).max]
        assert np.array_equal(top[:len(v)].view(np.uint32), v.view(np.uint32)), i
