"""CPU tests of the oracle: known-answer tests from the reference's own
in-source checks and golden vectors produced by the reference's code."""
import math

import numpy as np
import pytest

from hfx_gb300 import synth


def test_choose_matches_reference(oracle, golden):
    g = golden("ref_combinatorics.npz")["choose"]
    for n in range(g.shape[0]):
        for k in range(g.shape[1]):
            assert oracle.choose(n, k) == g[n, k], (n, k)


def test_choose_table_is_binomial(oracle):
    # combinatorics.h:13-57 tabulates C(n<=42, k<=11)
    for n in range(43):
        for k in range(12):
            assert oracle.choose(n, k) == (math.comb(n, k) if k <= n else 0)


def test_unrank_matches_reference(oracle, golden):
    g = golden("ref_combinatorics.npz")
    for (n, k, rank), row in zip(g["unrank_keys"], g["unrank_rows"]):
        got = oracle.unrank_comb(int(n), int(k), int(rank))
        assert list(got) == list(row[:k]), (n, k, rank)


def test_unrank_dual_rank_quirk(oracle):
    """combinatorics.h:109-131 maps ranks above total/2 through the dual
    combination; that is not a bijection for every (n, k): C(5,2) yields 9
    distinct combinations out of 10 (one isoform twice, one never).  The
    oracle reproduces the reference exactly (test above); this records it."""
    distinct = {}
    for n in range(1, 12):
        for k in range(1, n + 1):
            seen = {tuple(sorted(oracle.unrank_comb(n, k, r))) for r in range(math.comb(n, k))}
            assert all(0 <= v < n for s in seen for v in s)
            distinct[(n, k)] = len(seen)
    assert distinct[(5, 2)] == 9
    assert distinct[(4, 3)] == 4 and distinct[(2, 1)] == 2   # the worked example is intact
    assert all(distinct[(n, 1)] == n for n in range(1, 12))


def test_worked_example_isoform_count(oracle):
    # gen_mod_pep.cu:25-27: 4 A's and 2 R's, mod 3A + 1R -> C(4,3)*C(2,1) = 8
    pep = b"AIGIRRAOQAANK"    # A x4, R x2 before the last residue
    ions = oracle.pack_ions(np.frombuffer(pep, np.uint8), b"AR")
    n, _, _ = oracle.mod_isoform(ions, 0, len(pep) - 1, b"AR", [3, 1])
    assert n == 8
    rows = set()
    for rk in range(8):
        _, un, md = oracle.mod_isoform(ions, 0, len(pep) - 1, b"AR", [3, 1], rank=rk, per_type=True)
        assert md.sum() == 4
        rows.add(tuple(un))
    assert len(rows) == 8


def test_prepare_ions_matches_reference(oracle, golden):
    g = golden("ref_prepare_ions.npz")
    for key in g.files:
        if not key.startswith("packed_"):
            continue
        ma = key[len("packed_"):]
        ma = b"" if ma == "none" else ma.encode()
        assert np.array_equal(oracle.pack_ions(g["seq"], ma), g[key]), key


def test_mod_combo_table(oracle):
    counts, sums, deltas = oracle.mod_combos([15.995, 79.966, 79.966, 79.966], 4)
    assert counts.shape == (34, 4)          # sum < 4 (strict), Fragment.hs:275
    assert (sums == counts.sum(1)).all() and sums.max() == 3 and sums.min() == 1
    # lexicographic with acid 0 most significant
    keys = [tuple(c) for c in counts]
    assert keys == sorted(keys)
    counts1, _, _ = oracle.mod_combos([-17.0], 2)
    assert counts1.tolist() == [[1]]        # hfx.params: mod_Q, max-modable-acids 2


def _rebuild_reference_pipeline(oracle, g):
    """Recompute the reference's stage (b)/(e) outputs with the oracle."""
    r, tc, tn, idx, ions = g["r"], g["tc"], g["tn"], g["idx_sorted"], g["ions"]
    masses, eps = g["masses"], np.float32(g["eps"])
    rs = r[idx]
    lo = (masses - eps).astype(np.float32)
    hi = (masses + eps).astype(np.float32)
    b, e = oracle.windows(rs, lo, hi)
    out = dict(plain_begin=b, plain_end=e)
    ma = bytes(g["ma"])
    counts, sums, deltas = oracle.mod_combos(g["ma_mass"], int(g["max_ma"]))
    nm = len(deltas)
    mb, me = [], []
    valid = []
    mpeps = []
    for s in range(len(masses)):
        mlo = (lo[s] - deltas).astype(np.float32)
        mhi = (hi[s] - deltas).astype(np.float32)
        bb, ee = oracle.windows(rs, mlo, mhi)
        mb.append(bb)
        me.append(ee)
        for m in range(nm):
            for q in range(bb[m], ee[m]):
                p = int(idx[q])
                niso, _, _ = oracle.mod_isoform(ions, int(tc[p]), int(tn[p]), ma, counts[m])
                if niso == 0:
                    continue
                valid.append((p, m))
                for rk in range(niso):
                    _, un, _ = oracle.mod_isoform(ions, int(tc[p]), int(tn[p]), ma, counts[m], rank=rk)
                    mpeps.append((p, m, rk, tuple(un)))
    out["mod_begin"] = np.concatenate(mb)
    out["mod_end"] = np.concatenate(me)
    return out, valid, mpeps


def test_enumeration_matches_reference(oracle, golden):
    """Stages (b) and (e) against the reference's own Thrust code."""
    g = golden("ref_enumeration.npz")
    # the oracle digest and sort reproduce the fixture's database
    r, tc, tn = oracle.digest(g["seq"], g["seg"], g["mt"], rule=1, missed=1, min_mass=400.0, max_mass=4000.0)
    assert np.array_equal(r, g["r"]) and np.array_equal(tc, g["tc"]) and np.array_equal(tn, g["tn"])
    assert np.array_equal(oracle.sort_idx(r), g["idx_sorted"])
    assert np.array_equal(oracle.pack_ions(g["seq"], bytes(g["ma"])), g["ions"])
    out, valid, mpeps = _rebuild_reference_pipeline(oracle, g)
    for k in ("plain_begin", "plain_end", "mod_begin", "mod_end"):
        assert np.array_equal(out[k], g[k]), k
    assert np.array_equal(g["plain_num"], g["plain_end"] - g["plain_begin"])
    vp = np.array([v[0] for v in valid], np.uint32)
    vm = np.array([v[1] for v in valid], np.uint32)
    assert np.array_equal(vp, g["valid_pep"]) and np.array_equal(vm, g["valid_mod"])
    assert len(mpeps) == len(g["mpep_pep"])
    assert np.array_equal(np.array([m[0] for m in mpeps], np.uint32), g["mpep_pep"])
    assert np.array_equal(np.array([m[1] for m in mpeps], np.uint32), g["mpep_mod"])
    assert np.array_equal(np.array([m[2] for m in mpeps], np.uint32), g["mpep_rank"])
    un = np.concatenate([np.array(m[3], np.uint32) for m in mpeps])
    assert np.array_equal(un, g["mpep_unrank"])


def test_window_invariants(oracle, golden):
    # filter_by_mod.cu:93-131 (_DEBUG self-check)
    g = golden("ref_enumeration.npz")
    rs = g["r"][g["idx_sorted"]]
    lo = np.sort(np.random.Generator(np.random.PCG64(3)).uniform(300, 3000, 200)).astype(np.float32)
    hi = (lo + 2.0).astype(np.float32)
    b, e = oracle.windows(rs, lo, hi)
    for i in range(len(lo)):
        assert b[i] <= e[i]
        if b[i] < e[i]:
            assert lo[i] <= rs[b[i]] and rs[e[i] - 1] <= hi[i]
        if b[i] > 0:
            assert rs[b[i] - 1] < lo[i]
        if e[i] < len(rs):
            assert hi[i] < rs[e[i]]


def _preprocess_py(mz, it, pcr, z, bw=np.float32(1.0005079), remove=True):
    """Step-by-step numpy float32 transcription of Correlation.hs:37-109."""
    f = np.float32
    pcr, z = f(pcr), f(z)
    mzcut = f(f(50) + f(pcr * z))
    mzlim = f(math.trunc(float(f(mz[-1] / f(10)))) * 10)
    cutoff = mzcut if mzcut <= mzlim else mzlim
    n = 75 + math.ceil(float(cutoff))
    e = np.zeros(n, np.float32)
    for x, y in zip(mz, it):
        keep = x <= cutoff and (x <= f(pcr - f(15)) or f(pcr + f(15)) <= x) if remove else x <= cutoff
        if keep:
            b = int(np.rint(f(x / bw)))
            v = np.sqrt(f(y))
            if e[b] <= v:
                e[b] = v
    sel = (n - 75) // 10
    rmax = np.zeros(11, np.float32)
    for i in range(n):
        g = min(10, i // sel)
        rmax[g] = e[i] if rmax[g] <= e[i] else rmax[g]
    a = np.zeros(n, np.float32)
    for i in range(n):
        m = rmax[min(10, i // sel)]
        a[i] = f(f(50) * f(e[i] / m)) if (m > f(1e-6) and i < sel * 10) else f(0)
    x = np.zeros(n, np.float32)
    for i in range(n):
        lo = max(0, i - 75)
        s = f(0)
        for j in range(lo, min(n, lo + 151)):
            s = f(s + a[j])
        x[i] = f(a[i] - f(s / f(150)))
    return x


def test_preprocess_two_restatements_agree(oracle, tiny):
    _, sp, _ = tiny
    for i in range(5):
        a, b = sp.off[i], sp.off[i + 1]
        x1 = oracle.preprocess(sp.mz[a:b], sp.it[a:b], sp.pcr[i], sp.z[i])
        x2 = _preprocess_py(sp.mz[a:b], sp.it[a:b], sp.pcr[i], sp.z[i])
        assert np.array_equal(x1.view(np.uint32), x2.view(np.uint32))


def test_preprocess_edge_cases(oracle):
    # i < 75 uses bins 0..150 (take 151 . drop (i-75)); divide by 150
    mz = np.array([100.0, 140.0, 900.0, 1200.0], np.float32)
    it = np.array([4.0, 9.0, 16.0, 1.0], np.float32)
    x = oracle.preprocess(mz, it, 600.0, 2.0, remove_pcr=False)
    assert len(x) == 75 + 1200
    x2 = _preprocess_py(mz, it, 600.0, 2.0, remove=False)
    assert np.array_equal(x, x2)
    assert oracle.preprocess(np.zeros(0, np.float32), np.zeros(0, np.float32), 500.0, 2.0) is None


def _ion_bins_py(seq_masses, residual, charges, length):
    """Serial restatement of ion_series.cu:59-232 (Hillis-Steele ladder)."""
    f = np.float32
    H2O, NH3, CO, H, BW = f(18.01056), f(17.02655), f(27.9949), f(1.0078246), f(1.0005079)
    lv = {}

    def add(x, l):
        if 0 <= x < length:
            lv[x] = max(lv.get(x, 0), l)

    def binmz(m):
        r = np.rint(f(m / BW))
        return 0 if not r > 0 else int(r)

    carry = f(0)
    n = len(seq_masses)
    for base in range(0, n, 32):
        v = [f(m) for m in seq_masses[base:base + 32]]
        v[0] = f(v[0] + carry)
        d = 1
        while d < 32:
            v = [f(v[l] + v[l - d]) if l >= d else v[l] for l in range(len(v))]
            d *= 2
        carry = v[-1]
        for b in v:
            y = f(residual - b)
            for c in range(1, charges + 1):
                cf = f(c)
                hc = f(H * cf)
                add(binmz(f(f(f(b - CO) + hc) / cf)), 1)
                m = f(f(b + hc) / cf)
                x = binmz(m)
                add(x, 3); add(x + 1, 2); add(x - 1, 2)
                add(binmz(f(m - f(H2O / cf))), 1)
                add(binmz(f(m - f(NH3 / cf))), 1)
                m = f(f(f(y + H2O) + hc) / cf)
                x = binmz(m)
                add(x, 3); add(x + 1, 2); add(x - 1, 2)
                add(binmz(f(m - f(NH3 / cf))), 1)
    ks = sorted(lv)
    return np.array(ks, np.uint32), np.array([lv[k] for k in ks], np.uint8)


def test_ion_bins_two_restatements_agree(oracle, tiny):
    prot, _, _ = tiny
    mt = oracle.mass_table(True, synth.static_mods())
    r, tc, tn = oracle.digest(prot.seq, prot.seg, mt, rule=1, missed=1)
    ions = oracle.pack_ions(prot.seq)
    rng = np.random.Generator(np.random.PCG64(5))
    long_ = np.nonzero(tn - tc > 33)[0][:3]
    for p in list(rng.integers(0, len(r), 30)) + list(long_):
        masses = [mt[c - 65] for c in prot.seq[tc[p]:tn[p]]]
        for ch in (1, 2, 3, 4):
            b1, l1 = oracle.ion_bins(ions, mt, tc[p], tn[p], r[p], ch, 3000)
            b2, l2 = _ion_bins_py(masses, r[p], ch, 3000)
            assert np.array_equal(b1, b2) and np.array_equal(l1, l2), (p, ch)


def test_score_canonical_order(oracle):
    rng = np.random.Generator(np.random.PCG64(9))
    x = rng.normal(0, 10, 2000).astype(np.float32)
    bins = np.sort(rng.choice(2000, 300, replace=False)).astype(np.uint32)
    lvl = rng.integers(1, 4, 300).astype(np.uint8)
    w = np.array([0, 10, 25, 50], np.float32)[lvl]
    acc = np.zeros(32, np.float32)
    for i in range(300):
        acc[i % 32] = np.float32(np.float64(w[i]) * np.float64(x[bins[i]]) + np.float64(acc[i % 32]))
    for off in (16, 8, 4, 2, 1):
        acc = (acc + acc[np.arange(32) ^ off]).astype(np.float32)
    assert np.float32(oracle.score32(bins, lvl, x)) == acc[0]
    s64 = oracle.score64(bins, lvl, x.astype(np.float64))
    assert abs(s64 - float((w.astype(np.float64) * x[bins]).sum())) < 1e-9 * max(1, abs(s64)) + 1e-9


def test_four_candidates_per_warp_keep_the_canonical_order(oracle):
    """The FP32 scorers' four-candidates-per-warp form: 8 lanes per candidate,
    entry k of every round of 32 into the lane's partial set k, the sets
    added as (s0 + s2) + (s1 + s3) in the lane, then XOR offsets 4, 2, 1
    within the 8 lanes.  The same float32 additions as the canonical 32
    partial sums with offsets 16, 8, 4, 2, 1, so the same bits (and the
    oracle's score)."""
    rng = np.random.Generator(np.random.PCG64(11))
    for n in (1, 7, 31, 32, 33, 95, 300, 1001):
        x = rng.normal(0, 10, 4000).astype(np.float32)
        bins = np.sort(rng.choice(4000, n, replace=False)).astype(np.uint32)
        lvl = rng.integers(1, 4, n).astype(np.uint8)
        w = np.array([0, 10, 25, 50], np.float32)[lvl]
        prod = lambda i, a: np.float32(np.float64(w[i]) * np.float64(x[bins[i]]) + np.float64(a))
        # canonical: lane i % 32 of one warp
        acc = np.zeros(32, np.float32)
        for i in range(n):
            acc[i % 32] = prod(i, acc[i % 32])
        for off in (16, 8, 4, 2, 1):
            acc = (acc + acc[np.arange(32) ^ off]).astype(np.float32)
        # four sets per lane, 8 lanes (entry i0 + 8 k + l of round i0 -> set k of lane l)
        sets = np.zeros((8, 4), np.float32)
        for i in range(n):
            sets[i % 8, (i % 32) // 8] = prod(i, sets[i % 8, (i % 32) // 8])
        lane = ((sets[:, 0] + sets[:, 2]).astype(np.float32) + (sets[:, 1] + sets[:, 3]).astype(np.float32))
        lane = lane.astype(np.float32)
        for off in (4, 2, 1):
            lane = (lane + lane[np.arange(8) ^ off]).astype(np.float32)
        assert lane[0].view(np.uint32) == acc[0].view(np.uint32), n
        assert np.float32(oracle.score32(bins, lvl, x)).view(np.uint32) == lane[0].view(np.uint32), n


def test_incremental_level_lists_equal_the_full_sort():
    """The long-row list generator's level recurrence: the level-z list is
    the level-(z-1) list merged with the charge-z keys (bin << 2 | level),
    each bin keeping its highest level -- the same list as sorting the keys
    of every charge <= z at once and keeping each bin's last key."""
    rng = np.random.Generator(np.random.PCG64(13))

    def keep_highest(keys):
        keys = np.sort(keys)
        last = np.ones(len(keys), bool)
        last[:-1] = (keys[1:] >> 2) != (keys[:-1] >> 2)
        return keys[last]

    for _ in range(200):
        nk = int(rng.integers(1, 400))
        span = int(rng.integers(50, 5000))
        charges = [(rng.integers(0, span, nk).astype(np.uint32) << 2) | rng.integers(1, 4, nk).astype(np.uint32)
                   for _ in range(4)]
        prev = np.zeros(0, np.uint32)
        for z in range(1, 5):
            inc = keep_highest(np.concatenate([prev, charges[z - 1]]))
            full = keep_highest(np.concatenate(charges[:z]))
            assert np.array_equal(inc, full), (nk, span, z)
            prev = inc


def test_ion_charges(oracle):
    # Search.hs:182 round (max 1 (z-1)); plain kernel 1..4 only
    assert [oracle.ion_charges(z) for z in (1, 2, 3, 4, 5, 6)] == [1, 1, 2, 3, 4, 0]
    assert [oracle.ion_charges(z, True) for z in (1, 5, 11, 12)] == [1, 4, 4, 0]


def test_search_finds_source_peptides(oracle, tiny):
    prot, sp, cfg = tiny
    mt = oracle.mass_table(True, synth.static_mods())
    d = {k: v for k, v in synth.DIGEST.items() if k != "mono"}
    r, tc, tn = oracle.digest(prot.seq, prot.seg, mt, **d)
    idx = oracle.sort_idx(r)
    ions = oracle.pack_ions(prot.seq)
    sc, _, key, pep, nc = oracle.search(ions, mt, r, tc, tn, idx, sp, topn=10)
    assert (nc > 0).all()
    assert np.all(np.diff(sc, axis=1) <= 0)
    hits = sum(prot.seq[tc[pep[i, 0]]:tn[pep[i, 0]]].tobytes().decode() in sp.source[i] for i in range(len(sp)))
    assert hits >= 90
