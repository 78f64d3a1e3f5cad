"""GPU parity of the per-stage C ABI (include/hfx_legacy.h: the reference's
algorithms.h symbols), called through ctypes with device pointers the way
the reference's Haskell host calls them.  Integer and ordering outputs are
compared exactly with the oracle or with numpy restatements of the
reference's semantics; the dense theoretical spectra use the reference's
__fdividef ion arithmetic, so they are compared row by row with the
oracle's IEEE bins: equal except where fast division moves a bin that sits
at a half-bin edge."""
import ctypes as C
import math

import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MA = b"MSTY"
MA_MASS = [15.995, 79.966, 79.966, 79.966]
U32, F32, VP = C.c_uint32, C.c_float, C.c_void_p


_KEEP = []


def _p(t):
    """Device pointer of t; t stays alive until the test ends (a temporary
    freed before the call would hand the kernel reused memory)."""
    _KEEP.append(t)
    return C.c_void_p(t.data_ptr())


@pytest.fixture(autouse=True)
def _keep_alive():
    yield
    torch.cuda.synchronize()
    _KEEP.clear()


def _dev(a, dtype=None):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    t = torch.from_numpy(a)
    if dtype is not None:
        t = t.to(dtype)
    return t.to("cuda:0")


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module")
def lib(gpulib):
    L = gpulib
    sig = {
        "prepare_ions": (None, [VP, U32, VP, U32]),
        "findIndicesInRange_f": (U32, [VP, VP, U32, F32, F32]),
        "findSpecCandsByMass": (U32, [VP, VP, VP, VP, VP, U32, VP, U32, F32]),
        "findBeginEnd_f": (U32, [VP, VP, VP, VP, VP, U32, VP, U32, F32, F32]),
        "findModablePeptides": (U32, [VP, VP, VP, VP, VP, U32, U32, VP, VP, VP, VP, VP, VP, VP, VP, U32, VP, U32]),
        "calcTotalModCands": (U32, [VP, VP, VP, VP, VP, VP, U32, U32, U32]),
        "prepareGenMod": (U32, [VP, VP, VP, VP, VP, VP, VP, VP, VP, U32, U32]),
        "genModCands": (None, [VP, VP, VP, VP, VP, VP, VP, VP, U32, U32]),
        "addModIons": (None, [VP, VP, VP, VP, VP, VP, VP, VP, VP, VP, U32, U32, VP, VP, VP, VP, U32, U32, U32, VP]),
        "addIons": (None, [VP, VP, VP, VP, VP, VP, VP, U32, U32, U32]),
        "prepare_scoring": (None, [VP, VP, VP, VP, U32]),
        "sort_val_f": (None, [VP, VP, U32]),
        "sort_idx_f": (None, [VP, VP, U32, U32]),
        "sort_rf": (None, [VP, VP, U32]),
        "sort_idx_rf": (None, [VP, VP, U32, U32]),
        "sort_b40c_f": (None, [VP, VP, U32]),
        "mvm_ff": (None, [VP, VP, VP, VP, U32, U32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


@pytest.fixture(scope="module")
def db(oracle, tiny):
    """The tiny database in the reference's device layout: packed residues
    (modable acids M, S, T, Y), fragment-order r / tc / tn and the mass-sorted
    index."""
    prot, sp, cfg = tiny
    mt = oracle.mass_table(True, synth.static_mods())
    d = dict(synth.DIGEST)
    d.pop("mono")
    r, tc, tn = oracle.digest(prot.seq, prot.seg, mt, **d)
    idx = oracle.sort_idx(r)
    ions = oracle.pack_ions(prot.seq, MA)
    return dict(prot=prot, sp=sp, mt=mt, r=r, tc=tc, tn=tn, idx=idx, ions=ions)


def test_prepare_ions(lib, oracle):
    rng = np.random.default_rng(3)
    letters = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWY", np.uint8)
    for n in (300, 511, 512, 5000):
        seq = rng.choice(letters, n).astype(np.uint8)
        d = _dev(seq)
        ma = _dev(np.frombuffer(MA, np.uint8).copy())
        lib.prepare_ions(_p(d), n, _p(ma), len(MA))
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), oracle.pack_ions(seq, MA, quirk=True)), n


def test_find_indices_in_range(lib):
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 100, 20000).astype(np.float32)
    out = torch.zeros(20000, dtype=torch.int32, device="cuda")
    n = lib.findIndicesInRange_f(_p(_dev(x)), _p(out), len(x), 25.0, 60.5)
    ref = np.nonzero((x >= np.float32(25.0)) & (x <= np.float32(60.5)))[0]
    assert n == len(ref)
    assert np.array_equal(_u32(out)[:n], ref)


def _windows_ref(r_sorted, lo, hi):
    return np.searchsorted(r_sorted, lo, "left"), np.searchsorted(r_sorted, hi, "right")


def test_find_spec_cands_by_mass(lib, db):
    r, idx = db["r"], db["idx"]
    rng = np.random.default_rng(5)
    masses = rng.uniform(500, 3000, 64).astype(np.float32)
    masses[:4] = r[idx[[0, 10, len(idx) // 2, len(idx) - 1]]]       # exact hits
    eps = np.float32(3.0)
    n = len(masses)
    b, e, num = (torch.zeros(n, dtype=torch.int32, device="cuda") for _ in range(3))
    total = lib.findSpecCandsByMass(_p(b), _p(e), _p(num), _p(_dev(r)), _p(_dev(idx)), len(r), _p(_dev(masses)), n,
                                    float(eps))
    rb, re_ = _windows_ref(r[idx], masses - eps, masses + eps)
    assert np.array_equal(_u32(b), rb) and np.array_equal(_u32(e), re_)
    assert np.array_equal(_u32(num), re_ - rb)
    assert total == int((re_ - rb).sum())


def _mod_windows(lib, db, mass, eps, delta):
    r, idx = db["r"], db["idx"]
    nm = len(delta)
    b, e, scan = (torch.zeros(nm, dtype=torch.int32, device="cuda") for _ in range(3))
    total = lib.findBeginEnd_f(_p(b), _p(e), _p(scan), _p(_dev(r)), _p(_dev(idx)), len(r), _p(_dev(delta)), nm,
                               float(mass), float(eps))
    return total, _u32(b), _u32(e), _u32(scan)


def test_find_begin_end(lib, db, oracle):
    counts, _, deltas = oracle.mod_combos(MA_MASS, 4)
    deltas = np.asarray(deltas, np.float32)
    r_sorted = db["r"][db["idx"]]
    for mass in (np.float32(1200.5), np.float32(2411.0)):
        eps = np.float32(3.0)
        total, b, e, scan = _mod_windows(lib, db, mass, eps, deltas)
        rb, re_ = _windows_ref(r_sorted, np.float32(mass - eps) - deltas, np.float32(mass + eps) - deltas)
        assert np.array_equal(b, rb) and np.array_equal(e, re_)
        sizes = (re_ - rb).astype(np.uint32)
        assert np.array_equal(scan, np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint32))
        assert total == int(sizes.sum())


def _letter_counts(ions, tc, tn, acids):
    seg = (ions[tc:tn] & 0x1F).astype(np.int32) + ord("A")
    return [int((seg == a).sum()) for a in acids]


def test_modification_pipeline(lib, db, oracle):
    """findBeginEnd_f per spectrum, findModablePeptides, calcTotalModCands,
    prepareGenMod and genModCands, as Search.hs:282-299 chains them, against
    a restatement of the reference's steps and the oracle's unranking."""
    r, tc, tn, idx, ions = db["r"], db["tc"], db["tn"], db["idx"], db["ions"]
    counts, _, deltas = oracle.mod_combos(MA_MASS, 4)
    counts = np.asarray(counts, np.uint32)
    deltas = np.asarray(deltas, np.float32)[:len(counts)]
    num_mod, num_ma = counts.shape
    rng = np.random.default_rng(6)
    masses = rng.uniform(900, 2200, 6).astype(np.float32)
    eps = np.float32(1.0)
    B, E, S, tot = [], [], [], []
    for m in masses:
        t, b, e, sc = _mod_windows(lib, db, m, eps, deltas)
        B.append(b), E.append(e), S.append(sc), tot.append(t)
    begin, end, scan = np.concatenate(B), np.concatenate(E), np.concatenate(S)
    spec_scan = np.concatenate([[0], np.cumsum(tot)[:-1]]).astype(np.uint32)
    ncand = int(sum(tot))
    assert ncand > 1000

    # reference rows (filter_by_mod.cu:145-378)
    rows = []
    for s in range(len(masses)):
        for mu in range(num_mod):
            o = s * num_mod + mu
            for i in range(begin[o], end[o]):
                rows.append((s, int(idx[i]), mu))
    assert len(rows) == ncand
    ref_pep, ref_mod, ref_cnt, ref_src = [], [], [], []
    for k, (s, p, mu) in enumerate(rows):
        c = _letter_counts(ions, int(tc[p]), int(tn[p]), MA)
        if all(c[a] >= counts[mu][a] for a in range(num_ma)):
            ref_pep.append(p), ref_mod.append(mu), ref_cnt.append(c), ref_src.append(k)
    ref_src = np.array(ref_src)
    ref_valid_scan = np.searchsorted(ref_src, spec_scan, "left")

    dv = lambda a: _dev(np.asarray(a, np.uint32).view(np.int32))
    o_pep, o_mod = (torch.zeros(ncand, dtype=torch.int32, device="cuda") for _ in range(2))
    o_cnt = torch.zeros(ncand * num_ma, dtype=torch.int32, device="cuda")
    o_vs = torch.zeros(len(masses), dtype=torch.int32, device="cuda")
    nvalid = lib.findModablePeptides(_p(o_pep), _p(o_mod), _p(o_cnt), _p(o_vs), _p(dv(spec_scan)), len(masses), ncand,
                                     _p(_dev(ions)), _p(dv(tc)), _p(dv(tn)), _p(dv(idx)), _p(dv(begin)), _p(dv(end)),
                                     _p(dv(scan)), _p(dv(counts.ravel())), num_mod,
                                     _p(_dev(np.frombuffer(MA, np.uint8).copy())), num_ma)
    assert nvalid == len(ref_pep) > 100
    assert np.array_equal(_u32(o_pep)[:nvalid], ref_pep)
    assert np.array_equal(_u32(o_mod)[:nvalid], ref_mod)
    assert np.array_equal(_u32(o_cnt)[:nvalid * num_ma].reshape(-1, num_ma), np.array(ref_cnt))
    assert np.array_equal(_u32(o_vs), ref_valid_scan)

    # calc_mod_cands.cu:27-119
    num_mpep = torch.zeros(nvalid, dtype=torch.int32, device="cuda")
    comb_scan = torch.zeros(nvalid * num_ma, dtype=torch.int32, device="cuda")
    total = lib.calcTotalModCands(_p(num_mpep), _p(comb_scan), _p(dv(counts.ravel())), _p(o_pep), _p(o_mod),
                                  _p(o_cnt), nvalid, num_mod, num_ma)
    ref_num, ref_cs = [], []
    for c, mu in zip(ref_cnt, ref_mod):
        num, row = 1, [0] * num_ma
        for i in range(num_ma - 1, -1, -1):
            num *= math.comb(c[i], int(counts[mu][i]))
            row[i] = num
        ref_num.append(num), ref_cs.append(row)
    assert np.array_equal(_u32(num_mpep), ref_num)
    assert np.array_equal(_u32(comb_scan).reshape(-1, num_ma), np.array(ref_cs))
    assert total == sum(ref_num)

    # prepare_gen_mod.cu:79-129
    nm = int(total)
    outs = [torch.zeros(nm, dtype=torch.int32, device="cuda") for _ in range(5)]
    sums = counts.sum(axis=1).astype(np.uint32)
    len_unrank = lib.prepareGenMod(*[_p(t) for t in outs], _p(dv(sums)), _p(o_pep), _p(o_mod), _p(num_mpep), nvalid,
                                   nm)
    m_pep, m_mod, m_rank, m_ith, m_scan = (_u32(t) for t in outs)
    ith = np.repeat(np.arange(nvalid), ref_num)
    assert np.array_equal(m_ith, ith)
    assert np.array_equal(m_pep, np.array(ref_pep)[ith]) and np.array_equal(m_mod, np.array(ref_mod)[ith])
    assert np.array_equal(m_rank, np.concatenate([np.arange(n) for n in ref_num]))
    size = sums[np.array(ref_mod)[ith]]
    assert np.array_equal(m_scan, np.concatenate([[0], np.cumsum(size)[:-1]]).astype(np.uint32))
    assert len_unrank == int(size.sum())

    # gen_mod_pep.cu:127-312 against the oracle's unranking
    unrank = torch.zeros(len_unrank, dtype=torch.int32, device="cuda")
    lib.genModCands(_p(unrank), _p(dv(counts.ravel())), _p(outs[3]), _p(outs[2]), _p(outs[4]), _p(o_mod), _p(o_cnt),
                    _p(comb_scan), nm, num_ma)
    torch.cuda.synchronize()
    un = _u32(unrank)
    rng2 = np.random.default_rng(8)
    for t in rng2.choice(nm, min(nm, 3000), replace=False):
        k = int(ith[t])
        x = int(m_rank[t])
        cs = ref_cs[k]
        ranks = []
        for i in range(num_ma):
            if i != num_ma - 1:
                nxt = cs[i + 1]
                ranks.append(x // nxt if x >= nxt else 0)
                x = x % nxt if x >= nxt else x
            else:
                ranks.append(x)
        want, pos = [], 0
        for i in range(num_ma):
            kk = int(counts[ref_mod[k]][i])
            if kk:
                want.extend(oracle.unrank_comb(ref_cnt[k][i], kk, ranks[i]))
        got = un[m_scan[t]:m_scan[t] + len(want)]
        assert np.array_equal(got, np.array(want, np.uint32)), t


def _dense_from_bins(bins, lvl, len_spec):
    row = np.zeros(len_spec, np.float32)
    row[bins] = np.array([0, 10, 25, 50], np.float32)[lvl]
    return row


@pytest.mark.parametrize("max_charge", [1, 2, 3, 4])
def test_add_ions_dense(lib, db, oracle, max_charge):
    """addIons: the dense rows of the reference (10/25/50, the highest level
    per bin, __fdividef arithmetic) match the oracle's bins except where
    fast division moves a bin at a half-bin edge."""
    r, tc, tn, ions, mt = db["r"], db["tc"], db["tn"], db["ions"], db["mt"]
    rng = np.random.default_rng(9)
    sel = rng.choice(len(r), 300, replace=False).astype(np.uint32)
    len_spec = 3000
    spec = torch.zeros((len(sel), len_spec), dtype=torch.float32, device="cuda")
    dv = lambda a: _dev(np.asarray(a, np.uint32).view(np.int32))
    lib.addIons(_p(spec), _p(_dev(r)), _p(_dev(mt)), _p(_dev(ions)), _p(dv(tc)), _p(dv(tn)), _p(dv(sel)), len(sel),
                max_charge, len_spec)
    torch.cuda.synchronize()
    got = spec.cpu().numpy()
    same = 0
    for i, f in enumerate(sel):
        ob, ol = oracle.ion_bins(ions, mt, int(tc[f]), int(tn[f]), float(r[f]), max_charge, len_spec)
        ref = _dense_from_bins(ob, ol, len_spec)
        assert set(np.unique(got[i])) <= {0.0, 10.0, 25.0, 50.0}
        same += np.array_equal(got[i], ref)
        # a fast-division bin moves by one at most
        assert abs(int((got[i] > 0).sum()) - len(ob)) <= 4, i
    assert same >= 0.8 * len(sel), same


def test_add_mod_ions_dense(lib, db, oracle):
    """addModIons: modified residues (type-agnostic i-th counter, the
    reference's default) shift the ladder; rows match the oracle's modified
    bins except at fast-division half-bin edges."""
    r, tc, tn, ions, mt = db["r"], db["tc"], db["tn"], db["ions"], db["mt"]
    counts, _, deltas = oracle.mod_combos(MA_MASS, 4)
    counts = np.asarray(counts, np.uint32)
    deltas = np.asarray(deltas, np.float32)[:len(counts)]
    num_mod, num_ma = counts.shape
    rng = np.random.default_rng(10)
    rows_pep, rows_mod, rows_unrank, mods_flags = [], [], [], []
    while len(rows_pep) < 200:
        f = int(rng.integers(len(r)))
        mu = int(rng.integers(num_mod))
        niso, un, md = oracle.mod_isoform(ions, int(tc[f]), int(tn[f]), MA, counts[mu])
        if niso == 0:
            continue
        rank = int(rng.integers(niso))
        _, un, md = oracle.mod_isoform(ions, int(tc[f]), int(tn[f]), MA, counts[mu], rank=rank)
        rows_pep.append(f), rows_mod.append(mu), rows_unrank.append(np.asarray(un, np.uint32)), mods_flags.append(md)
    sizes = np.array([len(u) for u in rows_unrank], np.uint32)
    scan = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint32)
    unrank = np.concatenate(rows_unrank).astype(np.uint32)
    len_spec, max_charge = 3000, 3
    spec = torch.zeros((len(rows_pep), len_spec), dtype=torch.float32, device="cuda")
    dv = lambda a: _dev(np.asarray(a, np.uint32).view(np.int32))
    lib.addModIons(_p(spec), _p(_dev(r)), _p(_dev(mt)), _p(_dev(ions)), _p(dv(tc)), _p(dv(tn)), _p(dv(rows_pep)),
                   _p(dv(rows_mod)), _p(dv(unrank)), _p(dv(scan)), len(unrank), len(rows_pep),
                   _p(dv(counts.ravel())), _p(_dev(deltas)), _p(_dev(np.frombuffer(MA, np.uint8).copy())),
                   _p(_dev(np.asarray(MA_MASS, np.float32))), num_ma, len_spec, max_charge, None)
    torch.cuda.synchronize()
    got = spec.cpu().numpy()
    same = 0
    for i, f in enumerate(rows_pep):
        L = int(tn[f] - tc[f])
        md = np.asarray(mods_flags[i][:L], np.uint8)
        add = np.zeros(L, np.float32)
        for j in range(L):
            if md[j]:
                add[j] = np.float32(MA_MASS[int((ions[tc[f] + j] >> 5) & 7) - 1])
        res = np.float32(r[f] + deltas[rows_mod[i]])
        ob, ol = oracle.ion_bins(ions, mt, int(tc[f]), int(tn[f]), float(res), max_charge, len_spec, res_add=add,
                                 modded=md)
        ref = _dense_from_bins(ob, ol, len_spec)
        same += np.array_equal(got[i], ref)
        assert abs(int((got[i] > 0).sum()) - len(ob)) <= 4, i
    assert same >= 0.8 * len(rows_pep), same


def test_prepare_scoring(lib, db):
    idx = db["idx"]
    rng = np.random.default_rng(11)
    begin = rng.integers(0, len(idx) - 500, 40).astype(np.uint32)
    num = rng.integers(0, 400, 40).astype(np.uint32)
    out = torch.zeros(int(num.sum()), dtype=torch.int32, device="cuda")
    dv = lambda a: _dev(np.asarray(a, np.uint32).view(np.int32))
    lib.prepare_scoring(_p(out), _p(dv(idx)), _p(dv(begin)), _p(dv(num)), len(begin))
    torch.cuda.synchronize()
    ref = np.concatenate([idx[b:b + n] for b, n in zip(begin, num)])
    assert np.array_equal(_u32(out), ref)


@pytest.mark.parametrize("fn", ["sort_val_f", "sort_b40c_f", "sort_rf", "sort_idx_f", "sort_idx_rf"])
def test_sorts_are_stable(lib, fn):
    rng = np.random.default_rng(12)
    n = 50000
    keys = np.round(rng.uniform(0, 500, n), 1).astype(np.float32)        # many ties
    vals = rng.permutation(n).astype(np.uint32)
    dk, dvv = _dev(keys), _dev(vals.view(np.int32))
    desc = fn in ("sort_rf", "sort_idx_rf")
    if fn.startswith("sort_idx"):
        getattr(lib, fn)(_p(dk), _p(dvv), n, 7)
        vals = np.arange(7, 7 + n, dtype=np.uint32)
    else:
        getattr(lib, fn)(_p(dk), _p(dvv), n)
    torch.cuda.synchronize()
    order = np.argsort(-keys if desc else keys, kind="stable")
    assert np.array_equal(dk.cpu().numpy(), keys[order])
    assert np.array_equal(_u32(dvv), vals[order])


def test_mvm(lib):
    rng = np.random.default_rng(13)
    m, n = 777, 2049
    A = rng.standard_normal((m, n)).astype(np.float32)
    x = rng.standard_normal(n).astype(np.float32)
    y = torch.zeros(m, dtype=torch.float32, device="cuda")
    lib.mvm_ff(None, _p(y), _p(_dev(A)), _p(_dev(x)), m, n)
    torch.cuda.synchronize()
    ref = A.astype(np.float64) @ x.astype(np.float64)
    assert np.allclose(y.cpu().numpy(), ref, rtol=1e-5, atol=1e-4)
