"""Generate the golden fixtures of tests/golden from the REFERENCE's own code.

Run where the reference checkout is (not on a GPU machine): it needs it and
oracle/_ref/libhfx_ref.so, which `HFX_REFERENCE=<checkout> make -C oracle ref`
compiles from the
reference's unmodified Thrust sources (filter.cu, filter_by_mod.cu,
calc_mod_cands.cu, prepare_gen_mod.cu, gen_mod_pep.cu, prepare_scoring.cu,
sort.cu, prepare_ions_test.cu) with Thrust's host (CPP) system.

    python tests/golden/make_golden.py

Fixtures:
  ref_combinatorics.npz  choose(n, k) and unrankComb rows (combinatorics.h)
  ref_prepare_ions.npz   packed residues (prepare_ions_test.cu:20-55)
  ref_enumeration.npz    a small seeded database, spectrum masses and every
                         output of the reference's stage (b)/(e) pipeline in
                         the order Search.hs:151-165 and :305-394 call it
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from hfx_gb300 import synth  # noqa: E402

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libhfx_ref.so")


def ref_lib():
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    return C.CDLL(REF_LIB)


def p(a):
    return a.ctypes.data


def u32(n):
    return np.zeros(max(int(n), 1), np.uint32)


def run_enumeration(L, ions, r, tc, tn, idx, masses, eps, ma, ma_mass, max_ma):
    """The reference's searchWithoutMods/searchWithMods device pipeline."""
    u = C.c_uint32
    f = C.c_float
    L.findSpecCandsByMass.restype = u
    L.findBeginEnd_f.restype = u
    L.findModablePeptides.restype = u
    L.calcTotalModCands.restype = u
    L.prepareGenMod.restype = u
    ns, npep = len(masses), len(r)
    out = {}
    # filter.cu:75-127 (Search.hs:151-165)
    b, e, n = u32(ns), u32(ns), u32(ns)
    tot = L.findSpecCandsByMass(C.c_void_p(p(b)), C.c_void_p(p(e)), C.c_void_p(p(n)), C.c_void_p(p(r)),
                                C.c_void_p(p(idx)), u(npep), C.c_void_p(p(masses)), u(ns), f(eps))
    out.update(plain_begin=b[:ns], plain_end=e[:ns], plain_num=n[:ns], plain_total=np.uint32(tot))
    # prepare_scoring.cu:47-67
    flat = u32(tot)
    L.prepare_scoring(C.c_void_p(p(flat)), C.c_void_p(p(idx)), C.c_void_p(p(b)), C.c_void_p(p(n)), u(ns))
    out["plain_flat"] = flat[:tot]
    # Fragment.hs:260-289 combination table (host side, restated by the oracle)
    counts, sums, deltas = O.mod_combos(np.array(ma_mass, np.float32), max_ma)
    num_mod, num_ma = counts.shape
    mc = np.ascontiguousarray(counts.reshape(-1).astype(np.uint32))
    mcs = np.ascontiguousarray(sums.astype(np.uint32))
    md = np.ascontiguousarray(deltas.astype(np.float32))
    out.update(mod_counts=counts, mod_sums=sums, mod_deltas=deltas)
    # filter_by_mod.cu:35-143 per spectrum (Search.hs:317-322)
    mb, me, ms = u32(ns * num_mod), u32(ns * num_mod), u32(ns * num_mod)
    spec_num_cand = []
    for s in range(ns):
        o = s * num_mod
        spec_num_cand.append(L.findBeginEnd_f(
            C.c_void_p(mb.ctypes.data + 4 * o), C.c_void_p(me.ctypes.data + 4 * o), C.c_void_p(ms.ctypes.data + 4 * o),
            C.c_void_p(p(r)), C.c_void_p(p(idx)), u(npep), C.c_void_p(p(md)), u(num_mod), f(masses[s]), f(eps)))
    out.update(mod_begin=mb[: ns * num_mod], mod_end=me[: ns * num_mod], mod_scan=ms[: ns * num_mod],
               spec_num_cand=np.array(spec_num_cand, np.uint32))
    total = int(sum(spec_num_cand))
    scan = np.zeros(ns + 1, np.uint32)
    scan[1:] = np.cumsum(spec_num_cand)
    pep_idx, pep_mod, pep_mac, valid_scan = u32(total), u32(total), u32(total * num_ma), u32(ns)
    mab = np.frombuffer(ma, np.uint8).copy()
    nvalid = L.findModablePeptides(
        C.c_void_p(p(pep_idx)), C.c_void_p(p(pep_mod)), C.c_void_p(p(pep_mac)), C.c_void_p(p(valid_scan)),
        C.c_void_p(p(scan)), u(ns), u(total), C.c_void_p(p(ions)), C.c_void_p(p(tc)), C.c_void_p(p(tn)),
        C.c_void_p(p(idx)), C.c_void_p(p(mb)), C.c_void_p(p(me)), C.c_void_p(p(ms)), C.c_void_p(p(mc)),
        u(num_mod), C.c_void_p(p(mab)), u(num_ma))
    out.update(valid_pep=pep_idx[:nvalid], valid_mod=pep_mod[:nvalid], valid_ma_count=pep_mac[: nvalid * num_ma],
               valid_scan=valid_scan[:ns])
    # calc_mod_cands.cu:76-119
    pnm, pncs = u32(nvalid), u32(nvalid * num_ma)
    nmpep = L.calcTotalModCands(C.c_void_p(p(pnm)), C.c_void_p(p(pncs)), C.c_void_p(p(mc)), C.c_void_p(p(pep_idx)),
                                C.c_void_p(p(pep_mod)), C.c_void_p(p(pep_mac)), u(nvalid), u(num_mod), u(num_ma))
    out.update(pep_num_mpep=pnm[:nvalid], pep_comb_scan=pncs[: nvalid * num_ma])
    # prepare_gen_mod.cu:79-129
    a1, a2, a3, a4, a5 = (u32(nmpep) for _ in range(5))
    len_unrank = L.prepareGenMod(C.c_void_p(p(a1)), C.c_void_p(p(a2)), C.c_void_p(p(a3)), C.c_void_p(p(a4)),
                                 C.c_void_p(p(a5)), C.c_void_p(p(mcs)), C.c_void_p(p(pep_idx)),
                                 C.c_void_p(p(pep_mod)), C.c_void_p(p(pnm)), u(nvalid), u(nmpep))
    out.update(mpep_pep=a1[:nmpep], mpep_mod=a2[:nmpep], mpep_rank=a3[:nmpep], mpep_ith=a4[:nmpep],
               mpep_unrank_off=a5[:nmpep])
    # gen_mod_pep.cu:229-312
    unrank = u32(len_unrank)
    L.genModCands(C.c_void_p(p(unrank)), C.c_void_p(p(mc)), C.c_void_p(p(a4)), C.c_void_p(p(a3)), C.c_void_p(p(a5)),
                  C.c_void_p(p(pep_mod)), C.c_void_p(p(pep_mac)), C.c_void_p(p(pncs)), u(nmpep), u(num_ma))
    out["mpep_unrank"] = unrank[:len_unrank]
    return out


def main():
    L = ref_lib()
    L.ref_choose.restype = C.c_uint32
    L.ref_choose.argtypes = [C.c_uint32, C.c_uint32]
    # combinatorics.h
    ch = np.array([[L.ref_choose(n, k) for k in range(17)] for n in range(65)], np.uint32)
    rows, keys = [], []
    for n in range(0, 15):
        for k in range(1, min(n, 5) + 1):
            tot = int(ch[n, k])
            for rank in range(tot):
                a = np.zeros(8, np.uint32)
                L.ref_unrank_comb(C.c_void_p(p(a)), C.c_uint32(n), C.c_uint32(k), C.c_uint32(rank))
                rows.append(a)
                keys.append((n, k, rank))
    np.savez_compressed(os.path.join(HERE, "ref_combinatorics.npz"), choose=ch, unrank_keys=np.array(keys, np.uint32),
                        unrank_rows=np.array(rows, np.uint32))
    # prepare_ions_test.cu
    rng = np.random.Generator(np.random.PCG64(7))
    seq = np.frombuffer(synth.AA.encode(), np.uint8)[rng.integers(0, 20, 4000)].copy()
    outs = {}
    for ma in (b"", b"M", b"MSTY", b"CQ"):
        o = np.zeros(len(seq), np.uint8)
        mab = np.frombuffer(ma, np.uint8).copy() if ma else np.zeros(1, np.uint8)
        L.ref_prepare_ions(C.c_void_p(p(o)), C.c_void_p(p(seq)), C.c_uint32(len(seq)), C.c_void_p(p(mab)),
                           C.c_uint32(len(ma)))
        outs["packed_" + (ma.decode() or "none")] = o
    np.savez_compressed(os.path.join(HERE, "ref_prepare_ions.npz"), seq=seq, **outs)
    # stage (b)/(e) pipeline on a small seeded database
    prot = synth.proteins(150, seed=11)
    mt = O.mass_table(True, synth.static_mods())
    r, tc, tn = O.digest(prot.seq, prot.seg, mt, rule=1, missed=1, min_mass=400.0, max_mass=4000.0)
    idx = np.zeros(len(r), np.uint32)
    rr = r.copy()
    L.sort_idx_f(C.c_void_p(p(rr)), C.c_void_p(p(idx)), C.c_uint32(len(r)), C.c_uint32(0))
    ma, ma_mass, max_ma = b"MSTY", [15.995, 79.966, 79.966, 79.966], 4
    ions = O.pack_ions(prot.seq, ma)
    rng = np.random.Generator(np.random.PCG64(12))
    # spectrum residual masses: some at database masses (exact ties), some random
    masses = np.concatenate([r[rng.integers(0, len(r), 6)],
                             rng.uniform(500.0, 2500.0, 6).astype(np.float32)]).astype(np.float32)
    eps = np.float32(1.5)
    out = run_enumeration(L, ions, r, tc, tn, idx, masses, eps, ma, ma_mass, max_ma)
    np.savez_compressed(os.path.join(HERE, "ref_enumeration.npz"), seq=prot.seq, seg=prot.seg, mt=mt, r=r, tc=tc,
                        tn=tn, ions=ions, idx_sorted=idx, masses=masses, eps=eps,
                        ma=np.frombuffer(ma, np.uint8), ma_mass=np.array(ma_mass, np.float32),
                        max_ma=np.int32(max_ma), **out)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
