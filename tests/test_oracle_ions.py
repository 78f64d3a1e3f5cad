"""The oracle's "Ions" column (hfxo_match_ions) against a literal
single-precision restatement of Match.hs:36-44 scoreSP and
IonSeries.hs:87-147 (extractPeaks, matchIonSequence, bions, ionMZ), on
seeded spectra and peptides, plus hand-checked cases."""
import numpy as np
import pytest

f32 = np.float32
H = f32(1.007276)       # Mass.hs:25
H2O = f32(18.010565)    # Mass.hs:20


def _hs_round(v):
    """Haskell round: halves to even."""
    return int(np.rint(v))


def _literal(x, z, pep, mt, mh, nstar, bw):
    x = np.asarray(x, f32)
    n = len(x)
    # extractPeaks: the 200 largest values (lower index first on ties),
    # accumulate max into zeros of length n div 3 + 1
    order = sorted(range(n), key=lambda i: (-float(x[i]), i))[:200]
    peaks = [f32(0)] * (n // 3 + 1)
    for i in order:
        peaks[i // 3] = max(peaks[i // 3], x[i])
    # bions: concatMap over [1 .. max 1 (charge-1)] of map (`ionMZ` c) (scanl1 (+) masses)
    lim = max(f32(1), f32(f32(z) - f32(1)))
    ions = []
    c = f32(1)
    while c <= f32(lim + f32(0.5)):
        m = None
        for ch in pep:
            a = f32(mt[ch - ord("A")])
            m = a if m is None else f32(m + a)
            ions.append(f32(f32(m + f32(H * c)) / c))
        c = f32(c + f32(1))

    def matched(v):
        i = _hs_round(f32(f32(v / f32(bw)) / f32(3)))
        return 0 <= i < len(peaks) and peaks[i] > 0

    b = [matched(v) for v in ions][:-1]
    y = [matched(f32(f32(mh) - v)) for v in ions][1:]
    return sum(b) + sum(y), (len(pep) + 4 + nstar - 5) * 2


def _mt(oracle):
    from hfx_gb300 import synth
    return oracle.mass_table(True, synth.static_mods())


@pytest.mark.parametrize("seed", range(6))
def test_match_ions_matches_literal(oracle, seed):
    rng = np.random.default_rng(seed)
    mt = _mt(oracle)
    letters = b"ACDEFGHIKLMNPQRSTVWY"
    for _ in range(20):
        n = int(rng.integers(76, 2200))
        x = rng.normal(0.0, 1.0, n).astype(f32)
        x[rng.random(n) < 0.3] = 0.0
        if seed % 2:
            x = np.round(x, 1).astype(f32)     # many ties at the 200th value
        L = int(rng.integers(4, 30))
        pep = bytes(int(v) for v in rng.choice(list(letters), L))
        res = f32(0)
        for ch in pep:
            res = f32(res + f32(mt[ch - ord("A")]))
        mh = f32(f32(res + H) + H2O)
        z = float(rng.integers(1, 6))
        nstar = int(rng.integers(0, 3))
        bw = [1.0005079, 1.0011413, 0.02][int(rng.integers(0, 3))]
        got = oracle.match_ions(x, z, pep, mt, mh, nstar, bw)
        assert got == _literal(x, z, pep, mt, mh, nstar, bw)


def test_match_ions_hand_cases(oracle):
    mt = _mt(oracle)
    # a single positive peak: the b1 ion of charge 1 of "GG...": mass(G)+H
    pep = b"GAGA"
    g = f32(mt[ord("G") - ord("A")])
    b1 = f32(f32(g + H) / f32(1))
    bw = 1.0005079
    k = int(np.rint(f32(f32(b1 / f32(bw)) / f32(3))))
    x = np.zeros(3 * k + 90, f32) - 1.0
    x[3 * k + 1] = 5.0                    # same peak bin (index div 3 = k)
    res = f32(0)
    for ch in pep:
        res = f32(res + f32(mt[ch - ord("A")]))
    mh = f32(f32(res + H) + H2O)
    m, t = oracle.match_ions(x, 2.0, pep, mt, mh, 0, bw)
    assert t == (4 - 1) * 2
    assert m >= 1 and (m, t) == _literal(x, 2.0, pep, mt, mh, 0, bw)
    # no positive value: nothing matches
    m, t = oracle.match_ions(-np.abs(x), 3.0, pep, mt, mh, 2, bw)
    assert (m, t) == (0, (4 + 2 - 1) * 2)
