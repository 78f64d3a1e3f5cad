"""Seeded synthetic workloads (proteins + MS2 spectra) for the search path.

The reference's own data (UniProt FASTA, .dta spectra) is not in its tree and
the benchmark names no public dataset, so every workload is generated here
from a fixed seed with the sizes and distributions of the five benchmark
configurations:

  tiny      2,000 proteins (lengths U[100,800]), 100 spectra at charge 2-3,
            150 uniform noise peaks, +-3 Da, 1.0005 Da bins, top-10
  full      20,000 proteins, 10,000 spectra at charge 1/2/3/4 in proportions
            5/50/35/10 %, 50-400 peaks each, +-3 Da, top-10
  mods      `full` + variable M oxidation (+15.995) and S/T/Y phospho
            (+79.966), up to 3 modifications (max-modable-acids = 4)
  batch     100,000 spectra, 80 % at +-10 ppm, 20 % at +-500 Da
  highres   `batch` binned at 0.02 Da

Residues are i.i.d. with the UniProtKB/Swiss-Prot amino-acid composition
(published release statistics).  Each spectrum comes from a random tryptic
peptide of the database (cleave after K/R not before P, <= 1 missed
cleavage, length 6-50, carbamidomethyl C +57.021): its b/y ions at fragment
charges 1..max(1, z-1) with N(0, 0.2 Da) m/z jitter, LogNormal(0, 1)
intensities and 70 % of ions kept, plus uniform noise peaks over 200-2000
m/z.  Peaks are sorted by m/z (Correlation.hs:66 reads the last peak).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

AA = "ACDEFGHIKLMNPQRSTVWY"
# UniProtKB/Swiss-Prot amino-acid composition, percent.
AA_FREQ = {
    "A": 8.25, "R": 5.53, "N": 4.06, "D": 5.46, "C": 1.38, "Q": 3.93, "E": 6.72,
    "G": 7.07, "H": 2.27, "I": 5.91, "L": 9.64, "K": 5.80, "M": 2.41, "F": 3.86,
    "P": 4.74, "S": 6.65, "T": 5.36, "W": 1.10, "Y": 2.92, "V": 6.86,
}
MONO = {
    "A": 71.037114, "R": 156.101111, "N": 114.042927, "D": 115.026943, "C": 103.009185,
    "E": 129.042593, "Q": 128.058578, "G": 57.021464, "H": 137.058912, "I": 113.084064,
    "L": 113.084064, "K": 128.094963, "M": 131.040485, "F": 147.068414, "P": 97.052764,
    "S": 87.032028, "T": 101.047679, "W": 186.079313, "Y": 163.06332, "V": 99.068414,
}
PROTON = 1.007276     # Mass.hs:25
WATER = 18.010565     # Mass.hs:20
CARBAMIDOMETHYL = 57.021


@dataclass
class Proteins:
    seq: np.ndarray   # uint8 concatenated residues
    seg: np.ndarray   # uint32 [n+1] offsets


@dataclass
class Spectra:
    mz: np.ndarray
    it: np.ndarray
    off: np.ndarray
    pcr: np.ndarray
    z: np.ndarray
    tol: np.ndarray
    source: list = field(default_factory=list)   # generating peptide of each spectrum
    title: list = field(default_factory=list)    # ms2info (MGF TITLE) of each spectrum, when read from a file

    def arrays(self):
        return self.mz, self.it, self.off, self.pcr, self.z, self.tol

    def __len__(self):
        return len(self.pcr)

    def subset(self, idx) -> "Spectra":
        idx = np.asarray(idx)
        mz, it, off = [], [], [0]
        for i in idx:
            a, b = self.off[i], self.off[i + 1]
            mz.append(self.mz[a:b])
            it.append(self.it[a:b])
            off.append(off[-1] + (b - a))
        return Spectra(np.concatenate(mz).astype(np.float32), np.concatenate(it).astype(np.float32),
                       np.array(off, np.int64), self.pcr[idx].copy(), self.z[idx].copy(),
                       self.tol[idx].copy(), [self.source[i] for i in idx] if self.source else [],
                       [self.title[i] for i in idx] if self.title else [])


def proteins(n: int, seed: int, len_lo: int = 100, len_hi: int = 800) -> Proteins:
    rng = np.random.Generator(np.random.PCG64(seed))
    letters = np.frombuffer("".join(AA_FREQ.keys()).encode(), np.uint8)
    p = np.array(list(AA_FREQ.values()), np.float64)
    p /= p.sum()
    lens = rng.integers(len_lo, len_hi + 1, size=n)
    seg = np.zeros(n + 1, np.uint32)
    seg[1:] = np.cumsum(lens)
    seq = letters[rng.choice(len(letters), size=int(seg[-1]), p=p)]
    return Proteins(seq.astype(np.uint8), seg)


def tryptic_peptides(prot: Proteins, missed: int = 1, min_len: int = 6, max_len: int = 50):
    """(start, end) of tryptic peptides: after K/R not before P."""
    s = prot.seq
    kr = (s == ord("K")) | (s == ord("R"))
    nxt_p = np.zeros_like(kr)
    nxt_p[:-1] = s[1:] == ord("P")
    site = kr & ~nxt_p
    out = []
    for i in range(len(prot.seg) - 1):
        a, b = int(prot.seg[i]), int(prot.seg[i + 1])
        cuts = [a] + list(np.nonzero(site[a:b])[0] + a + 1)
        if cuts[-1] != b:
            cuts.append(b)
        for j in range(len(cuts) - 1):
            for k in range(j + 1, min(j + 2 + missed, len(cuts))):
                L = cuts[k] - cuts[j]
                if min_len <= L <= max_len:
                    out.append((cuts[j], cuts[k]))
    return np.array(out, np.int64)


def _residue_masses(seq: bytes) -> np.ndarray:
    m = np.array([MONO[chr(c)] for c in seq], np.float64)
    m[np.frombuffer(seq, np.uint8) == ord("C")] += CARBAMIDOMETHYL
    return m


def spectra(prot: Proteins, n: int, seed: int, charge_p: dict, npeaks=(None, None), n_noise: int = 150,
            tol_da: float = 3.0, ppm_frac: float = 0.0, ppm_tol: float = 10.0, open_tol: float = 500.0,
            peps: np.ndarray | None = None) -> Spectra:
    """Synthetic MS2 spectra from random database peptides.

    npeaks=(lo, hi): total peaks per spectrum drawn U[lo, hi] (noise fills the
    rest); (None, None) uses n_noise noise peaks.  ppm_frac of the spectra
    get a +-ppm_tol ppm window, stored as -ppm_tol (the per-spectrum unit
    convention, tol_ppm = 2), the rest a Da window (open_tol if ppm_frac>0,
    else tol_da).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    if peps is None:
        peps = tryptic_peptides(prot)
    charges = np.array(list(charge_p.keys()), np.float32)
    cp = np.array(list(charge_p.values()), np.float64)
    cp /= cp.sum()
    mzs, its, off = [], [], [0]
    pcr = np.empty(n, np.float32)
    zz = np.empty(n, np.float32)
    tol = np.empty(n, np.float32)
    src = []
    for i in range(n):
        a, b = peps[rng.integers(len(peps))]
        seqb = prot.seq[a:b].tobytes()
        m = _residue_masses(seqb)
        z = float(rng.choice(charges, p=cp))
        neutral = m.sum() + WATER
        pcr[i] = (neutral + z * PROTON) / z
        zz[i] = z
        pre = np.cumsum(m)[:-1]
        suf = neutral - pre
        ions = []
        for c in range(1, max(1, int(z) - 1) + 1):
            ions.append((pre + c * PROTON) / c)
            ions.append((suf + c * PROTON) / c)
        ion = np.concatenate(ions)
        ion = ion[rng.random(len(ion)) < 0.7]
        ion = ion + rng.normal(0.0, 0.2, size=len(ion))
        if npeaks[0] is not None:
            total = int(rng.integers(npeaks[0], npeaks[1] + 1))
            if len(ion) > total:
                ion = rng.choice(ion, size=total, replace=False)
            nn = total - len(ion)
        else:
            nn = n_noise
        noise = rng.uniform(200.0, 2000.0, size=nn)
        allmz = np.concatenate([ion, noise])
        allit = rng.lognormal(0.0, 1.0, size=len(allmz))
        keep = allmz > 1.0
        allmz, allit = allmz[keep], allit[keep]
        o = np.argsort(allmz, kind="stable")
        mzs.append(allmz[o].astype(np.float32))
        its.append(allit[o].astype(np.float32))
        off.append(off[-1] + len(o))
        if ppm_frac > 0.0:
            tol[i] = -ppm_tol if rng.random() < ppm_frac else open_tol
        else:
            tol[i] = tol_da
        src.append(seqb.decode())
    return Spectra(np.concatenate(mzs), np.concatenate(its), np.array(off, np.int64), pcr, zz, tol, src)


def static_mods() -> np.ndarray:
    add = np.zeros(26, np.float32)
    add[ord("C") - ord("A")] = CARBAMIDOMETHYL
    return add


# Digest settings of the benchmark configurations (tryptic with the P rule,
# <= 1 missed cleavage, length 6-50; mass window of the reference defaults).
DIGEST = dict(mono=True, rule=1, missed=1, min_mass=400.0, max_mass=7200.0, proline_rule=True,
              min_len=6, max_len=50)


# Variable modifications of the modification workload: Met oxidation and
# Ser/Thr/Tyr phosphorylation, up to 3 per peptide (max-modable-acids 4,
# whose combination sums are strictly below it).
MODS = dict(ma="MSTY", ma_mass=[15.995, 79.966, 79.966, 79.966], max_ma=4)


def workload(name: str, n_spectra: int | None = None):
    """(proteins, spectra, search settings) of a named configuration."""
    if name == "tiny":
        prot = proteins(2000, seed=0)
        sp = spectra(prot, n_spectra or 100, seed=100, charge_p={2: 0.5, 3: 0.5}, n_noise=150)
        return prot, sp, dict(bin_width=1.0005079, top_n=10)
    if name in ("full", "mods"):
        prot = proteins(20000, seed=1)
        sp = spectra(prot, n_spectra or 10000, seed=101, charge_p={1: 0.05, 2: 0.5, 3: 0.35, 4: 0.10},
                     npeaks=(50, 400))
        cfg = dict(bin_width=1.0005079, top_n=10)
        if name == "mods":
            cfg.update(MODS)
        return prot, sp, cfg
    if name in ("batch", "highres"):
        prot = proteins(20000, seed=1)
        sp = spectra(prot, n_spectra or 100000, seed=103, charge_p={1: 0.05, 2: 0.5, 3: 0.35, 4: 0.10},
                     npeaks=(50, 400), ppm_frac=0.8)
        bw = 0.02 if name == "highres" else 1.0005079
        hr = int(name == "highres")
        return prot, sp, dict(bin_width=bw, top_n=10, tol_ppm=2, custom_bin_width=hr, ion_bins_custom=hr)
    raise KeyError(name)
