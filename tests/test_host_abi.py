"""CPU tests of the C ABI library: it loads, exports every symbol the
public header declares, and its host-side database steps (digest, residue
packing) match the oracle.  No device work."""
import os
import re
import subprocess

import numpy as np
import pytest

from hfx_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    """Function names declared by a public header (return type, name, '(')."""
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    ret = r"(?:void|u?int(?:8|16|32|64)_t|size_t|const char|char|float|double)"
    return sorted(set(re.findall(ret + r"\s*\**\s+\**([A-Za-z_]\w*)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpulib):
    import hfx_gb300
    nm = subprocess.run(["nm", "-D", "--defined-only", hfx_gb300.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (\w+)\b", nm))
    headers = sorted(os.listdir(os.path.join(ROOT, "include")))
    assert "hfx_legacy.h" in headers
    for h in headers:
        syms = _declared(h)
        assert syms, h
        for sym in syms:
            assert sym in exported, (h, sym)
            assert hasattr(gpulib, sym)
    assert set(hfx_gb300.EXPORTED) <= exported


def test_legacy_header_matches_the_reference_abi():
    """The per-stage symbols the reference's Haskell host binds (Algorithms.hs
    foreign imports of algorithms.h), every one declared with the C ABI."""
    want = {"prepare_ions", "findIndicesInRange_f", "findSpecCandsByMass", "findBeginEnd_f",
            "findModablePeptides", "calcTotalModCands", "prepareGenMod", "genModCands", "addModIons", "addIons",
            "prepare_scoring", "sort_val_f", "sort_idx_f", "sort_rf", "sort_idx_rf", "sort_b40c_f", "mvm_ff"}
    assert want <= set(_declared("hfx_legacy.h"))


def test_product_digest_matches_oracle(gpulib, oracle, tiny):
    import hfx_gb300
    prot, _, _ = tiny
    for mono, rule, missed, pr, lo, hi in [(True, 1, 1, True, 6, 50), (True, 1, 2, False, 0, 0),
                                           (False, 2, 0, False, 0, 0), (True, 0, 0, False, 0, 0),
                                           (True, 13, 1, True, 3, 30)]:
        mt = oracle.mass_table(mono, synth.static_mods())
        a = hfx_gb300.digest(prot.seq, prot.seg, mt, rule=rule, missed=missed, proline_rule=pr, min_len=lo,
                             max_len=hi)
        b = oracle.digest(prot.seq, prot.seg, mt, rule=rule, missed=missed, proline_rule=pr, min_len=lo,
                          max_len=hi)
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_digest_terminal_convention(gpulib, oracle):
    """Fragment.hs:383-390: a fragment ending at a cleavage site stores the
    index of its last residue; the last piece of a protein stores one past."""
    import hfx_gb300
    seq = np.frombuffer(b"AAAAKGGGGGGRCCCCCCCCCC", np.uint8)
    seg = np.array([0, len(seq)], np.uint32)
    mt = oracle.mass_table(True)
    r, tc, tn = hfx_gb300.digest(seq, seg, mt, rule=1, missed=0, min_mass=0.0, max_mass=1e9)
    assert list(zip(tc, tn)) == [(0, 4), (5, 11), (12, 22)]


def test_product_packing_matches_reference(gpulib, golden):
    import hfx_gb300
    g = golden("ref_prepare_ions.npz")
    for key in g.files:
        if key.startswith("packed_"):
            ma = key[len("packed_"):]
            ma = b"" if ma == "none" else ma.encode()
            assert np.array_equal(hfx_gb300.pack_ions(g["seq"], ma), g[key]), key


def test_no_cpu_fallback_without_library(tmp_path):
    import hfx_gb300
    try:
        hfx_gb300._lib_saved = hfx_gb300._lib
        hfx_gb300._lib = None
        try:
            hfx_gb300.load_library(str(tmp_path / "missing.so"))
            raise AssertionError("expected a loud failure")
        except OSError:
            pass
    finally:
        hfx_gb300._lib = hfx_gb300._lib_saved


def test_headers_are_plain_c(tmp_path):
    """Every public header compiles as C99, and a C program that links
    libhfx_gpu.so calls the host-only readers and formatters (no GPU)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(ROOT, "include")
    for h in sorted(os.listdir(inc)):
        if h.endswith(".h"):
            r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-x", "c",
                                os.path.join(inc, h)], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr
    src = tmp_path / "io_check.c"
    src.write_text(r'''
#include <stdio.h>
#include <string.h>
#include "hfx_io.h"
#include "hfx_report.h"
int main(void) {
    const char mgf[] = "BEGIN IONS\nTITLE=t\nCHARGE=2+\nPEPMASS=500.25\n100 1\n200 2\nEND IONS\n";
    hfx_spectra *s = 0;
    char err[128];
    if (hfx_parse_spectra(mgf, (int64_t)strlen(mgf), 1, &s, err, sizeof err) != 0) return 1;
    const float *mz, *it, *pcr, *z;
    const int64_t *off;
    hfx_spectra_arrays(s, &mz, &it, &off, &pcr, &z);
    char num[64];
    hfx_format_number((double)pcr[0], 0, num, sizeof num);
    printf("%lld %lld %s %g\n", (long long)hfx_spectra_count(s), (long long)off[1], num, (double)mz[1]);
    hfx_spectra_free(s);
    return 0;
}
''')
    lib_dir = os.path.join(ROOT, "hfx_gb300")
    exe = tmp_path / "io_check"
    r = subprocess.run([cc, "-std=c99", "-I", inc, str(src), "-L", lib_dir, "-lhfx_gpu", "-Wl,-rpath," + lib_dir,
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split() == ["1", "2", "500.25", "200"], (r.stdout, r.stderr)
