"""The allocation-free entry point (hfx_score_spectrum_noalloc), for callers
that cannot call cudaMalloc, must give the same matches as the regular
per-spectrum search path.  Two calls in a row share its fixed device scratch,
so the second call must not see the first call's leftovers.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _noalloc_fn(lib):
    f = lib.hfx_score_spectrum_noalloc
    P = C.c_void_p
    f.restype = C.c_int32
    f.argtypes = [P, P, P, P, P, C.c_uint32, P, P, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_int32,
                  C.c_int32, P, P, P, P]
    return f


def _charges(z):
    ch = int(np.rint(max(1.0, float(z) - 1.0)))
    return ch if ch <= 4 else 0


def test_noalloc_matches_regular_path(gpulib):
    import hfx_gb300
    prot, sp, _ = synth.workload("tiny", n_spectra=24)
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
        topn = 10
        regular = eng.search(sp, hfx_gb300.default_params(top_n=topn, batch_mode=0))

        d = torch.device("cuda:0")
        r, tc, tn, idx, mt = eng.db_export()
        ions = torch.from_numpy(hfx_gb300.pack_ions(prot.seq)).to(d)
        r_s = torch.from_numpy(np.ascontiguousarray(r[idx])).to(d)
        tc_s = torch.from_numpy(np.ascontiguousarray(tc[idx]).view(np.int32)).to(d)
        tn_s = torch.from_numpy(np.ascontiguousarray(tn[idx]).view(np.int32)).to(d)
        idx_d = torch.from_numpy(idx.view(np.int32)).to(d)
        dev = dict(mz=torch.from_numpy(sp.mz).to(d), it=torch.from_numpy(sp.it).to(d),
                   off=torch.from_numpy(sp.off).to(d), pcr=torch.from_numpy(sp.pcr).to(d),
                   z=torch.from_numpy(sp.z).to(d), tol=torch.from_numpy(sp.tol).to(d))
        p = hfx_gb300.default_params(top_n=topn)
        stride = 8192
        rows = torch.zeros((len(sp), stride), dtype=torch.float32, device=d)
        lens = torch.zeros(len(sp), dtype=torch.int32, device=d)
        eng.preprocess(dev, p, stride, rows, None, None, lens, None)
        wb = torch.zeros(len(sp), dtype=torch.int32, device=d)
        we = torch.zeros(len(sp), dtype=torch.int32, device=d)
        eng.find_windows(dev, p, wb, we)
        lens_h, wb_h, we_h = lens.cpu().numpy(), wb.cpu().numpy(), we.cpu().numpy()

        f = _noalloc_fn(hfx_gb300.load_library())
        mt_h = np.ascontiguousarray(mt, np.float32)
        stream = torch.cuda.current_stream(d)
        out_s = torch.empty(topn, dtype=torch.float32, device=d)
        out_k = torch.empty(topn, dtype=torch.int64, device=d)
        out_p = torch.empty(topn, dtype=torch.int32, device=d)
        checked = 0
        # two calls in a row first (spectra 0 and 1), then the rest
        for s in range(len(sp)):
            if lens_h[s] <= 0:
                continue
            rc = f(ions.data_ptr(), r_s.data_ptr(), tc_s.data_ptr(), tn_s.data_ptr(), idx_d.data_ptr(), len(r),
                   mt_h.ctypes.data, rows[s].data_ptr(), int(lens_h[s]), _charges(sp.z[s]), int(wb_h[s]),
                   int(we_h[s]), topn, 0, stream.cuda_stream, out_s.data_ptr(), out_k.data_ptr(),
                   out_p.data_ptr())
            assert rc == 0
            torch.cuda.synchronize()
            got_k = out_k.cpu().numpy().view(np.uint64)
            got_s = out_s.cpu().numpy()
            got_p = out_p.cpu().numpy().view(np.uint32)
            assert np.array_equal(got_k, regular.key[s]), s
            # same canonical FP32 order as the regular path: bit-identical scores
            assert np.array_equal(got_s.view(np.uint32), regular.score[s].view(np.uint32)), s
            assert np.array_equal(got_p, regular.pep[s]), s
            checked += 1
        assert checked >= 2

        # the __fdividef variant, and a window of every candidate (more than
        # HFX_NOALLOC_MAX_BLOCKS x 32, so each block strides over several
        # chunks), both against the regular path on the same settings
        s0 = int(np.nonzero(lens_h > 0)[0][0])
        wide = sp.subset(np.array([s0, s0]))
        wide.tol[:] = 20000.0  # a Da window covering the whole database
        for fastdiv, spec in ((1, sp.subset(np.array([s0]))), (0, wide), (1, wide)):
            ref = eng.search(spec, hfx_gb300.default_params(top_n=topn, batch_mode=0, fastdiv=fastdiv))
            b, e = (int(wb_h[s0]), int(we_h[s0])) if len(spec) == 1 else (0, len(r))
            assert int(ref.ncand[0]) == e - b
            for _ in range(2):
                rc = f(ions.data_ptr(), r_s.data_ptr(), tc_s.data_ptr(), tn_s.data_ptr(), idx_d.data_ptr(), len(r),
                       mt_h.ctypes.data, rows[s0].data_ptr(), int(lens_h[s0]), _charges(sp.z[s0]), b, e, topn,
                       fastdiv, stream.cuda_stream, out_s.data_ptr(), out_k.data_ptr(), out_p.data_ptr())
                assert rc == 0
                torch.cuda.synchronize()
                assert np.array_equal(out_k.cpu().numpy().view(np.uint64), ref.key[0]), (fastdiv, e - b)
                assert np.array_equal(out_s.cpu().numpy().view(np.uint32), ref.score[0].view(np.uint32))
                assert np.array_equal(out_p.cpu().numpy().view(np.uint32), ref.pep[0])
        assert len(r) > 304 * 32

        # sizes beyond the fixed scratch are rejected, nothing is launched
        rc = f(ions.data_ptr(), r_s.data_ptr(), tc_s.data_ptr(), tn_s.data_ptr(), idx_d.data_ptr(), len(r),
               mt_h.ctypes.data, rows[0].data_ptr(), int(lens_h[0]), 1, 0, 10, 33, 0, stream.cuda_stream,
               out_s.data_ptr(), out_k.data_ptr(), out_p.data_ptr())
        assert rc == 1
        rc = f(ions.data_ptr(), r_s.data_ptr(), tc_s.data_ptr(), tn_s.data_ptr(), idx_d.data_ptr(), len(r),
               mt_h.ctypes.data, rows[0].data_ptr(), 9000, 1, 0, 10, topn, 0, stream.cuda_stream,
               out_s.data_ptr(), out_k.data_ptr(), out_p.data_ptr())
        assert rc == 1
    finally:
        eng.close()
