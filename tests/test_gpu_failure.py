"""Failure detection without a GPU fault.  A bounded device wait that runs
out, a workspace allocation beyond the context's cap, and a cancellation
between batches must each reach the caller as a status (HFX_ERR_TIMEOUT,
HFX_ERR_OOM, SearchCancelled), and the context must stay usable: the next
search returns the same results as before the failure.

The timeout is made on purpose with HFX_TEST_HOLD_LOCK=1: every scorer CTA
starts with one member's admission lock held by nobody and gives up on it
after its bounded number of attempts, records the timeout in the error word
and finishes its work.  Nothing waits without a bound, and no kernel traps."""
import threading

import numpy as np
import pytest

from hfx_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def engine(gpulib, tiny):
    import hfx_gb300
    prot, sp, _ = tiny
    eng = hfx_gb300.Engine(0)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    yield eng, prot, sp.subset(np.arange(48))
    eng.close()


@pytest.mark.parametrize("mode,prec", [(1, 1), (1, 0), (2, 1)])
def test_lock_wait_runs_out_reports_timeout(engine, monkeypatch, mode, prec):
    import hfx_gb300
    eng, prot, sp = engine
    p = hfx_gb300.default_params(top_n=10, batch_mode=mode, precision=prec)
    ref = eng.search(sp, p)
    monkeypatch.setenv("HFX_TEST_HOLD_LOCK", "1")
    with pytest.raises(hfx_gb300.HfxError) as ei:
        eng.search(sp, p)
    assert ei.value.code == hfx_gb300.HFX_ERR_TIMEOUT
    assert "timed out" in str(ei.value)
    monkeypatch.delenv("HFX_TEST_HOLD_LOCK")
    again = eng.search(sp, p)
    assert np.array_equal(again.key, ref.key)
    assert np.array_equal(again.score.view(np.uint32), ref.score.view(np.uint32))


def test_lock_wait_in_modification_scorer(gpulib, tiny, monkeypatch):
    import hfx_gb300
    prot, sp, _ = tiny
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
        eng.set_mods("MSTY", [15.995, 79.966, 79.966, 79.966], 4, False)
        sub = sp.subset(np.arange(12))
        p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1, search_plain=0, search_mods=1)
        ref = eng.search(sub, p)
        monkeypatch.setenv("HFX_TEST_HOLD_LOCK", "1")
        with pytest.raises(hfx_gb300.HfxError) as ei:
            eng.search(sub, p)
        assert ei.value.code == hfx_gb300.HFX_ERR_TIMEOUT
        monkeypatch.delenv("HFX_TEST_HOLD_LOCK")
        assert np.array_equal(eng.search(sub, p).key, ref.key)
    finally:
        eng.close()


def test_workspace_cap_reports_oom(gpulib, tiny):
    import hfx_gb300
    prot, sp, _ = tiny
    sub = sp.subset(np.arange(32))
    eng = hfx_gb300.Engine(0)
    try:
        eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
        p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1)
        assert eng.set_workspace_limit(1 << 16) >= 0
        with pytest.raises(hfx_gb300.HfxError) as ei:
            eng.search(sub, p)
        assert ei.value.code == hfx_gb300.HFX_ERR_OOM
        used = eng.set_workspace_limit(0)
        assert used <= 1 << 16
        ref = eng.search(sub, p)
        # a cap at what that search holds lets the same search run again
        held = eng.set_workspace_limit(0)
        eng.set_workspace_limit(held)
        again = eng.search(sub, p)
        assert np.array_equal(again.key, ref.key)
        eng.set_workspace_limit(0)
    finally:
        eng.close()


def test_cancel_between_batches(engine):
    import hfx_gb300
    eng, prot, sp = engine
    p = hfx_gb300.default_params(top_n=10, batch_mode=1, precision=1)
    whole = eng.search_batches(sp, p, batch=16)
    one = eng.search(sp, p)
    assert np.array_equal(whole.key, one.key) and np.array_equal(whole.ncand, one.ncand)
    stop = threading.Event()
    seen = []

    def after(i, lo, hi):
        seen.append((lo, hi))
        if i == 1:
            stop.set()
    with pytest.raises(hfx_gb300.SearchCancelled) as ei:
        eng.search_batches(sp, p, batch=16, cancel=stop, on_batch=after)
    assert seen == [(0, 16), (16, 32)] and ei.value.done == 32
    assert np.array_equal(ei.value.partial.key, one.key[:32])
    # the context still searches normally
    assert np.array_equal(eng.search(sp, p).key, one.key)
