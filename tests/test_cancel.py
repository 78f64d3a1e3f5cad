"""Cancellation between batches, host logic only (no device work): a fake
search stands in for hfx_search_host, so the batching, the cancel check
before each batch and the partial result run on the CPU."""
import threading

import numpy as np
import pytest

import hfx_gb300
from hfx_gb300 import synth


class _FakeEngine(hfx_gb300.Engine):
    def __init__(self):  # no CUDA context
        self.h = None
        self.calls = []

    def search(self, spectra, params=None):
        n = len(spectra)
        self.calls.append(n)
        base = np.asarray(spectra.pcr, np.float32)
        return hfx_gb300.SearchResult(np.repeat(base[:, None], 3, 1), np.arange(3 * n, dtype=np.uint64).reshape(n, 3),
                                      np.zeros((n, 3), np.uint32), np.full(n, 7, np.int64))


class _P:
    top_n = 3


def test_batches_concatenate_in_order():
    _, sp, _ = synth.workload("tiny", n_spectra=10)
    eng = _FakeEngine()
    res = eng.search_batches(sp, _P(), batch=4)
    assert eng.calls == [4, 4, 2]
    assert np.array_equal(res.score[:, 0], sp.pcr.astype(np.float32)) and res.ncand.tolist() == [7] * 10


def test_cancel_stops_before_the_next_batch():
    _, sp, _ = synth.workload("tiny", n_spectra=10)
    eng = _FakeEngine()
    stop = threading.Event()
    with pytest.raises(hfx_gb300.SearchCancelled) as ei:
        eng.search_batches(sp, _P(), batch=4, cancel=stop, on_batch=lambda i, lo, hi: stop.set())
    assert eng.calls == [4] and ei.value.done == 4 and len(ei.value.partial.key) == 4
    stop2 = threading.Event()
    stop2.set()
    with pytest.raises(hfx_gb300.SearchCancelled) as ei:
        _FakeEngine().search_batches(sp, _P(), batch=4, cancel=stop2)
    assert ei.value.done == 0 and ei.value.partial.key.shape == (0, 3)
