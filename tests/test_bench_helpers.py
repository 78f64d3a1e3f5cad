"""The bench's bookkeeping of captured traffic: a capture stays valid while
the code of its kernel's source files is unchanged (comments and whitespace
aside), and is reported stale (no figure) once the code changes."""
import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_traffic_entries_match_the_current_code():
    for (kern, _, _, _), t in bench.TRAFFIC.items():
        assert t["src"] == bench._src_hash(kern), kern
        assert t["bytes"] > 0 and t["inst"] > 0
        assert t["profile"].startswith("profiles/") and os.path.exists(os.path.join(ROOT, t["profile"].split()[0]))


def test_comments_do_not_make_a_capture_stale(tmp_path, monkeypatch):
    src = os.path.join(ROOT, "hfx_gb300", "csrc", "lists.cu")
    copy = tmp_path / "lists.cu"
    shutil.copy(src, copy)
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    monkeypatch.setitem(bench.KERNEL_SRC, "k_test", ["lists.cu"])
    h0 = bench._src_hash("k_test")
    text = copy.read_text()
    copy.write_text("// a new comment\n" + text.replace("\n", "  \n", 3) + "\n/* and another */\n")
    assert bench._src_hash("k_test") == h0
    copy.write_text(text.replace("constexpr int kLowpCands = 4;", "constexpr int kLowpCands = 2;"))
    assert bench._src_hash("k_test") != h0
    monkeypatch.setitem(bench.TRAFFIC, ("k_test", "full", 1, 1), {"src": h0, "bytes": 1, "inst": 1, "profile": "p"})
    tr, note = bench._traffic("k_test", "full", 1, 1)
    assert tr is None and note.startswith("stale")
