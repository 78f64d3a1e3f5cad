"""Benchmark: peptide-spectrum XCorrs/s of the SEQUEST search hot path.

One step = one full search (stages a-e) of one batch of synthetic spectra
against the synthetic database.  Default workload 'full': 20,000 random
proteins, 10,000 spectra at charge 1-4, 50-400 peaks, +-3 Da, 1.0005 Da
bins, top-10, searched by the batched engine over per-step ion lists with
BF16-stored spectra and FP32 rescoring (the top-10 equals the FP32
search's).  `value` times steps whose inputs are already resident in HBM
(hfx_search_device); `e2e` times the same search through hfx_search_host
with pinned host buffers, copies included.  Between timed steps the L2 is
flushed by writing a 512 MB buffer (outside the timed events).

Beside the headline the line carries the plain FP32 path (one launch per
spectrum) timed on the same spectra and its top-10 agreement; `parity`: the
timed search's top-10 keys, FP32 scores and candidate counts compared bit
for bit with the oracle's FP32 search of every spectrum (the +-3 Da
workloads; a sample of the open-window ones) and its agreement with the
FP64 oracle; the oracle timed on the host cores (cpu_baseline); and the
rooflines of the step and of each kernel.

--impl reference times the reference's search restated on the CPU (the
oracle port: the reference's Haskell host and CUDA kernels cannot run on
this machine) on the same spectra, with every host thread, plus a one-thread
figure on a sample.

Multi-GPU: spectra are independent, so each rank searches its own batch
(weak scaling, no collective on the data path); value = all ranks' pairs /
max over ranks of the elapsed time.  `--gpus N` without torchrun re-runs the
command under torchrun.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "peptide-spectrum XCorrs/s"
UNIT = "PSM/s"
KERNELS = {0: "k_score_spectrum", 1: "k_score_lists", 2: "k_score_batched"}

# DRAM bytes (read + write) per launch, from ncu captures (summaries under
# profiles/), keyed by (kernel, workload, precision, spectra).  Each figure
# carries the hash of the kernel's source files at capture time; when the
# source has changed since, the figure is not reported (traffic null, marked
# stale).
_COMMON_SRC = ["hfx_gb300/csrc/device_common.cuh", "hfx_gb300/csrc/batched_common.cuh",
               "hfx_gb300/csrc/lists_device.cuh"]
KERNEL_SRC = {
    "k_gen_lists": ["hfx_gb300/csrc/lists.cu"] + _COMMON_SRC,
    "k_score_lists": ["hfx_gb300/csrc/lists.cu"] + _COMMON_SRC,
    "k_gen_iso_lists": ["hfx_gb300/csrc/iso_lists.cu", "hfx_gb300/csrc/mods_device.cuh"] + _COMMON_SRC,
    "k_score_iso_lists": ["hfx_gb300/csrc/iso_lists.cu", "hfx_gb300/csrc/mods_device.cuh"] + _COMMON_SRC,
}
# Scaled captures: the DRAM bytes (and the warp instructions, `inst`) of one
# launch on the 2,000-spectrum (full) or 1,000-spectrum (mods) case, times
# the ratio of the full-size launch's moved bytes (the run's work counters,
# per-kernel basis below) to the small case's.
TRAFFIC = {
    ("k_gen_lists", "full", 1, 10000): {
        "src": "514a0af75598", "bytes": 2205793354, "inst": 4522799000,
        "profile": "profiles/k_gen_lists_2k_bf16.md (2,000-spectrum capture x 1.729 moved-bytes ratio)"},
    ("k_score_lists", "full", 1, 10000): {
        "src": "514a0af75598", "bytes": 3319129096, "inst": 2310847000,
        "profile": "profiles/k_score_lists_2k_bf16.md (2,000-spectrum capture x 2.482 moved-bytes ratio)"},
    ("k_gen_iso_lists", "mods", 1, 10000): {
        "src": "b9b44833cf01", "bytes": 50181657886, "inst": 91095407000,
        "profile": "profiles/iso_lists_mods1k_bf16.md (1,000-spectrum capture x 3.904 moved-bytes ratio)"},
    ("k_score_iso_lists", "mods", 1, 10000): {
        "src": "b9b44833cf01", "bytes": 62823028595, "inst": 31125280000,
        "profile": "profiles/iso_lists_mods1k_bf16.md (1,000-spectrum capture x 4.815 moved-bytes ratio)"},
}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="full")
    ap.add_argument("--spectra", type=int, default=0, help="override the number of spectra")
    ap.add_argument("--precision", type=int, default=1, help="0 fp32, 1 bf16+rescore, 2 fp16+rescore")
    ap.add_argument("--batch-mode", type=int, default=1,
                    help="0 per-spectrum launches, 1 batched over ion lists, 2 batched fused")
    ap.add_argument("--cpu-sample", type=int, default=-1,
                    help="spectra in the CPU baseline sample (-1: whole 'full' workload, 300 otherwise)")
    ap.add_argument("--agree-sample", type=int, default=-1,
                    help="spectra checked against the FP64 oracle (-1: 1000 for 'full', 200 otherwise)")
    ap.add_argument("--plain-sample", type=int, default=-1,
                    help="spectra timed on the plain FP32 path (-1: all for 'full', 2000 otherwise)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and the FP64 agreement")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 comparison")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--out", default="")
    ap.add_argument("--group-size", type=int, default=0, help="spectra per batched work item (0 = default)")
    ap.add_argument("--chunk", type=int, default=0, help="candidates per batched work item (0 = default)")
    ap.add_argument("--no-graph", action="store_true", help="eager launches instead of CUDA-graph replays")
    ap.add_argument("--evalues", action="store_true",
                    help="also time hfx_search_evalues (the search plus every pair's FP32 score and the fits)")
    ap.add_argument("--shard", action="store_true",
                    help="N > 1: split ONE batch across the ranks by candidate counts (strong scaling) instead of "
                         "one batch per rank (weak scaling)")
    ap.add_argument("--tune", default="auto", choices=["auto", "on", "off"],
                    help="hfx_autotune of group size and work-item size before the warm-up (auto = on "
                         "unless --group-size or --chunk is given)")
    return ap.parse_args()


def _src_hash(kern):
    """Hash of a kernel's source files without their comments and runs of
    whitespace, so that only a change of code marks a capture stale."""
    import hashlib
    import re
    files = KERNEL_SRC.get(kern, ["hfx_gb300/csrc/lists.cu"] + _COMMON_SRC)
    h = hashlib.sha1()
    for f in files:
        with open(os.path.join(ROOT, f), encoding="utf-8") as fh:
            text = fh.read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)  # block comments
        text = re.sub(r"//[^\n]*", " ", text)                 # line comments
        h.update(" ".join(text.split()).encode())
    return h.hexdigest()[:12]


def _traffic(kern, workload, prec, ns, field="bytes"):
    """(bytes or instructions per launch, note) of a captured kernel, None
    when absent or stale."""
    t = TRAFFIC.get((kern, workload, prec, ns))
    if t is None:
        return None, "no capture for this kernel and workload"
    if t["src"] != _src_hash(kern):
        return None, "stale: kernel source changed since the capture"
    return t[field], t["profile"]


def _relaunch(a):
    """--gpus N > 1 without a launcher: re-run this command under torchrun."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={a.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", os.environ.get("MASTER_PORT", "29517")] + sys.argv
    os.execvp(cmd[0], cmd)


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


DESCRIBE = {
    "tiny": "2000 proteins, {n} spectra, +-3 Da, 1.0005 Da bins, top-10",
    "full": "20000 proteins, {n} spectra, +-3 Da, 1.0005 Da bins, top-10",
    "mods": "20000 proteins, {n} spectra, +-3 Da, 1.0005 Da bins, top-10, variable M+15.995 S/T/Y+79.966 up to 3",
    "batch": "20000 proteins, {n} spectra, 80% +-10 ppm / 20% +-500 Da, 1.0005 Da bins, top-10",
    "highres": "20000 proteins, {n} spectra, 80% +-10 ppm / 20% +-500 Da, 0.02 Da bins, top-10",
}


def _samples(a):
    """Workload-dependent default sample sizes of the CPU-side arms: every
    spectrum of the +-3 Da workloads (the oracle searches 10,000 of them in
    seconds on the host cores), samples of the open-window ones."""
    full = a.workload in ("full", "tiny")
    cpu = a.cpu_sample if a.cpu_sample >= 0 else (1 << 30 if full else 300)
    agree = a.agree_sample if a.agree_sample >= 0 else (1 << 30 if full else 200)
    plain = a.plain_sample if a.plain_sample >= 0 else (1 << 30 if full else 2000)
    return cpu, agree, plain


def _workload(name, n, rank):
    from hfx_gb300 import synth
    prot, sp, cfg = synth.workload(name, n_spectra=n or None)
    if rank:
        # each rank its own batch of spectra over the same database
        peps = synth.tryptic_peptides(prot)
        sp = synth.spectra(prot, len(sp), seed=1000 + rank, charge_p={1: 0.05, 2: 0.5, 3: 0.35, 4: 0.10},
                           npeaks=(50, 400), peps=peps)
    return prot, sp, cfg


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _charges(z):
    zm = z - 1.0
    mc = zm if zm >= 1.0 else 1.0
    ch = int(np.rint(mc))
    return ch if 1 <= ch <= 4 else 0


def _bytes_per_psm(eng, rows_dtype_bytes, wb, we, lens, charges, idx_tc_tn, rng, n=4000):
    """Algorithmic bytes per pair: U*s + L + 16 (U = distinct in-range ion
    bins, s = stored element size, L = residue bytes, 16 = r, tc, tn, id),
    averaged over a random sample of the pairs the step scores."""
    import torch
    counts = (we - wb).astype(np.int64)
    ok = np.nonzero(counts > 0)[0]
    sp = rng.choice(ok, n, p=counts[ok] / counts[ok].sum())
    pos = (wb[sp] + (rng.random(n) * counts[sp]).astype(np.int64)).astype(np.int32)
    d = torch.device("cuda")
    cap = 8192
    bins = torch.zeros((n, cap), dtype=torch.int32, device=d)
    lvl = torch.zeros((n, cap), dtype=torch.uint8, device=d)
    cnt = torch.zeros(n, dtype=torch.int32, device=d)
    eng.ion_bins(torch.from_numpy(pos).to(d), torch.from_numpy(charges[sp].astype(np.int32)).to(d),
                 torch.from_numpy(lens[sp].astype(np.int32)).to(d), cap, bins, lvl, cnt)
    U = cnt.cpu().numpy().astype(np.float64)
    tc, tn = idx_tc_tn
    L = (tn[pos] - tc[pos]).astype(np.float64)
    return float(np.mean(U * rows_dtype_bytes + L + 16)), float(U.mean())


def _okw(cfg):
    """Oracle search settings of a workload."""
    return dict(bw=cfg["bin_width"], custom_bw=bool(cfg.get("custom_bin_width", 0)), ppm=cfg.get("tol_ppm", 0),
                ion_bw=cfg["bin_width"] if cfg.get("ion_bins_custom", 0) else 0.0)


def _pkw(cfg):
    """Engine search settings of a workload."""
    return dict(bin_width=cfg["bin_width"], tol_ppm=cfg.get("tol_ppm", 0),
                custom_bin_width=cfg.get("custom_bin_width", 0), ion_bins_custom=cfg.get("ion_bins_custom", 0))


def _oracle_inputs(prot, cfg):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from hfx_gb300 import synth
    O.build()
    mt = O.mass_table(True, synth.static_mods())
    d = {k: v for k, v in synth.DIGEST.items() if k != "mono"}
    r, tc, tn = O.digest(prot.seq, prot.seg, mt, **d)
    idx = O.sort_idx(r)
    ma = cfg.get("ma", "").encode()
    ions = O.pack_ions(prot.seq, ma)
    mods = dict(ma=ma, ma_mass=cfg.get("ma_mass", ()), max_ma=cfg.get("max_ma", 0))
    return O, (ions, mt, r, tc, tn, idx), mods


def run_reference(a, rank, world):
    """CPU arm: the oracle port of the reference search on the same spectra as
    the GPU arm, all host threads; rank 0 only.  Beside it, the same search on
    one thread over a bounded sample."""
    if rank != 0:
        return
    prot, sp, cfg = _workload(a.workload, a.spectra, 0)
    O, db, mods = _oracle_inputs(prot, cfg)
    cpu_n, _, _ = _samples(a)
    sample = sp if cpu_n >= len(sp) else sp.subset(np.arange(cpu_n))
    threads = os.cpu_count() or 1
    kw = dict(topn=cfg["top_n"], **_okw(cfg), **mods)
    warm = sample.subset(np.arange(min(50, len(sample))))
    for _ in range(max(1, a.warmup)):
        O.search(*db, warm, nthreads=threads, **kw)
    t0 = time.perf_counter()
    psm = 0
    for _ in range(a.steps):
        res = O.search(*db, sample, nthreads=threads, **kw)
        psm += int(res[4].sum())
    dt = time.perf_counter() - t0
    v = psm / dt
    # one thread, a bounded sample (about a second of work)
    one = sample.subset(np.arange(min(len(sample), 200)))
    t1 = time.perf_counter()
    r1 = O.search(*db, one, nthreads=1, **kw)
    dt1 = time.perf_counter() - t1
    whole = len(sample) == len(sp)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1000 * dt / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{a.workload}: " + DESCRIBE.get(a.workload, "{n} spectra").format(n=len(sp))
                       + ("" if whole else f" ({len(sample)} of {len(sp)} spectra per step)"),
                       "psm_per_step": psm // a.steps},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": (f"all {len(sp)} spectra" if whole else f"{len(sample)} of {len(sp)} spectra")
                             + f" of the {a.workload} workload per step"},
            "cpu_1thread": {"value": float(r1[4].sum()) / dt1, "unit": UNIT, "cores": 1, "kind": "port",
                            "sample": f"first {len(one)} spectra, {int(r1[4].sum())} pairs, {dt1:.2f} s"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _cpu_baseline(a, O, db, mods, sp, cfg):
    """The oracle (ref32, the reference's FP32 operation order) timed on the
    host cores; returns the baseline figure and the oracle's result."""
    n = min(len(sp), a.cpu_sample)
    sample = sp if n == len(sp) else sp.subset(np.arange(n))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    res = O.search(*db, sample, topn=cfg["top_n"], nthreads=threads, **_okw(cfg), **mods)
    dt = time.perf_counter() - t0
    return {"value": float(res[4].sum()) / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {len(sample)} of {len(sp)} spectra, {int(res[4].sum())} pairs, {dt:.1f} s"}, res


def _parity(res32, key, score, ncand):
    """Bitwise comparison of the GPU result with the oracle's FP32 result on
    the spectra the oracle searched: per spectrum, the top-N keys (candidate
    set and order), the FP32 scores and the candidate counts."""
    s32, k32, n32 = res32[0], res32[2], res32[4]
    n = len(k32)
    keys = np.all(k32 == key[:n], axis=1)
    scores = np.all(s32.view(np.uint32) == score[:n].view(np.uint32), axis=1)
    counts = n32.astype(np.int64) == ncand[:n].astype(np.int64)
    return {"spectra": int(n), "keys_bitexact": float(keys.mean()), "scores_bitexact": float(scores.mean()),
            "candidate_counts_equal": float(counts.mean())}


def _agreement(a, O, db, mods, sp, cfg, key, score):
    """Top-N agreement of the GPU result with the FP64 oracle: the fraction
    of spectra whose top-N candidates (keys, in order) match, and the
    largest relative XCorr difference of the matched entries."""
    n = min(len(sp), a.agree_sample)
    sample = sp if n == len(sp) else sp.subset(np.arange(n))
    threads = os.cpu_count() or 1
    _, s64, k64, _, _ = O.search(*db, sample, topn=cfg["top_n"], prec=3, nthreads=threads, **_okw(cfg), **mods)
    same_order = np.all(k64 == key[:n], axis=1)
    same_set = np.array([set(k64[i]) == set(key[i]) for i in range(n)])
    ok = (k64 != np.iinfo(np.uint64).max) & (k64 == key[:n])
    denom = np.maximum(np.abs(s64[ok]), 1e-30)
    rel = np.abs(score[:n][ok].astype(np.float64) - s64[ok]) / denom
    return {"spectra": n, "top_order": float(same_order.mean()), "top_set": float(same_set.mean()),
            "max_rel_err": float(rel.max()) if rel.size else 0.0,
            "mean_rel_err": float(rel.mean()) if rel.size else 0.0}


def _timed(eng, dev, p, out, steps, flush, stream):
    """Device time of `steps` searches, L2 flushed before each (outside the events)."""
    import torch
    total_ms = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.search_device(dev, p, out)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    return total_ms


def main():
    a = _args()
    rank, world, local = _dist()
    if a.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return _relaunch(a)
    if world != a.gpus:
        print(f"bench: --gpus {a.gpus} but WORLD_SIZE {world}; using {world}", file=sys.stderr)
    if a.impl == "reference":
        return run_reference(a, rank, world)
    import torch
    import hfx_gb300
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    strong = a.shard and world > 1
    prot, sp, cfg = _workload(a.workload, a.spectra, 0 if strong else rank)
    from hfx_gb300 import synth
    eng = hfx_gb300.Engine(local)
    eng.build_db(prot.seq, prot.seg, static_add=synth.static_mods(), **synth.DIGEST)
    has_mods = bool(cfg.get("ma"))
    if has_mods:
        eng.set_mods(cfg["ma"], cfg["ma_mass"], cfg["max_ma"])
    stream = torch.cuda.current_stream()
    eng.set_stream(stream.cuda_stream)
    prec, mode = a.precision, a.batch_mode
    shard_range = None
    if strong:
        # this rank's run of the batch, balanced by the windows' candidate counts
        from hfx_gb300 import shard
        d0 = torch.device("cuda", local)
        dv = {k: torch.from_numpy(v).to(d0) for k, v in zip(("mz", "it", "off", "pcr", "z", "tol"), sp.arrays())}
        b0 = torch.empty(len(sp), dtype=torch.int32, device=d0)
        e0 = torch.empty(len(sp), dtype=torch.int32, device=d0)
        eng.find_windows(dv, hfx_gb300.default_params(top_n=cfg["top_n"], **_pkw(cfg)), b0, e0)
        nc = np.maximum((e0 - b0).cpu().numpy().astype(np.int64), 0)
        shard_range = shard.partition(nc, world)[rank]
        sp = sp.subset(np.arange(*shard_range))
    cpu_n, agree_n, plain_n = _samples(a)
    a.cpu_sample, a.agree_sample = cpu_n, agree_n
    graph = int(mode != 0 and not a.no_graph)
    # candidates rescored in FP32: the top-50 at 0.02 Da (its configuration asks for them), 32 elsewhere
    rk = (50 if a.workload == "highres" else 32) if prec else 0
    p = hfx_gb300.default_params(top_n=cfg["top_n"], precision=prec, batch_mode=mode, rescore_k=rk,
                                 group_size=a.group_size, chunk=a.chunk, use_graph=graph, **_pkw(cfg))
    # stage events and work counters need the eager launches
    p_prof = hfx_gb300.default_params(top_n=cfg["top_n"], precision=prec, batch_mode=mode,
                                      rescore_k=rk, group_size=a.group_size, chunk=a.chunk,
                                      **_pkw(cfg))
    d = torch.device("cuda", local)
    dev = dict(mz=torch.from_numpy(sp.mz).to(d), it=torch.from_numpy(sp.it).to(d),
               off=torch.from_numpy(sp.off).to(d), pcr=torch.from_numpy(sp.pcr).to(d),
               z=torch.from_numpy(sp.z).to(d), tol=torch.from_numpy(sp.tol).to(d))
    ns, tn_ = len(sp), cfg["top_n"]

    def outputs():
        return dict(score=torch.empty((ns, tn_), dtype=torch.float32, device=d),
                    key=torch.empty((ns, tn_), dtype=torch.int64, device=d),
                    pep=torch.empty((ns, tn_), dtype=torch.int32, device=d),
                    ncand=torch.empty(ns, dtype=torch.int64, device=d))
    out = outputs()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=d)
    tuned = None
    if mode != 0 and a.group_size == 0 and a.chunk == 0 and a.tune in ("on", "auto"):
        ms_t = eng.autotune(dev, p, out, reps=2)
        p_prof.group_size, p_prof.chunk = p.group_size, p.chunk
        tuned = {"group_size": p.group_size, "chunk": p.chunk, "ms": ms_t}
    for _ in range(a.warmup):
        eng.search_device(dev, p, out)
    torch.cuda.synchronize()
    psm_step = int(out["ncand"].sum().item())
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    total_ms = _timed(eng, dev, p, out, a.steps, flush, stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    # the timed searches' own result (the stage-event pass below overwrites `out`)
    key = out["key"].cpu().numpy().view(np.uint64)
    score = out["score"].cpu().numpy()
    ncand = out["ncand"].cpu().numpy()
    psm_all = psm_step
    if world > 1:
        t = torch.tensor([total_ms], device=d)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        c = torch.tensor([psm_step], dtype=torch.int64, device=d)
        torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
        psm_all = int(c.item())
    ms_step = total_ms / a.steps
    value = psm_all / (ms_step / 1000.0)
    # per-stage device times and work counters: the same steps again, with stage events
    eng.set_profiling(True)
    eng.stage_stats(reset=True)
    eng.counters(reset=True)
    eng.mod_counters(reset=True)
    _timed(eng, dev, p_prof, out, a.steps, flush, stream)
    stats = eng.stage_stats(reset=True)
    work = {k: v // a.steps for k, v in eng.counters(reset=True).items()}
    mwork = {k: v // a.steps for k, v in eng.mod_counters(reset=True).items()}
    eng.set_profiling(False)
    eager_same = bool(np.array_equal(out["key"].cpu().numpy().view(np.uint64), key))
    # e2e through the host-buffer C ABI (pinned buffers, copies in the timed region)
    pin = {k: torch.from_numpy(v).pin_memory() for k, v in
           dict(mz=sp.mz, it=sp.it, off=sp.off, pcr=sp.pcr, z=sp.z, tol=sp.tol).items()}

    class Pinned:
        def arrays(self):
            return tuple(pin[k].numpy() for k in ("mz", "it", "off", "pcr", "z", "tol"))
    h2d = sum(int(v.numel() * v.element_size()) for v in pin.values())
    d2h = ns * tn_ * (4 + 8 + 4) + ns * 8
    r_e2e = eng.search(Pinned(), p)
    torch.cuda.synchronize()
    e2e_same = bool(np.array_equal(r_e2e.key, key) and np.array_equal(r_e2e.score.view(np.uint32),
                                                                       score.view(np.uint32)))
    e2e_tot = 0.0
    for _ in range(a.e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        eng.search(Pinned(), p)
        e2e_tot += time.perf_counter() - t1
    e2e_value = psm_all / (e2e_tot / a.e2e_steps)
    # the plain FP32 path (one launch per spectrum) on the same spectra
    plain = None
    if not a.no_plain and not has_mods:
        # the plain FP32 path: one launch per spectrum (rows beyond 8192 bins
        # always take the batched list path, there in FP32)
        p0 = hfx_gb300.default_params(top_n=tn_, precision=0, batch_mode=0, **_pkw(cfg))
        n_pl = min(ns, plain_n)
        sub = sp if n_pl == ns else sp.subset(np.arange(n_pl))
        dev0 = dev if n_pl == ns else dict(mz=torch.from_numpy(sub.mz).to(d), it=torch.from_numpy(sub.it).to(d),
                                           off=torch.from_numpy(sub.off).to(d), pcr=torch.from_numpy(sub.pcr).to(d),
                                           z=torch.from_numpy(sub.z).to(d), tol=torch.from_numpy(sub.tol).to(d))
        out0 = dict(score=torch.empty((n_pl, tn_), dtype=torch.float32, device=d),
                    key=torch.empty((n_pl, tn_), dtype=torch.int64, device=d),
                    pep=torch.empty((n_pl, tn_), dtype=torch.int32, device=d),
                    ncand=torch.empty(n_pl, dtype=torch.int64, device=d))
        eng.search_device(dev0, p0, out0)
        torch.cuda.synchronize()
        psm0 = int(out0["ncand"].sum().item())
        n0 = max(1, min(3, a.steps))
        ms0 = _timed(eng, dev0, p0, out0, n0, flush, stream) / n0
        k0 = out0["key"].cpu().numpy().view(np.uint64)
        s0 = out0["score"].cpu().numpy()
        v0 = psm0 / (ms0 / 1000.0)
        plain = {"value": v0, "unit": UNIT, "ms_per_step": ms0, "spectra": n_pl, "pairs": psm0,
                 "speedup": (psm_step / (ms_step / 1000.0)) / v0,
                 "top_agreement": float(np.mean(np.all(k0 == key[:n_pl], axis=1))),
                 "scores_bitexact": bool(np.array_equal(s0.view(np.uint32), score[:n_pl].view(np.uint32)))}
    # roofline of the dominant kernel
    stage = "mods" if has_mods and stats["mods"][0] > stats["score"][0] else "score"
    mod_kern = "k_score_iso_lists" if mode == 1 else "k_score_mods"
    kern = mod_kern if stage == "mods" else KERNELS[mode if mode in KERNELS else 1]
    if has_mods and mode == 0:
        kern = mod_kern if stage == "mods" else "k_score_batched"
    rng = np.random.Generator(np.random.PCG64(7))
    r, tc, tn, idx, mt = eng.db_export()
    bsz = 2 if prec else 4
    b_dev = torch.empty(ns, dtype=torch.int32, device=d)
    e_dev = torch.empty(ns, dtype=torch.int32, device=d)
    eng.find_windows(dev, p, b_dev, e_dev)
    wb = b_dev.cpu().numpy().astype(np.int64)
    we = e_dev.cpu().numpy().astype(np.int64)
    long_rows = bool(cfg.get("custom_bin_width", 0)) and cfg["bin_width"] < 0.5
    if not long_rows:
        rows = torch.empty((ns, 8192), dtype=torch.float32, device=d)
        lens_d = torch.empty(ns, dtype=torch.int32, device=d)
        eng.preprocess(dev, p, 8192, rows, None, None, lens_d, None)
        lens = lens_d.cpu().numpy().astype(np.int64)
        del rows
        charges = np.array([_charges(z) for z in sp.z], np.int64)
        bpp, meanU = _bytes_per_psm(eng, bsz, wb, we, lens, charges, (tc[idx], tn[idx]), rng)
        u_basis = "distinct in-range ion bins, 4000 sampled pairs"
    else:
        # ~10^5-bin rows: U from the run's own counters (list entries streamed
        # per candidate hand-out), L from sampled window positions
        lens = np.where(we > wb, 1, 0)
        meanU = work["entries_streamed"] / max(1, work["candidates"])
        cnt = (we - wb).astype(np.int64)
        ok = np.nonzero(cnt > 0)[0]
        sp_i = rng.choice(ok, 4000, p=cnt[ok] / cnt[ok].sum())
        pos = (wb[sp_i] + (rng.random(4000) * cnt[sp_i]).astype(np.int64))
        meanL = float(np.mean((tn[idx] - tc[idx])[pos]))
        bpp = meanU * bsz + meanL + 16
        u_basis = "list entries streamed per candidate (run counters)"
    # pairs scored by the modification scorer or the plain scorer
    psm_kernel = psm_step
    if stage == "mods":
        psm_kernel = psm_step - int(np.sum(np.where(lens > 0, we - wb, 0)))
    elif has_mods:
        psm_kernel = int(np.sum(np.where(lens > 0, we - wb, 0)))
    peak, peak_kind = _peaks()
    launches_per_step = sum(v[1] for v in stats.values()) / a.steps
    # Per-kernel rooflines.  "moved" bytes are what each kernel reads and
    # writes by design, from the run's own work counters: the generator
    # reads each needed peptide's residues and metadata and writes its lists;
    # the list scorer streams list entries, list metadata and the spectrum
    # tiles it stages; the isoform-list generator and scorer of the
    # modification search likewise, plus their per-isoform records.  The
    # per-pair figure U*s + L + 16 of the search as a
    # whole is reported for the step (`step`), where the benchmark spec's target is
    # defined.
    es = 4 if long_rows else 2
    kern_rows = {}
    stage_of = {"lists": "k_gen_lists" + ("_long" if long_rows else ""), "score": kern, "mods": mod_kern}
    if mode == 1 and has_mods:
        stage_of["mod_lists"] = "k_gen_iso_lists"
    step_ms_all = sum(v[0] for v in stats.values()) / a.steps
    for st, kname in stage_of.items():
        ms_st, nl_st, _ = stats.get(st, (0.0, 0, 0))
        if not nl_st or ms_st <= 0:
            continue
        ms_st /= a.steps
        if st == "lists":
            moved = work["list_entries"] * es + work["residues_read"] + 16 * work["lists"]
            basis = "list entries written + residues read + 16 B per list"
        elif st == "score" and mode == 1:
            moved = work["entries_streamed"] * es + work["tile_bytes"] + 8 * work["candidates"]
            basis = "list entries streamed + spectrum tiles staged + 8 B per candidate"
        elif st == "mod_lists":
            moved = mwork["list_entries"] * 2 + mwork["residues_read"] + 40 * mwork["isoforms"]
            basis = ("isoform list entries written + residues read + 40 B per isoform record (key and slot "
                     "offset written and read back, level lengths)")
        elif st == "mods" and mode == 1:
            moved = mwork["entries_streamed"] * 2 + mwork["tile_bytes"] + 26 * mwork["candidates"]
            basis = ("isoform list entries streamed + spectrum tiles staged + 26 B per isoform hand-out (key, "
                     "slot offset, length, list start)")
        else:
            moved = bpp * (psm_kernel if st == stage else psm_step)
            basis = "U*s + L + 16 per pair (ions rebuilt from residues per pair)"
        tr, tr_note = _traffic(kname, a.workload, prec, ns)
        ach = moved / (ms_st / 1000.0) / 1e9
        kern_rows[kname] = {"stage_ms_per_step": ms_st, "share": ms_st / max(1e-9, step_ms_all),
                            "moved_bytes": moved, "bytes_basis": basis, "achieved": ach, "frac": ach / peak,
                            "traffic": tr, "traffic_note": tr_note}
        # the axis that binds these kernels: warp-instruction issue (4 per
        # SM per cycle at the highest SM clock seen)
        ins, _ = _traffic(kname, a.workload, prec, ns, "inst")
        if ins:
            mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
            peak_i = torch.cuda.get_device_properties(d).multi_processor_count * 4 * mhz * 1e6
            ach_i = ins / (ms_st / 1000.0)
            kern_rows[kname]["issue"] = {"warp_inst_per_launch": ins, "achieved": ach_i, "peak": peak_i,
                                         "unit": "warp instructions/s", "frac": ach_i / peak_i,
                                         "basis": "ncu warp instructions of the small case, scaled like traffic"}
    dom = max(kern_rows, key=lambda k: kern_rows[k]["stage_ms_per_step"]) if kern_rows else kern
    drow = kern_rows.get(dom, {})
    step_ach = bpp * psm_step / (ms_step / 1000.0) / 1e9
    psm_ach = None
    if dom in (kern,):
        psm_ach = bpp * psm_kernel / (drow.get("stage_ms_per_step", ms_step) / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong" if strong else "weak",
        "vs_baseline": None,
        "dtype": ["f32", "bf16", "f16"][prec], "data": "synthetic",
        "config": {"workload": f"{a.workload}: " + DESCRIBE.get(a.workload, "{n} spectra").format(n=ns),
                   "psm_per_step": psm_step,
                   "precision": ["fp32", "bf16 store, fp32 accumulate, fp32 rescore",
                                 "fp16 store, fp32 accumulate, fp32 rescore"][prec]
                   + (f" of the top {rk}" if prec else ""),
                   "batch_mode": ["per-spectrum launches", "batched over ion lists", "batched fused"][mode],
                   "launch": "one CUDA-graph replay per step" if graph else "eager launches",
                   "autotuned": tuned,
                   "l2": "flushed between timed steps (512 MB write)",
                   "stage_ms_per_step": {k: v[0] / a.steps for k, v in stats.items() if v[1]},
                   "work_per_step": work,
                   **({"mod_work_per_step": mwork} if has_mods and mode == 1 else {})},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "result_equals_device_run": e2e_same},
        "gpu_launches": int(launches_per_step * a.steps),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": drow.get("achieved"), "peak": peak, "unit": "GB/s",
                     "frac": drow.get("frac"), "traffic": drow.get("traffic"),
                     "traffic_note": drow.get("traffic_note"), "bytes_basis": drow.get("bytes_basis"),
                     "peak_kind": peak_kind,
                     "binding": "SM instruction issue and shared-memory wavefronts, not DRAM "
                                "(ncu summaries under profiles/)",
                     "issue": drow.get("issue"),
                     "kernels": kern_rows,
                     "step": {"achieved": step_ach, "frac": step_ach / peak, "bytes_per_psm": bpp,
                              "mean_distinct_bins": meanU, "u_basis": u_basis,
                              "basis": "U*s + L + 16 bytes per pair x pairs per step / ms_per_step"},
                     "psm_basis_achieved": psm_ach},
        "clocks": clocks,
        "graph_equals_eager": eager_same,
    }
    if strong:
        line["config"]["shard"] = f"one batch split by candidate counts; rank 0 spectra {shard_range}"
    if a.evalues:
        # the search with E-values (eager), against the same search without
        pe = hfx_gb300.default_params(top_n=cfg["top_n"], precision=prec, batch_mode=1, rescore_k=rk,
                                      group_size=p.group_size, chunk=p.chunk, **_pkw(cfg))
        oe = {k: torch.empty_like(v) for k, v in out.items()}
        oe.update(ev=torch.empty((ns, tn_), dtype=torch.float64, device=d),
                  fit=torch.empty((ns, 3), dtype=torch.float64, device=d))
        eng.search_evalues(dev, pe, oe)
        torch.cuda.synchronize()
        n_e = max(1, min(3, a.steps))
        t_ev = t_plain = 0.0
        for _ in range(n_e):
            for which in (0, 1):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                if which:
                    eng.search_evalues(dev, pe, oe)
                else:
                    eng.search_device(dev, pe, out)
                e1.record(stream)
                e1.synchronize()
                if which:
                    t_ev += e0.elapsed_time(e1)
                else:
                    t_plain += e0.elapsed_time(e1)
        fitted = oe["fit"][:, 2].cpu().numpy()
        line["evalues"] = {"ms_per_search": t_ev / n_e, "ms_search_alone": t_plain / n_e,
                           "ratio": t_ev / max(1e-9, t_plain), "spectra_with_fit": float(np.mean(fitted >= 2)),
                           "launch": "eager",
                           "top_keys_equal": bool(np.array_equal(oe["key"].cpu().numpy().view(np.uint64), key))}
    if plain is not None:
        line["plain_fp32"] = plain
    if rank == 0 and not a.no_cpu:
        O, db, mods = _oracle_inputs(prot, cfg)
        line["cpu_baseline"], res32 = _cpu_baseline(a, O, db, mods, sp, cfg)
        # rescored FP32 scores and keys against the oracle's FP32 search
        if prec == 0 or rk >= cfg["top_n"]:
            line["parity"] = _parity(res32, key, score, ncand)
        line["fp64_agreement"] = _agreement(a, O, db, mods, sp, cfg, key, score)
        if "parity" in line:
            line["parity"].update({"fp64_top_order": line["fp64_agreement"]["top_order"],
                                   "fp64_max_rel_err": line["fp64_agreement"]["max_rel_err"]})
    if rank == 0:
        s = json.dumps(line)
        print(s, flush=True)
        if a.out:
            with open(a.out, "w") as f:
                f.write(s + "\n")
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
