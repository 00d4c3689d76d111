"""Benchmark of the POA hot path on GB300 (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload batch_10k|uneven_2k|single_500|long_10k]

A step is one pass of the path over one batch: every read of every window
aligned (graph-to-sequence DP + traceback) and added to its window's graph
(AddAlignment + topological sort), then each window's consensus.  The
default workload is the 10,000-window polishing batch (450-550 nt windows,
depth 10-60, OV convex 5/-4/-8/-6/-10/-4), seeded synthetic reads.

value     windows/s of the persistent kernel with the inputs resident in HBM
          (CUDA events on the launching stream).
e2e       windows/s through the public batch API from pinned host buffers:
          upload, kernel, consensus download, every step.
plain     windows/s of the one-window-per-launch form on a sample.
roofline  HBM view: algorithmic bytes (the 4-bit traceback state of every
          cell) per second against the measured copy bandwidth; int_roofline
          is the integer-pipe view (max/add operations per cell: linear
          2d+1, affine 3d+3, convex 5d+4, +1 for SW, d the row's
          predecessors, against a measured max/add rate), the bound that
          applies.
cpu_baseline  the reference's own library (oracle/ref_bench.cpp over the
          reference sources: its SimdAlignmentEngine on an AVX2 host, its
          SisdAlignmentEngine elsewhere), one window per host thread, on a
          bounded sample of the same workload; the C oracle (the reference
          algorithm restated in C) timed beside it.  Where the reference
          sources are not staged, the C oracle alone.
parity    a sample of the timed workload rerun with alignments returned,
          every read's score and alignment and every consensus compared with
          the oracle.

Under torchrun every rank runs its own batch (weak scaling: windows are
independent and are sharded with no collective); value is the sum of the
windows over the max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from spoa_gb300 import synth  # noqa: E402

# tiles chosen by the tuner are kept per device model for later runs
os.environ.setdefault("SPOA_GB300_TILE_CACHE",
                      os.path.join(ROOT, "spoa_gb300", "_build", "tile_cache.txt"))

OPS = {0: (2, 1), 1: (3, 3), 2: (5, 4)}  # per cell: a * preds + b (SW adds 1)
# score width the kernels compute in (the reference's width rule, per read)
DTYPES = {"batch_10k": "int16", "single_500": "int16", "long_10k": "int32",
          "uneven_2k": "int16/int32"}
TRACEBACK_BYTES_PER_CELL = 0.5          # 4-bit traceback code per DP cell


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch_10k",
                    choices=["batch_10k", "uneven_2k", "single_500", "long_10k", "serve"])
    ap.add_argument("--rates", default="1000,10000,50000",
                    help="serve: offered loads in windows/s")
    ap.add_argument("--serve-windows", type=int, default=600,
                    help="serve: windows per offered load")
    ap.add_argument("--windows", type=int, default=0, help="override the window count")
    ap.add_argument("--long-reads", type=int, default=0,
                    help="long_10k: only the first N reads of the window (a small case)")
    ap.add_argument("--plain-sample", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--windows-per-cta", type=int, default=1, choices=[1, 2, 4],
                    help="windows in flight per CTA (16-bit windows)")
    ap.add_argument("--cluster", type=int, default=0, choices=[0, 1, 2, 4, 8],
                    help="0: long 32-bit rows on thread-block clusters; 1: one CTA per "
                         "window; 2, 4, 8: CTAs per cluster")
    ap.add_argument("--parity-windows", type=int, default=256,
                    help="windows rerun with alignments and checked against the oracle")
    ap.add_argument("--no-resident", action="store_true",
                    help="serve: launch every window instead of the resident kernel")
    ap.add_argument("--tile", default="",
                    help="CPTxTHREADS: force the tile of every pass (no tuner)")
    return ap.parse_args()


def shard_start(n_per_rank: int, rank: int) -> int:
    """First window id of a rank: ranks own disjoint, equally sized ranges of
    independent windows (weak scaling; no data crosses ranks)."""
    return rank * n_per_rank


def max_over_ranks(value: float, dist, device: str) -> float:
    """The step time every rank reports is the maximum over ranks."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def common_config(cfg: dict, world: int) -> dict:
    """The config keys both arms print (the workload, not the GPU's tile)."""
    return dict(cfg, parallelism=f"windows sharded over {world} GPU(s), no collective",
                l2="inputs and per-CTA arenas larger than L2 (129 MB)")


def workload(name: str, n_override: int, rank: int, long_reads: int = 0):
    """Returns (windows, type, params, per-window types, strand flags, config)."""
    if name == "batch_10k":
        n = n_override or 10000
        wins = synth.batch_windows(n, start=shard_start(n, rank))
        typ, params = synth.SCORING["batch_10k"]
        cfg = {"workload": "batch_10k: 10,000 polishing windows, L~U[450,550], depth U[10,60], "
                           "8% error, 20% truncated reads, OV convex 5/-4/-8/-6/-10/-4",
               "windows": n}
        return wins, typ, params, None, None, cfg
    if name == "uneven_2k":
        n = n_override or 2000
        wins = synth.uneven_windows(n, start=shard_start(n, rank))
        _, params = synth.SCORING["uneven_2k"]
        cfg = {"workload": "uneven_2k: 2,000 windows, L log-uniform [100,5000], depth U[5,100], "
                           "NW/OV per window, strand-ambiguous, affine 5/-4/-8/-6", "windows": n}
        return (wins, 1, params, [w.type for w in wins], [1] * len(wins), cfg)
    if name == "single_500":
        wins = [synth.single_500(1 + rank)]
        typ, params = synth.SCORING["single_500"]
        return wins, typ, params, None, None, {"workload": "single_500: one 500-nt window, 30 "
                                                            "reads, NW affine", "windows": 1}
    wins = [synth.long_10k(2 + rank)]
    cfg = {"workload": "long_10k: one 10-kb window, 40 reads 2-10 kb, SW convex", "windows": 1}
    if long_reads:
        wins[0].reads = wins[0].reads[:long_reads]
        cfg["reads"] = long_reads
    typ, params = synth.SCORING["long_10k"]
    return wins, typ, params, None, None, cfg


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i",
                 os.environ.get("LOCAL_RANK", "0")],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().split("\n"):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[4 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def traffic_per_cell():
    """DRAM bytes per DP cell from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh).get("dram_bytes_per_cell")
    return None


def _types_strands(wins, typ, wtypes, wstrand):
    types = wtypes if wtypes is not None else [typ] * len(wins)
    strands = wstrand if wstrand is not None else [0] * len(wins)
    return types, strands


def _sample_size(wins, seconds, per_window, threads, floor):
    return int(min(len(wins), max(floor, seconds / max(per_window, 1e-6) * threads)))


def reference_cpu(wins, typ, params, wtypes, wstrand, seconds, threads, want_consensus=False):
    """The reference's own library on `threads` host threads over a sample of
    the workload sized to about `seconds`; None when it is not built."""
    from oracle import pyoracle as po
    if po.reference_bench() is None:
        return None
    types, strands = _types_strands(wins, typ, wtypes, wstrand)
    k = min(len(wins), threads)
    probe = po.run_reference_bench([w.reads for w in wins[:k]], types[:k], strands[:k], params,
                                   threads)
    per_window = probe["seconds"] / max(k, 1) * threads
    n = _sample_size(wins, seconds, per_window, threads, k)
    rec = po.run_reference_bench([w.reads for w in wins[:n]], types[:n], strands[:n], params,
                                 threads, want_consensus=want_consensus)
    rec["n"] = n
    return rec


def cpu_baseline(wins, typ, params, wtypes, wstrand, seconds):
    """The reference library (kind "reference") and the C oracle (kind
    "port") on all host threads, each on a bounded sample of the workload."""
    from oracle import pyoracle as po
    threads = os.cpu_count() or 1
    po.lib()
    # the port: estimate the cost of one window per thread, then size the sample
    probe = wins[:threads]
    t0 = time.perf_counter()
    _run_oracle(po, probe, typ, params, wtypes, wstrand, threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    per_window = dt / max(len(probe), 1) * threads
    n = _sample_size(wins, seconds, per_window, threads, len(probe))
    sample = wins[:n]
    secs = []
    t0 = time.perf_counter()
    cons, cells = _run_oracle(po, sample, typ, params, wtypes, wstrand, threads, secs)
    dt = time.perf_counter() - t0
    secs.sort()
    pct = lambda f: secs[min(len(secs) - 1, int(f * len(secs)))] if secs else None  # noqa: E731
    port = {"value": n / dt, "unit": "windows/s", "cores": threads, "kind": "port",
            "sample": f"first {n} windows of the workload, {dt:.1f} s, "
                      f"{cells / dt / 1e9:.3f} GCUPS",
            "window_seconds_p50": pct(0.50), "window_seconds_p99": pct(0.99),
            "consensus": cons, "n": n}
    ref = reference_cpu(wins, typ, params, wtypes, wstrand, seconds, threads,
                        want_consensus=True)
    if ref is None:
        return port
    rn = ref.pop("n")
    rcons = ref.pop("consensus")
    out = {"value": rn / ref["seconds"], "unit": "windows/s", "cores": ref["threads"],
           "kind": "reference",
           "engine": "spoa " + ("SimdAlignmentEngine" if ref["engine"] == "simd"
                                else "SisdAlignmentEngine") + " (the reference's own library, "
                                "built from its sources on this host)",
           "sample": f"first {rn} windows of the workload, {ref['seconds']:.1f} s, "
                     f"{ref['cells'] / ref['seconds'] / 1e9:.3f} GCUPS",
           "window_seconds_p50": ref["window_seconds_p50"],
           "window_seconds_p99": ref["window_seconds_p99"],
           "reference_consensus": rcons, "reference_n": rn,
           "consensus": port.pop("consensus"), "n": port.pop("n"), "port": port}
    return out


def _run_oracle(po, wins, typ, params, wtypes, wstrand, threads, secs=None):
    """The oracle on host threads; secs (a list) gets per-window wall times."""
    if wtypes is None:
        return po.batch_run(typ, *params, [w.reads for w in wins], n_threads=threads,
                            window_seconds=secs)
    # per-window type/strand: group by (type, strand)
    cons = [None] * len(wins)
    cells = 0
    groups = {}
    for k, w in enumerate(wins):
        groups.setdefault((wtypes[k], wstrand[k]), []).append(k)
    for (t, s), idx in groups.items():
        c, ce = po.batch_run(t, *params, [wins[k].reads for k in idx], strand_ambiguous=bool(s),
                             n_threads=threads, window_seconds=secs)
        cells += ce
        for k, cc in zip(idx, c):
            cons[k] = cc
    return cons, cells


def flatten(wins, pinned: bool):
    reads = [r for w in wins for r in w.reads]
    lens = np.fromiter((len(r) for r in reads), np.uint64, len(reads))
    off = np.zeros(len(reads) + 1, np.uint64)
    np.cumsum(lens, out=off[1:])
    blob = b"".join(reads)
    wro = np.zeros(len(wins) + 1, np.uint32)
    wro[1:] = np.cumsum([len(w.reads) for w in wins])
    seqs = np.frombuffer(blob + b"\0", np.uint8)
    if pinned:
        try:
            import torch
            t = torch.empty(seqs.size, dtype=torch.uint8, pin_memory=True)
            host = t.numpy()
            host[:] = seqs
            seqs = host
            seqs._keep = t  # noqa: SLF001
        except Exception:  # noqa: BLE001
            pass
    return seqs, off, wro


def int_peaks():
    """Integer max/add rates measured in this run: the 32-bit forms and the
    16x2 forms (lane-operations per second), or (None, None)."""
    try:
        import ctypes as C
        pl = C.CDLL(os.path.join(ROOT, "spoa_gb300", "libspoa_peak.so"))
        pl.spoa_gb300_int_peak_ops.restype = C.c_double
        pl.spoa_gb300_int_peak_ops16x2.restype = C.c_double
        p32 = pl.spoa_gb300_int_peak_ops(4096)
        p16 = pl.spoa_gb300_int_peak_ops16x2(4096)
        return (p32 if p32 > 0 else None), (p16 if p16 > 0 else None)
    except (OSError, AttributeError):
        return None, None


def parity_sample(sg, wins, typ, params, wtypes, wstrand, k, device):
    """The first k windows rerun with alignments returned; every read's
    score, strand and alignment and every consensus compared with the
    oracle (run on host threads: the ctypes calls release the GIL)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import pyoracle as po
    k = min(k, len(wins))
    if k <= 0:
        return None
    types, strands = _types_strands(wins, typ, wtypes, wstrand)
    res = sg.batch_poa([w.reads for w in wins[:k]], typ, *params, window_types=types[:k],
                       window_strand=strands[:k], want_alignments=True, device=device)
    po.lib()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        refs = list(ex.map(lambda j: po.run_window(types[j], *params, wins[j].reads,
                                                   strand_ambiguous=bool(strands[j]),
                                                   with_msa=False), range(k)))
    scores = aligns = cons = True
    r0 = 0
    for j, ref in enumerate(refs):
        n = len(wins[j].reads)
        scores &= res.scores[r0:r0 + n].tolist() == ref.scores and \
            res.reversed[r0:r0 + n].tolist() == ref.reversed
        aligns &= all(np.array_equal(a, b) for a, b in zip(res.alignments[r0:r0 + n],
                                                           ref.alignments))
        cons &= res.consensus[j] == ref.consensus
        r0 += n
    return {"windows": k, "reads": r0, "scores_equal": bool(scores),
            "alignments_equal": bool(aligns), "consensus_equal": bool(cons)}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import spoa_gb300 as sg
    if sg.lib().spoa_gb300_device_count() <= 0:
        raise SystemExit("no CUDA device visible")
    # the library links its own CUDA runtime: name the rank's device to it
    device = local if world > 1 else None
    if args.workload == "serve":
        return serve(args, sg, rank, world, dist, device)

    wins, typ, params, wtypes, wstrand, cfg = workload(args.workload, args.windows, rank,
                                                       args.long_reads)
    n_windows = len(wins)
    seqs, off, wro = flatten(wins, pinned=True)

    cpt, nt = (int(x) for x in args.tile.split("x")) if args.tile else (0, 0)

    def make_batch():
        return sg.Batch.from_arrays(seqs, off, wro, typ, *params, window_types=wtypes,
                                    window_strand=wstrand,
                                    autotune=args.workload == "batch_10k" and not args.tile,
                                    columns_per_thread=cpt, threads_per_window=nt,
                                    windows_per_cta=args.windows_per_cta, cluster=args.cluster,
                                    device=device)

    batch = make_batch()
    for _ in range(args.warmup):
        batch.launch()
    res = batch.fetch()
    assert (res.status == 0).all(), "windows failed"

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    clocks = Clocks()
    clocks.start()
    barrier()
    kernel_ms = 0.0
    launches = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.launch()
        r = batch.fetch()
        kernel_ms += r.kernel_ms
        launches += r.launches
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    step_s = max_over_ranks(kernel_ms / 1e3 / args.steps, dist, "cuda")
    total_windows = n_windows * world
    value = total_windows / step_s
    cells, pred_cells = res.cells, res.pred_cells
    gcups = cells * world / step_s / 1e9

    # end to end through the public API, pinned host inputs every step
    e2e = None
    if not args.no_e2e:
        h2d = int(seqs.nbytes + off.nbytes + wro.nbytes)
        barrier()
        te = time.perf_counter()
        d2h = 0
        for _ in range(max(1, args.steps)):
            b = make_batch()
            b.launch()
            rr = b.fetch()
            d2h = sum(len(c) for c in rr.consensus) + rr.scores.nbytes + rr.status.nbytes
            del b
        barrier()
        e2e_s = (time.perf_counter() - te) / max(1, args.steps)
        e2e = {"value": total_windows / e2e_s, "unit": "windows/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": int(d2h)}

    # one-window-per-launch form on a sample
    plain = None
    if rank == 0 and args.plain_sample > 0 and n_windows > 1:
        k = min(args.plain_sample, n_windows)
        ps, po_, pw = flatten(wins[:k], pinned=False)
        pb = sg.Batch.from_arrays(ps, po_, pw, typ, *params,
                                  window_types=wtypes[:k] if wtypes else None,
                                  window_strand=wstrand[:k] if wstrand else None, device=device)
        pb.launch_plain()
        pr = pb.fetch()
        plain = {"value": k / (pr.kernel_ms / 1e3), "unit": "windows/s", "sample_windows": k,
                 "launches": pr.launches}
        del pb

    # rooflines
    hbm_peak, peak_kind = measured_peaks()
    achieved_gbs = cells * TRACEBACK_BYTES_PER_CELL / step_s / 1e9
    tpc = traffic_per_cell()
    sub = batch.subtype
    a_, b_ = OPS[sub]
    ops = a_ * pred_cells + b_ * cells + (cells if typ == 0 else 0)
    p32, p16 = int_peaks()
    # the 16-bit kernels issue the 16x2 forms, the 32-bit ones the 32-bit forms
    int_peak = p16 if DTYPES.get(args.workload) == "int16" else p32
    int_roof = None
    if int_peak:
        int_roof = {"achieved": ops / step_s / 1e9, "peak": int_peak / 1e9, "unit": "Gop/s",
                    "frac": ops / step_s / int_peak,
                    "ops_per_cell": ops / max(cells, 1),
                    "peak_kind": "measured in this run: " + (
                        "__viaddmax_s16x2 / __vimax3_s16x2 / __vadd2 chains, two lane-ops each"
                        if int_peak is p16 else "__viaddmax_s32 / __vimax3_s32 / add chains"),
                    "peak_s32": p32 / 1e9 if p32 else None,
                    "peak_s16x2": p16 / 1e9 if p16 else None}

    parity = None
    if rank == 0 and args.parity_windows > 0:
        parity = parity_sample(sg, wins, typ, params, wtypes, wstrand, args.parity_windows,
                               device)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(wins, typ, params, wtypes, wstrand, args.cpu_seconds)
        k = cpu.pop("n")
        cons = cpu.pop("consensus")
        cpu["parity_sample_windows"] = k
        cpu["parity_sample_equal"] = bool(cons == res.consensus[:k])
        if "reference_consensus" in cpu:
            rc, rn = cpu.pop("reference_consensus"), cpu.pop("reference_n")
            cpu["reference_consensus_equal_windows"] = int(
                sum(a == b for a, b in zip(rc, res.consensus[:rn])))
            cpu["reference_windows"] = rn

    line = {
        "metric": "windows/s", "value": value, "unit": "windows/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES.get(args.workload, "int16/int32"),
        "data": "synthetic (seeded; see spoa_gb300/synth.py)",
        "config": common_config(cfg, world),
        "tile": {"threads_per_window": res.threads_per_window,
                 "columns_per_thread": res.columns_per_thread, "ctas": res.ctas,
                 "windows_per_cta": args.windows_per_cta, "cluster": args.cluster},
        "gcups": gcups, "cells_per_step": cells * world,
        "e2e": e2e, "plain": plain,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak,
                     "traffic": (tpc * cells) if tpc else None,
                     "peak_kind": peak_kind,
                     "algorithmic_bytes": "0.5 B per DP cell (4-bit traceback state)",
                     "binding": "the integer max/add pipe (int_roofline); HBM is not the "
                                "bound of this path"},
        "int_roofline": int_roof,
        "parity": parity,
        "cpu_baseline": cpu,
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def serve_stream(n: int, rate: float, seed: int):
    """A Poisson arrival stream: n windows drawn 70/30 from the polishing and
    the uneven distributions, exponential gaps at `rate` windows/s.
    Returns [(reads, type, strand, arrival seconds)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        if rng.random() < 0.7:
            w = synth.batch_window(5_000_000 + seed * 100_000 + k)
            out.append((w.reads, 2, False, t))
        else:
            w = synth.uneven_window(6_000_000 + seed * 100_000 + k)
            out.append((w.reads, w.type, True, t))
    return out


def serve(args, sg, rank, world, dist, device=None):
    """Served form: windows arrive over time (Poisson, at each offered load
    of --rates) and are served as they come; reports the completed windows/s
    and the latency (completion minus arrival) percentiles.  The 70/30 mix of
    polishing-shaped (OV convex 5/-4/-8/-6/-10/-4) and uneven-shaped windows
    (NW/OV per window, strand-ambiguous, affine 5/-4/-8/-6) goes to two
    servers on the one GPU, one per scoring: the polishing server runs its
    windows on the resident persistent kernel (unless --no-resident), the
    uneven server launches."""
    p_params = synth.SCORING["batch_10k"][1]
    u_params = synth.SCORING["uneven_2k"][1]
    rates = [float(x) for x in args.rates.split(",") if x]
    sweep = []
    clocks = Clocks()
    clocks.start()

    def servers():
        budget = 0
        try:
            import torch
            free, _ = torch.cuda.mem_get_info()
            budget = int(free * 0.35)
        except Exception:  # noqa: BLE001
            pass
        return (sg.Server(2, *p_params, memory_budget=budget, gather_seconds=0.0005,
                          device=device, resident=not args.no_resident),
                sg.Server(1, *u_params, memory_budget=budget, gather_seconds=0.0005,
                          device=device))

    for i, rate in enumerate(rates):
        stream = serve_stream(args.serve_windows, rate, seed=rank * 101 + i)
        ps, us = servers()
        try:
            # warm-up: the kernels of every width and class once
            for reads, typ, strand, _ in stream[:8]:
                sv = us if strand else ps
                sv.wait(sv.submit(reads, typ, strand), timeout=600)
            t0 = time.perf_counter()
            tickets = []
            for r, t, st_, a in stream:
                sv = us if st_ else ps
                tickets.append((sv, sv.submit(r, t, st_, a)))
            res = [sv.wait(t, timeout=3600) for sv, t in tickets]
            wall = time.perf_counter() - t0
            st_p, st_u = ps.stats(), us.stats()
        finally:
            ps.close()
            us.close()
        lat = np.array([x[2] for x in res])
        ok = sum(1 for x in res if x[0] == 0)
        wall = max_over_ranks(wall, dist, "cuda")
        sweep.append({"offered_windows_per_s": rate, "windows": len(stream) * world,
                      "completed_ok": ok, "windows_per_s": len(stream) * world / wall,
                      "p50_latency_s": float(np.percentile(lat, 50)),
                      "p99_latency_s": float(np.percentile(lat, 99)),
                      "launches": st_p["launches"] + st_u["launches"],
                      "resident_windows": st_p["resident_windows"],
                      "resident_launches": st_p["resident_launches"], "wall_s": wall})
    clk = clocks.stop()
    best = max(sweep, key=lambda x: x["windows_per_s"])
    line = {"metric": "windows/s (served)", "value": best["windows_per_s"], "unit": "windows/s",
            "n_gpus": world, "steps": len(rates), "warmup": 1,
            "ms_per_step": best["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int16/int32",
            "data": "synthetic (seeded; see bench.py serve_stream)",
            "config": {"workload": "serve: Poisson arrivals, 70/30 polishing (batch_10k shape, "
                                   "OV convex 5/-4/-8/-6/-10/-4) / uneven (uneven_2k shape, "
                                   "NW/OV strand-ambiguous, affine 5/-4/-8/-6) windows",
                       "windows_per_rate": args.serve_windows, "rates": rates,
                       "resident": not args.no_resident,
                       "parallelism": f"arrival streams sharded over {world} GPU(s), no collective"},
            "serving": sweep, "gpu_launches": sum(x["launches"] for x in sweep), "clocks": clk}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def reference_arm(args):
    """The reference's CPU implementation on all host cores: its own library
    built from its sources (oracle/ref_bench.cpp; the SisdAlignmentEngine on
    the aarch64 GPU machine, where the reference has no SIMD path), else the C
    oracle.  Each step times a bounded sample of the same workload."""
    from oracle import pyoracle as po
    world = int(os.environ.get("WORLD_SIZE", "1"))
    wins, typ, params, wtypes, wstrand, cfg = workload(args.workload, args.windows, 0,
                                                       args.long_reads)
    threads = os.cpu_count() or 1
    types, strands = _types_strands(wins, typ, wtypes, wstrand)
    total_steps = args.steps + args.warmup
    budget = 150.0 / max(total_steps, 1)
    use_ref = po.reference_bench() is not None
    if use_ref:
        k = min(len(wins), threads)
        probe = po.run_reference_bench([w.reads for w in wins[:k]], types[:k], strands[:k],
                                       params, threads)
        per_window = probe["seconds"] / max(k, 1) * threads
        engine = probe["engine"]
    else:
        po.lib()
        probe = wins[:threads]
        t0 = time.perf_counter()
        _run_oracle(po, probe, typ, params, wtypes, wstrand, threads)
        per_window = max(time.perf_counter() - t0, 1e-3) / max(len(probe), 1) * threads
    n = _sample_size(wins, budget, per_window, threads, min(len(wins), threads))
    sample = wins[:n]

    def step():
        if use_ref:
            return po.run_reference_bench([w.reads for w in sample], types[:n], strands[:n],
                                          params, threads)["seconds"]
        t0 = time.perf_counter()
        _run_oracle(po, sample, typ, params, wtypes, wstrand, threads)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    dt = sum(step() for _ in range(args.steps)) / max(args.steps, 1)
    value = n / dt
    kind = "reference" if use_ref else "port"
    what = (("spoa SisdAlignmentEngine" if engine == "sisd" else "spoa SimdAlignmentEngine") +
            " (the reference's own library, built from its sources on this host)"
            if use_ref else "the C oracle (the reference algorithm restated in C)")
    line = {"impl": "reference", "metric": "windows/s", "value": value, "unit": "windows/s",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES.get(args.workload, "int16/int32"),
            "data": "synthetic (seeded; see spoa_gb300/synth.py)",
            "config": common_config(cfg, world),
            "cpu_baseline": {"value": value, "unit": "windows/s", "cores": threads,
                             "kind": kind, "engine": what,
                             "sample": f"first {n} windows of the workload per step "
                                       f"(of {len(wins)}), one window per host thread"},
            "e2e": {"value": value, "unit": "windows/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
