"""Benchmark: variant-points/s of the batched mixed-precision GB300 path.

Workload (default): the variant sweep - 2,000,000 2-D FP64 points (64 Gaussian
blobs + 10% uniform background, seed 1) x 16 variants eps {0.1,0.2,0.4,0.8} x
minpts {4,16,64,256}.  A step clusters all 16 variants of the dataset:
index, four neighbour tables (one per epsilon), 16 labellings.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value: variant-points/s with the points already in HBM (CUDA events on the
library's stream, L2 flushed between steps); e2e: the same through the public
API with host buffers (H2D of the coordinates and D2H of the labels inside the
timed region).  Multi-GPU runs are independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from variantdbscan_gb300 import synthetic as syn  # noqa: E402

METRIC = "variant-points/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="variant_sweep", choices=sorted(WORKLOADS),
                   help="variant_sweep (default): 2M points x 16 variants; lattice: 10M "
                        "points on a 0.01 deg lattice x 8 variants; single: 50k points x 1 "
                        "variant; multi: 64 datasets of uneven size, 4-12 variants each; "
                        "serving: a request stream under an admission budget")
    p.add_argument("--n", type=int, default=0,
                   help="points (datasets for multi); 0: the workload's size")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--no-e2e", action="store_true", help="skip the end-to-end measurement")
    p.add_argument("--cpu-sample", type=int, default=40_000)
    p.add_argument("--cells-per-eps", type=int, default=0,
                   help="grid cells per epsilon (0: the library's choice)")
    p.add_argument("--no-reuse-compare", action="store_true",
                   help="skip the measurement without reuse across variants")
    p.add_argument("--no-labels-only", action="store_true",
                   help="skip the labels-only measurement (border rows of the tables)")
    p.add_argument("--serving-table", default="border", choices=["border", "all"],
                   help="table rows written by the serving workload's requests")
    p.add_argument("--entry-bytes", type=int, default=0, choices=[0, 2, 4],
                   help="neighbour-table entries: 0/2 = 16-bit where tiles allow, 4 = 32-bit")
    p.add_argument("--streams", type=int, default=0,
                   help="concurrent dataset streams of the library (0: autotuned)")
    p.add_argument("--tile-cells", type=int, default=0,
                   help="grid cells per tile group (0: autotuned per table)")
    p.add_argument("--compare-fixed", action="store_true",
                   help="also time the step with the untuned shapes (one-cell tiles, "
                        "min(4, datasets) streams); on by default for --workload multi")
    p.add_argument("--unit-candidates", type=int, default=0, choices=[0, 1024, 2048, 4096],
                   help="candidates per work unit (0: by dataset size)")
    p.add_argument("--graph", action="store_true",
                   help="time the main steps as graph replays (vdb_options.graph)")
    p.add_argument("--graph-compare", action="store_true",
                   help="also time the step replayed as one CUDA graph; on by default for "
                        "--workload single and multi")
    p.add_argument("--no-graph-compare", action="store_true",
                   help="skip the graph-replay measurement")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


WORKLOADS = {
    # name: (generator, default points, description of the variants)
    "variant_sweep": (lambda n: syn.variant_sweep(n=n, seed=1), 2_000_000,
                      "variant_sweep: {n} points x {v} variants (eps 0.1/0.2/0.4/0.8 x "
                      "minpts 4/16/64/256), MBBsize 70"),
    "lattice": (lambda n: syn.lattice_stress(n=n, seed=3), 10_000_000,
                "lattice_stress: {n} points on a 0.01 deg lattice x {v} variants "
                "(eps 0.05/0.1/0.25/0.5 x minpts 8/32), MBBsize 70"),
    "single": (lambda n: syn.single_variant(n=n, seed=0), 50_000,
               "single_variant: {n} points x {v} variant (eps 0.5, minpts 10), MBBsize 70"),
    # n = number of requests: a prefix of the 2,000-request stream (the whole
    # stream holds ~1.6e9 points and ~2.6e10 variant-points, ~26 GB of
    # coordinates and ~106 GB of labels in host memory, over 2 minutes a pass)
    "serving": (lambda n: syn.request_stream(count=n, seed=4), 200,
                "serving: first {k} requests of the 2000-request Poisson stream (seed 4; "
                "1e4-5e6 points log-uniform, 1-32 variants, eps log-uniform in [0.05, 1.5] "
                "deg, minpts uniform in [4, 128]), {n} points, {v} variants, 150 GiB "
                "admission budget, 4 worker streams"),
    # n = number of datasets
    "multi": (lambda n: syn.multi_dataset(count=n, seed=2), 64,
              "multi_dataset: {k} datasets of 1e4-1e6 points (log-uniform), {n} points, "
              "{v} variants in all (4-12 per dataset, eps log-uniform in [0.05, 1.5] deg, "
              "minpts uniform in [4, 128]), MBBsize 70, one vdb_run_batch call"),
}


def workload(args):
    """The workload's datasets (a list) and its description."""
    gen, n0, desc = WORKLOADS[args.workload]
    d = gen(args.n or n0)
    dss = d if isinstance(d, list) else [d]
    if dss and isinstance(dss[0], tuple):  # (arrival, Dataset) request stream
        return dss, desc.format(n=sum(x.n for _, x in dss),
                                v=sum(len(x.eps) for _, x in dss), k=len(dss))
    return dss, desc.format(n=sum(x.n for x in dss), v=sum(len(x.eps) for x in dss),
                            k=len(dss))


def largest(dss):
    return max(dss, key=lambda d: d.n)


def cpu_sample(d, target):
    """A longitude stripe of the dataset holding about `target` points (keeps
    the local density, hence the per-point work, of the full workload);
    target 0 or >= n: the whole dataset."""
    if target <= 0 or target >= d.n:
        return d.x, d.y, None
    order = np.argsort(d.x, kind="stable")
    mid = len(order) // 2
    lo = max(0, mid - target // 2)
    idx = np.sort(order[lo:lo + target])
    x0, x1 = float(d.x[order[lo]]), float(d.x[order[min(lo + target, len(order)) - 1]])
    return d.x[idx].copy(), d.y[idx].copy(), (x0, x1)


def sample_desc(d, n_sample, stripe):
    """Names the points a CPU leg ran on."""
    if stripe is None:
        return f"the whole {d.n}-point dataset, all {len(d.eps)} variants in one libVDBSCAN call"
    return (f"{n_sample} points of the {d.n}-point dataset in the longitude stripe "
            f"[{stripe[0]:.3f}, {stripe[1]:.3f}] deg, all {len(d.eps)} variants in one "
            f"libVDBSCAN call")


def time_reference_cpu(d, target, steps=1, warmup=0):
    from oracle.oracle import REF_SO, RestatedOracle, ReferenceLibrary, build_reference
    sx, sy, stripe = cpu_sample(d, target)
    kind, cores = "reference", None
    try:
        if not os.path.exists(REF_SO):
            build_reference()
        ref = ReferenceLibrary()
        fn = lambda: ref.run(sx, sy, d.eps, d.minpts)  # noqa: E731
        cores = ref.threads
    except Exception:
        orc = RestatedOracle()
        fn = lambda: orc.variants(sx, sy, d.eps, d.minpts)  # noqa: E731
        kind, cores = "port", os.cpu_count()
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(steps):
        t = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t)
    units = len(sx) * len(d.eps)
    return units, ts, kind, cores, sample_desc(d, len(sx), stripe)


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.proc, self.lines = gpu, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [c.strip() for c in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def aggregate(t_local, units_local, world, device):
    """Whole-job throughput of replicas that each processed units_local units
    in t_local seconds: the slowest rank's time (max over ranks) and
    world * units_local / that time."""
    t = t_local
    if world > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([t_local], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
        dist.barrier()
    return t, units_local * world / t


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per neighbour pair of the expand (table) kernel, from the
    committed ncu capture of a smaller variant sweep, or None."""
    p = os.path.join(ROOT, "profiles", "expand_traffic_variant_sweep.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def run_ours(args):
    import torch
    import torch.distributed as dist

    import variantdbscan_gb300 as v

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dss, desc = workload(args)
    per_step = sum(d.n * len(d.eps) for d in dss)  # variant-points of one step
    # the library launches on this stream, so CUDA events recorded on it time
    # its kernels; inputs are made ready before the first call
    stream = torch.cuda.Stream()
    dev = []
    for d in dss:
        xt = torch.from_numpy(d.x).cuda()
        yt = torch.from_numpy(d.y).cuda()
        lab = torch.zeros(len(d.eps) * d.n, dtype=torch.int32, device="cuda")
        dev.append((xt, yt, lab))
    items_dev = [(xt.data_ptr(), yt.data_ptr(), d.n, d.eps, d.minpts, lab.data_ptr())
                 for d, (xt, yt, lab) in zip(dss, dev)]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    torch.cuda.synchronize()
    ctx = v.Context(stream=stream.cuda_stream)
    torch.cuda.set_stream(stream)

    def step(**kw):
        kw.setdefault("cells_per_eps", args.cells_per_eps)
        kw.setdefault("streams", args.streams)
        kw.setdefault("entry_bytes", args.entry_bytes)
        kw.setdefault("tile_cells", args.tile_cells)
        kw.setdefault("graph", args.graph)
        kw.setdefault("unit_candidates", args.unit_candidates)
        return ctx.run_device_batch(items_dev, **kw)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    evs = []
    stats = []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats.append(step())
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in evs]
    t_total, value = aggregate(sum(ms) / 1e3, per_step * args.steps, world, "cuda")

    # end to end through the public API with host buffers (pinned): the H2D
    # copy of the coordinates and the D2H copy of the labels are inside the call
    e2e = None
    items = None
    if not args.no_e2e:
        items = []
        for d in dss:
            xp = torch.from_numpy(d.x).pin_memory().numpy()
            yp = torch.from_numpy(d.y).pin_memory().numpy()
            lp = torch.zeros((len(d.eps), d.n), dtype=torch.int32).pin_memory().numpy()
            items.append(v.BatchItem(xp, yp, d.eps, d.minpts, labels=lp.view(np.uint32)))
        for _ in range(2 if args.graph else 1):  # (with --graph: capture, then a replay)
            ctx.run(items, entry_bytes=args.entry_bytes, graph=args.graph)
        torch.cuda.synchronize()
        k_e2e = max(1, min(args.steps, 3))
        t = time.perf_counter()
        for _ in range(k_e2e):
            ctx.run(items, entry_bytes=args.entry_bytes, graph=args.graph)
        e2e_s = (time.perf_counter() - t) / k_e2e
        direct_labels = [np.array(it.labels) for it in items]
        e2e = {"value": per_step / e2e_s, "unit": METRIC,
               "h2d_bytes_per_step": int(sum(16 * d.n for d in dss)),
               "d2h_bytes_per_step": int(sum(4 * d.n * len(d.eps) for d in dss))}

    st = stats[-1]
    # roofline of the neighbour-table (expand) kernel: algorithmic bytes
    # 16 N (coordinates) + 4 (N+1) (row offsets) per table plus the neighbour
    # entries written (2 bytes each in compact tables, else 4)
    tables = st["tables"]
    # one table per distinct epsilon of a dataset
    alg_bytes = sum(len(np.unique(d.eps)) * (16 * d.n + 4 * (d.n + 1)) for d in dss) \
        + st["entry_bytes"]
    entry = "compact" if st["compact_tables"] == tables else \
        ("wide" if st["compact_tables"] == 0 else None)
    fill_s = sum(s["ms_table"] for s in stats) / len(stats) / 1e3
    # (graph replays report no phase times: no roofline then)
    achieved = alg_bytes / fill_s / 1e9 if fill_s > 0 else float("nan")
    peak, peak_kind = measured_peak()
    tr = profiled_traffic()
    traffic = None
    key = {"compact": "expand_compact", "wide": "expand"}.get(entry)
    if args.workload == "variant_sweep" and tr and key and tr.get(key, {}).get("dram_bytes_per_pair"):
        # DRAM traffic grows with the pairs written: the capture's bytes per
        # pair times this run's pairs, per launch
        traffic = tr[key]["dram_bytes_per_pair"] * st["pairs"] / tables
    roofline = {"bound": "hbm", "kernel": "expand_kernel", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind,
                "traffic": traffic, "alg_bytes_per_launch": alg_bytes / tables,
                "launch_ms": fill_s * 1e3 / tables}

    # the count kernel is issue-bound (FP32 pair arithmetic and mask shifts):
    # its roofline is candidate tests per second against the issue rate of its
    # inner loop, 4.5 warp-instruction lanes per test (per 2 candidates and
    # query: 2 fma.f32x2, 2 sub.f32x2, 4 funnel shifts; 2 shared loads per
    # 4 tests), i.e. 32 / 4.5 tests per warp-instruction, 4 warp-instructions
    # per cycle per SM
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    sm_hz = (clk or {}).get("sm_mhz", 2070.0) * 1e6
    count_s = sum(s["ms_count"] for s in stats) / len(stats) / 1e3
    count_s = count_s if count_s > 0 else float("nan")
    tests_peak = nsm * 4 * sm_hz * 32 / 4.5
    roofline_count = {"bound": "issue", "kernel": "count_kernel",
                      "achieved": st["candidates"] / count_s, "peak": tests_peak,
                      "unit": "candidate tests/s", "frac": st["candidates"] / count_s / tests_peak,
                      "peak_source": f"model: {nsm} SMs x 4 warp-instructions/cycle x "
                                     f"{sm_hz / 1e6:.0f} MHz x 32/4.5 tests",
                      "launch_ms": count_s * 1e3 / tables}
    if not np.isfinite(achieved):
        roofline = None
    if not np.isfinite(count_s):
        roofline_count = None

    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(ms)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Gaussian blobs + uniform background)",
        "config": {"workload": desc,
                   "precision": "mixed (FP32 filter, FP64 band re-test)",
                   "schedule": "batched (tables shared per eps; union-find chained over "
                               "minpts; larger-eps components prune cell-pair searches)",
                   "table_entries": {"compact": "16-bit (position within a 4096-candidate work unit)",
                                     "wide": "32-bit (cell-ordered index)"}.get(entry, "mixed"),
                   "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e,
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "roofline": roofline,
        "roofline_count": roofline_count,
        "stats": {"pairs": st["pairs"], "candidates": st["candidates"],
                  "retested": st["retested"],
                  "retested_fraction": st["retested"] / max(1, st["candidates"]),
                  "ms_index": st["ms_index"], "ms_count": st["ms_count"],
                  "ms_table": st["ms_table"], "ms_cluster": st["ms_cluster"],
                  "wall_s": wall},
    }
    if clk:
        out["clocks"] = clk

    out["autotune"] = {"tables_by_tile_cells": {str(1 << i): c for i, c in
                                                enumerate(st["tables_by_tile_cells"]) if c},
                       "worker_streams": st["worker_streams"]}
    if (args.graph_compare or args.workload in ("single", "multi")) and not args.graph \
            and not args.no_graph_compare:
        # the same step replayed as one CUDA graph (vdb_options.graph): one
        # capture call, one warm replay, then the timed replays; the datasets
        # of the batch run as branches of the graph (no worker threads)
        step(graph=True)
        step(graph=True)
        ms_g, st_g = [], []
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st_g.append(step(graph=True))
            e1.record(stream)
            torch.cuda.synchronize()
            ms_g.append(e0.elapsed_time(e1))
        g = {"value": per_step / (float(np.mean(ms_g)) / 1e3), "unit": METRIC,
             "ms_per_step": float(np.mean(ms_g)),
             "states": sorted({int(s["graph"]) for s in st_g}),  # 2: replayed
             "checkpoints": int(st_g[-1]["graph_checks"]),
             "kernels_per_step": int(st_g[-1]["kernel_launches"]),
             "labels_equal_direct": None}
        if items is not None:
            # end to end with host buffers, replayed
            for it in items:
                it.labels[...] = 0
            for _ in range(2):
                ctx.run(items, entry_bytes=args.entry_bytes, graph=True)
            k = max(3, args.steps)
            t = time.perf_counter()
            for _ in range(k):
                _, gs = ctx.run(items, entry_bytes=args.entry_bytes, graph=True)
            g_s = (time.perf_counter() - t) / k
            g["labels_equal_direct"] = all(np.array_equal(a, np.array(it.labels))
                                           for a, it in zip(direct_labels, items))
            g["e2e"] = {"value": per_step / g_s, "unit": METRIC, "ms_per_call": g_s * 1e3,
                        "state": int(gs["graph"]),
                        "h2d_bytes_per_step": int(sum(16 * d.n for d in dss)),
                        "d2h_bytes_per_step": int(sum(4 * d.n * len(d.eps) for d in dss))}
            if e2e:
                g["e2e"]["direct_ms_per_call"] = per_step / e2e["value"] * 1e3
        out["graph"] = g

    if args.compare_fixed or (args.workload == "multi" and args.tile_cells == 0
                              and args.streams == 0):
        # the untuned shapes: one-cell tiles everywhere, min(4, datasets) streams
        fixed = dict(tile_cells=1, streams=min(4, len(dss)))
        step(**fixed)
        ms_f = []
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(**fixed)
            e1.record(stream)
            torch.cuda.synchronize()
            ms_f.append(e0.elapsed_time(e1))
        out["autotune"]["fixed_shapes"] = {
            "value": per_step / (float(np.mean(ms_f)) / 1e3), "ms_per_step": float(np.mean(ms_f)),
            "tile_cells": 1, "streams": fixed["streams"]}

    if not args.no_reuse_compare:
        # the same step with every variant labelled from scratch (no reuse of
        # a larger minpts's or epsilon's components): the reuse's measured gain
        step(reuse=False)
        ms_r, st_r = [], []
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st_r.append(step(reuse=False))
            e1.record(stream)
            torch.cuda.synchronize()
            ms_r.append(e0.elapsed_time(e1))
        out["reuse"] = {"skipped_cell_pairs": st["reuse_skipped_pairs"],
                        "ms_cluster": st["ms_cluster"],
                        "without_reuse": {"value": per_step / (float(np.mean(ms_r)) / 1e3),
                                          "ms_per_step": float(np.mean(ms_r)),
                                          "ms_cluster": st_r[-1]["ms_cluster"]}}

    if not args.no_labels_only:
        # the same step writing only the table rows the labelling reads
        # (VDB_TABLE_BORDER): identical labels, a fraction of the table
        step(table="border")
        ms_b, st_b = [], []
        for _ in range(args.steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st_b.append(step(table="border"))
            e1.record(stream)
            torch.cuda.synchronize()
            ms_b.append(e0.elapsed_time(e1))
        out["labels_only"] = {"value": per_step / (float(np.mean(ms_b)) / 1e3), "unit": METRIC,
                              "ms_per_step": float(np.mean(ms_b)),
                              "ms_table": st_b[-1]["ms_table"], "table_rows": "border"}

    if not args.no_plain:
        # the comparison path: one FP64 table and one labelling per variant;
        # one warm-up step, then 3 timed steps (mean, min, max)
        ps = step(precision="fp64", schedule="plain")
        torch.cuda.synchronize()
        pts = []
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            flush.fill_(1)
            e0.record(stream)
            ps = step(precision="fp64", schedule="plain")
            e1.record(stream)
            torch.cuda.synchronize()
            pts.append(e0.elapsed_time(e1) / 1e3)
        pt = float(np.mean(pts))
        out["plain_fp64"] = {"value": per_step / pt, "unit": METRIC, "ms_per_step": pt * 1e3,
                             "ms_per_step_min_max": [min(pts) * 1e3, max(pts) * 1e3],
                             "timed_steps": len(pts),
                             "speedup_batched_mixed": (per_step / (t_total / args.steps / world))
                             / (per_step / pt), "tables": ps["tables"]}
    if not args.no_e2e:
        # the reference arm's input (a longitude stripe of the largest dataset,
        # all its variants), run end to end through the public API with host
        # buffers: the same points and variants as the CPU reference's line
        dl = largest(dss)
        sx, sy, stripe = cpu_sample(dl, args.cpu_sample)
        item = [v.BatchItem(torch.from_numpy(np.ascontiguousarray(sx)).pin_memory().numpy(),
                            torch.from_numpy(np.ascontiguousarray(sy)).pin_memory().numpy(),
                            dl.eps, dl.minpts)]
        for _ in range(3):
            ctx.run(item, entry_bytes=args.entry_bytes)
        reps = 10
        t = time.perf_counter()
        for _ in range(reps):
            ctx.run(item, entry_bytes=args.entry_bytes)
        si_s = (time.perf_counter() - t) / reps
        out["same_input"] = {"sample": sample_desc(dl, len(sx), stripe),
                             "e2e": {"value": len(sx) * len(dl.eps) / si_s, "unit": METRIC,
                                     "ms_per_call": si_s * 1e3,
                                     "h2d_bytes_per_step": 16 * len(sx),
                                     "d2h_bytes_per_step": 4 * len(sx) * len(dl.eps)}}
    if rank == 0 and not args.no_cpu:
        units, ts, kind, cores, sample = time_reference_cpu(largest(dss), args.cpu_sample)
        out["cpu_baseline"] = {"value": units / float(np.mean(ts)), "unit": METRIC,
                               "cores": cores, "kind": kind, "sample": sample}
        if "same_input" in out:
            out["same_input"]["cpu_reference"] = out["cpu_baseline"]["value"]
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    dss, desc = workload(args)
    dss = [d[1] if isinstance(d, tuple) else d for d in dss]  # requests: their datasets
    units, ts, kind, cores, sample = time_reference_cpu(largest(dss), args.cpu_sample,
                                                        steps=args.steps,
                                                        warmup=args.warmup)
    value = units * len(ts) / float(np.sum(ts))
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(ts)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian blobs + uniform background)",
        # the points this arm ran: a stripe of the workload's largest dataset
        # unless --cpu-sample 0 (the whole dataset)
        "config": {"workload": f"{args.workload} sample: {sample}",
                   "full_workload": desc, "parallelism": f"{cores} host threads"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_serving(args):
    """Serving loop: requests from host memory (the copies are part of every
    request), admitted under a 150 GiB footprint budget onto 4 library
    contexts, the footprint per point measured on the stream's first requests.
    value: variant-points/s with every request offered at once (saturation);
    then open-loop passes at fractions of the saturation request rate (and one
    above it) give p50/p99 latency."""
    import torch

    from variantdbscan_gb300 import serving as sv

    rank, world, local = dist_env()
    if rank != 0 and world > 1:
        return
    torch.cuda.set_device(local)
    stream, desc = workload(args)
    reqs = sv.requests_from(stream)
    srv = sv.Server(sv.library_runner_factory(table=args.serving_table), workers=4,
                    hbm_budget=150 << 30)
    bpp, base = srv.calibrate(reqs[:16])
    for _ in range(args.warmup):
        srv.serve(reqs, rate=float("inf"))
    clocks = Clocks(local)
    clocks.start()
    sat = [srv.serve(reqs, rate=float("inf")) for _ in range(args.steps)]
    clk = clocks.stop()
    errs = sum(len(r.errors) for r in sat)
    span = sum(r.makespan for r in sat)
    vp = sum(r.variant_points for r in sat)
    rps = len(reqs) * len(sat) / span
    sweep = [{"offered_rps": "saturation", "p50_ms": sat[-1].percentile_ms(50),
              "p99_ms": sat[-1].percentile_ms(99), "variant_points_per_s": vp / span}]
    ratio = max(r.footprint_ratio for r in sat)
    # arrival times of the stream are in units of its mean gap: rate r = r requests/s
    for frac in (0.5, 0.8, 0.95, 1.2):
        r = srv.serve(reqs, rate=frac * rps)
        errs += len(r.errors)
        ratio = max(ratio, r.footprint_ratio)
        sweep.append({"offered_rps": frac * rps, "load": frac, "p50_ms": r.percentile_ms(50),
                      "p99_ms": r.percentile_ms(99), "variant_points_per_s": r.throughput,
                      "peak_admitted_gib": r.peak_footprint / 2**30})
    h2d = sum(16 * r.n for r in reqs)
    d2h = sum(4 * r.variant_points for r in reqs)
    out = {
        "metric": METRIC, "value": vp / span, "unit": METRIC, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": span / len(sat) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Gaussian blobs + uniform background)",
        "config": {"workload": desc, "step": "one pass of the request prefix, all offered "
                   "at once", "table_rows": args.serving_table, "l2": "not flushed: inputs stream from host memory",
                   "parallelism": "4 library contexts (streams) on one GPU"},
        "e2e": {"value": vp / span, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "serving": sweep, "request_errors": errs,
        "footprint": {"index_bytes_per_point_measured": bpp,
                      "index_base_bytes_measured": base,
                      "largest_measured_over_estimate": ratio,
                      "table_budget_gib_per_worker": srv.table_budget / 2**30},
    }
    if clk:
        out["clocks"] = clk
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serving":
        run_serving(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
