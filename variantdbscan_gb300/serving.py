"""Request serving on one GPU: an open-loop arrival stream of clustering
requests (each a dataset with its variants), admitted first-come first-served
while the estimated device-memory footprint of the requests in flight stays
under a budget, and run on a few concurrent library contexts.

A request runs as one vdb_run_batch call (all its variants share one index,
and its labels stay on the device until the call ends), so the footprint of a
request is its index, labels and neighbour-table budget.  The serving loop is
host code; the runner it calls is pluggable so that the admission logic can be
tested without a GPU.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

# device bytes of one dataset besides the neighbour table and the labels:
# a fixed part (the one-way pair list, scratch of the sorts and scans, a dense
# cell array of up to 4M cells) and a part per point (inputs, visit order, cell
# order, union-find state, tiles, counts, row offsets), until Server.calibrate
# measures both on sample requests
INDEX_BASE_BYTES = 64 << 20
INDEX_BYTES_PER_POINT = 200


@dataclass
class Request:
    arrival: float            # seconds after the start of the stream
    x: np.ndarray
    y: np.ndarray
    eps: np.ndarray
    minpts: np.ndarray
    mbb_size: int = 70
    # filled in by the server
    admitted: float = 0.0
    done: float = 0.0
    labels: np.ndarray | None = None
    error: str = ""
    device_bytes: int = 0     # measured footprint of its call (vdb_stats.device_bytes)
    table_bytes: int = 0      # of which its largest neighbour-table allocation

    @property
    def n(self) -> int:
        return len(self.x)

    @property
    def variant_points(self) -> int:
        return self.n * len(self.eps)


def footprint(req: Request, table_budget: int, index_bytes_per_point: float = INDEX_BYTES_PER_POINT,
              index_base_bytes: int = INDEX_BASE_BYTES) -> int:
    """Estimated device bytes of a request in flight: index and labels plus the
    neighbour-table budget it is given (larger tables are built in row chunks)."""
    return (int(index_base_bytes) + int(index_bytes_per_point * req.n) + 4 * req.variant_points
            + table_budget)


@dataclass
class ServeResult:
    rate: float                      # offered requests/s (inf: all at time 0)
    makespan: float                  # first arrival to last completion, s
    variant_points: int
    latencies: np.ndarray            # per request, s
    peak_footprint: int              # largest admitted footprint sum, bytes
    errors: list = field(default_factory=list)
    # largest measured footprint of a request over its admission estimate (0:
    # the runner measures nothing)
    footprint_ratio: float = 0.0

    @property
    def throughput(self) -> float:
        return self.variant_points / self.makespan if self.makespan > 0 else 0.0

    def percentile_ms(self, q: float) -> float:
        return float(np.percentile(self.latencies, q) * 1e3) if len(self.latencies) else 0.0


class Server:
    """Admission control plus `workers` concurrent runners.

    runner_factory() returns a callable run(req) -> labels; one runner per
    worker thread (each with its own library context and CUDA stream)."""

    def __init__(self, runner_factory, workers: int = 4, hbm_budget: int = 150 << 30,
                 table_budget: int | None = None):
        self.workers = workers
        self.hbm_budget = int(hbm_budget)
        # each worker may build a table of up to this many bytes at a time
        self.table_budget = int(table_budget if table_budget is not None
                                else self.hbm_budget // (2 * workers))
        self.runners = [runner_factory(self.table_budget) for _ in range(workers)]
        self.index_bytes_per_point = float(INDEX_BYTES_PER_POINT)
        self.index_base_bytes = int(INDEX_BASE_BYTES)

    def footprint(self, req: Request) -> int:
        return footprint(req, self.table_budget, self.index_bytes_per_point,
                         self.index_base_bytes)

    def calibrate(self, sample: list[Request]) -> tuple[float, int]:
        """Runs the sample requests one after another and fits the index part
        of the admission estimate (the call's measured device footprint less
        its neighbour-table allocation and its labels) as base + bytes x
        points: a least-squares slope, the base raised until no sample lies
        above the line.  Returns (bytes per point, base bytes)."""
        run = self.runners[0]
        pts = []
        for r in sample:
            run(r)
            if r.device_bytes and r.n:
                pts.append((r.n, r.device_bytes - r.table_bytes - 4 * r.variant_points))
        if not pts:
            return self.index_bytes_per_point, self.index_base_bytes
        n = np.array([p[0] for p in pts], np.float64)
        b = np.array([p[1] for p in pts], np.float64)
        slope = float(np.polyfit(n, b, 1)[0]) if len(pts) > 1 and np.ptp(n) > 0 else 0.0
        slope = max(slope, 0.0)
        base = float(np.max(b - slope * n))
        self.index_bytes_per_point = slope
        self.index_base_bytes = int(np.ceil(max(base, 0.0)))
        return self.index_bytes_per_point, self.index_base_bytes

    def serve(self, requests: list[Request], rate: float) -> ServeResult:
        """Replays the stream with arrivals scaled to `rate` requests/s (the
        requests' arrival fields are in units of the mean gap; inf: all at once)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        arrivals = [0.0 if not np.isfinite(rate) else r.arrival / rate for r in reqs]
        for r in reqs:
            fp = self.footprint(r)
            if fp > self.hbm_budget:
                raise ValueError(f"request of {r.n} points exceeds the device budget alone")
        cv = threading.Condition()
        state = {"inflight": 0, "peak": 0, "next": 0, "queue": []}
        t0 = time.perf_counter()

        def admit_loop():
            # FIFO: the head of the queue waits until its footprint fits
            for i, r in enumerate(reqs):
                delay = arrivals[i] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                fp = self.footprint(r)
                with cv:
                    while state["inflight"] + fp > self.hbm_budget:
                        cv.wait()
                    state["inflight"] += fp
                    state["peak"] = max(state["peak"], state["inflight"])
                    r.admitted = time.perf_counter() - t0
                    state["queue"].append((r, fp))
                    cv.notify_all()
            with cv:
                state["queue"].append(None)  # end of stream
                cv.notify_all()

        def worker(wi):
            run = self.runners[wi]
            while True:
                with cv:
                    while not state["queue"]:
                        cv.wait()
                    item = state["queue"][0]
                    if item is None:
                        return  # leave the end marker for the other workers
                    state["queue"].pop(0)
                r, fp = item
                try:
                    r.labels = run(r)
                except Exception as e:  # noqa: BLE001 - reported per request
                    r.error = str(e)
                r.done = time.perf_counter() - t0
                with cv:
                    state["inflight"] -= fp
                    cv.notify_all()

        threads = [threading.Thread(target=admit_loop)]
        threads += [threading.Thread(target=worker, args=(i,)) for i in range(self.workers)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        lat = np.array([r.done - a for r, a in zip(reqs, arrivals)])
        first = min(arrivals) if arrivals else 0.0
        makespan = max((r.done for r in reqs), default=0.0) - first
        ratio = max((r.device_bytes / self.footprint(r) for r in reqs), default=0.0)
        return ServeResult(rate=rate, makespan=makespan,
                           variant_points=sum(r.variant_points for r in reqs),
                           latencies=lat, peak_footprint=state["peak"],
                           errors=[r.error for r in reqs if r.error], footprint_ratio=ratio)


def library_runner_factory(precision: str = "mixed", table: str = "border"):
    """Runners backed by the CUDA library: one vdb_context per worker, host
    buffers in and labels out (the copies are part of each request).  A request
    returns labels only, so by default the tables hold just the rows the
    labelling reads (table="all" writes every row)."""
    import variantdbscan_gb300 as v

    def factory(table_budget):
        ctx = v.Context()

        def run(req: Request):
            out, st = ctx.run([v.BatchItem(req.x, req.y, req.eps, req.minpts, req.mbb_size)],
                              precision=precision, budget=table_budget, streams=1, table=table)
            req.device_bytes = int(st["device_bytes"])
            req.table_bytes = int(st["table_bytes"])
            return out[0]

        run.ctx = ctx
        return run

    return factory


def requests_from(stream) -> list[Request]:
    """Requests from synthetic.request_stream items (arrival, Dataset)."""
    return [Request(a, d.x, d.y, d.eps, d.minpts) for a, d in stream]
