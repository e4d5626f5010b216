"""GB300 (sm_103a) VariantDBSCAN: the reference's libVDBSCAN hot path on the GPU.

Python mirror of the reference's ctypes wrapper
(python_package/vdbscan/variantdbscan.py:32-109) plus the batched C API of
include/vdbscan.h.  Every call goes through the C ABI of
variantdbscan_gb300/lib/libSharedVDBSCAN.so; there is no CPU fallback: if the
library or a CUDA device is missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np
import numpy.ctypeslib as npct

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libSharedVDBSCAN.so")

VDB_OK = 0
ERRORS = {
    -1: "invalid argument",
    -2: "degenerate bounding box",
    -3: "CUDA error",
    -4: "out of device memory",
    -5: "internal list capacity exceeded",
    -6: "no CUDA device",
    -7: "input too large",
}
PRECISION = {"mixed": 0, "fp64": 1}
TABLE_ROWS = {"all": 0, "border": 1}
SCHEDULE = {"batched": 0, "plain": 1}
LOC_HOST, LOC_DEVICE = 0, 1
# stats["graph"] (vdb_stats.graph)
GRAPH_NONE, GRAPH_CAPTURED, GRAPH_REPLAYED, GRAPH_FALLBACK, GRAPH_UNSUPPORTED = 0, 1, 2, 3, 4

# names exported by the library (declared in include/vdbscan.h)
EXPORTS = ["libVDBSCAN", "vdb_default_options", "vdb_context_create", "vdb_context_destroy",
           "vdb_run_batch", "vdb_run_noalloc", "vdb_import_dataset", "vdb_import_variants",
           "vdb_last_error", "vdb_version"]


class VDBError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}){': ' + msg if msg else ''}")
        self.code = code


class Dataset(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("n", ctypes.c_uint32),
                ("mbb_size", ctypes.c_int32), ("eps", ctypes.c_void_p),
                ("minpts", ctypes.c_void_p), ("nv", ctypes.c_uint32),
                ("labels", ctypes.c_void_p)]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("schedule", ctypes.c_int32),
                ("location", ctypes.c_int32), ("cells_per_eps", ctypes.c_int32),
                ("verbose", ctypes.c_int32), ("table_budget_bytes", ctypes.c_int64),
                ("streams", ctypes.c_int32), ("table_rows", ctypes.c_int32),
                ("table_hash", ctypes.c_int32), ("table_entry_bytes", ctypes.c_int32),
                ("no_reuse", ctypes.c_int32), ("tile_cells", ctypes.c_int32),
                ("unit_candidates", ctypes.c_int32), ("graph", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_uint64), ("candidates", ctypes.c_uint64),
                ("retested", ctypes.c_uint64), ("asymmetric_pairs", ctypes.c_uint64),
                ("tables", ctypes.c_uint32), ("table_chunks", ctypes.c_uint32),
                ("kernel_launches", ctypes.c_uint32), ("clusters", ctypes.c_uint32),
                ("ms_index", ctypes.c_double), ("ms_count", ctypes.c_double),
                ("ms_table", ctypes.c_double), ("ms_cluster", ctypes.c_double),
                ("ms_total", ctypes.c_double), ("table_hash", ctypes.c_uint64),
                ("entry_bytes", ctypes.c_uint64), ("compact_tables", ctypes.c_uint32),
                ("pad", ctypes.c_uint32), ("reuse_skipped_pairs", ctypes.c_uint64),
                ("tables_by_tile_cells", ctypes.c_uint32 * 8), ("worker_streams", ctypes.c_uint32),
                ("pad2", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64),
                ("table_bytes", ctypes.c_uint64), ("graph", ctypes.c_uint32),
                ("graph_checks", ctypes.c_uint32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["tables_by_tile_cells"] = list(d["tables_by_tile_cells"])
        return d


_LIB = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the CUDA library (raises if it was not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    d1 = npct.ndpointer(dtype=np.float64, ndim=1, flags="C_CONTIGUOUS")
    u1 = npct.ndpointer(dtype=np.uint32, ndim=1, flags="C_CONTIGUOUS")
    lib.libVDBSCAN.restype = ctypes.c_int
    lib.libVDBSCAN.argtypes = [d1, d1, ctypes.c_uint, d1, u1, ctypes.c_uint, ctypes.c_int, u1,
                               ctypes.c_bool]
    lib.vdb_default_options.argtypes = [ctypes.POINTER(Options)]
    lib.vdb_default_options.restype = None
    lib.vdb_context_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
    lib.vdb_context_create.restype = ctypes.c_int
    lib.vdb_context_destroy.argtypes = [ctypes.c_void_p]
    lib.vdb_context_destroy.restype = None
    lib.vdb_run_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(Dataset), ctypes.c_int,
                                  ctypes.POINTER(Options), ctypes.POINTER(Stats)]
    lib.vdb_run_batch.restype = ctypes.c_int
    lib.vdb_last_error.argtypes = [ctypes.c_void_p]
    lib.vdb_last_error.restype = ctypes.c_char_p
    lib.vdb_version.argtypes = []
    lib.vdb_version.restype = ctypes.c_char_p
    for name in ("vdb_import_dataset", "vdb_import_variants"):
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                       ctypes.POINTER(ctypes.c_uint32)]
        fn.restype = ctypes.c_int
    _LIB = lib
    return lib


def _convert(a, dtype):
    # variantdbscan.py:74-87: coerce dtype and contiguity
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def VariantDBSCAN(eps_array, mp_array, x_array, y_array, mbbsize=70, verbose=False):
    """Drop-in for the reference's VariantDBSCAN (variantdbscan.py:32-109):
    returns the (N,) labels for one variant, (N, V) for several; 0 = noise."""
    lib = load_library()
    eps = _convert(np.atleast_1d(eps_array), np.float64)
    mp = _convert(np.atleast_1d(mp_array), np.uint32)
    x = _convert(x_array, np.float64)
    y = _convert(y_array, np.float64)
    if len(eps) != len(mp):
        raise ValueError("eps_array and mp_array must have the same length")
    res = np.zeros(len(x) * len(eps), dtype=np.uint32)
    rc = lib.libVDBSCAN(x, y, len(x), eps, mp, len(eps), int(mbbsize), res, bool(verbose))
    if rc != VDB_OK:
        raise VDBError(rc)
    if len(eps) > 1:
        res = res.reshape([len(eps), len(x)]).T
    return res


@dataclass
class BatchItem:
    x: object
    y: object
    eps: object
    minpts: object
    mbb_size: int = 70
    labels: np.ndarray | None = None   # optional (V, N) uint32 output buffer


class Context:
    """A vdb_context: its own CUDA stream and cached device memory."""

    def __init__(self, stream: int | None = None):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.vdb_context_create(ctypes.byref(h), stream)
        if rc != VDB_OK:
            raise VDBError(rc)
        self.h = h

    def close(self):
        if self.h:
            self.lib.vdb_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self.lib.vdb_last_error(self.h).decode()

    def run(self, items, precision="mixed", schedule="batched", cells_per_eps=0,
            budget=0, verbose=False, streams=0, table="all", table_hash=False, entry_bytes=0,
            reuse=True, tile_cells=0, graph=False, unit_candidates=0):
        """Clusters host (numpy) datasets; returns ([(V, N) uint32 labels], stats).
        graph=True replays repeated calls of the same shape as one CUDA graph
        (stats["graph"]: GRAPH_CAPTURED on the first, GRAPH_REPLAYED after)."""
        keep, dss, outs = [], [], []
        for it in items:
            x = _convert(it.x, np.float64)
            y = _convert(it.y, np.float64)
            eps = _convert(np.atleast_1d(it.eps), np.float64)
            mp = _convert(np.atleast_1d(it.minpts), np.uint32)
            lab = it.labels
            if lab is None:
                lab = np.zeros((len(eps), len(x)), np.uint32)
            elif (lab.dtype != np.uint32 or lab.shape != (len(eps), len(x))
                  or not lab.flags["C_CONTIGUOUS"]):
                raise ValueError("labels must be a C-contiguous (V, N) uint32 array")
            keep += [x, y, eps, mp, lab]
            outs.append(lab)
            dss.append(Dataset(x.ctypes.data, y.ctypes.data, len(x), int(it.mbb_size),
                               eps.ctypes.data, mp.ctypes.data, len(eps), lab.ctypes.data))
        arr = (Dataset * len(dss))(*dss)
        st = self._call(arr, len(dss), precision, schedule, LOC_HOST, cells_per_eps, budget,
                        verbose, streams, table, table_hash, entry_bytes, reuse, tile_cells,
                        graph, unit_candidates)
        return outs, st

    def run_device(self, x_ptr, y_ptr, n, eps, minpts, labels_ptr, mbb_size=70,
                   precision="mixed", schedule="batched", cells_per_eps=0, budget=0,
                   table="all", table_hash=False, entry_bytes=0, reuse=True, tile_cells=0,
                   graph=False, unit_candidates=0):
        """Clusters one dataset already resident on the device (raw pointers,
        e.g. torch.Tensor.data_ptr()); labels_ptr receives V*n uint32.  The
        inputs must be complete on the context's stream (synchronize after
        producing them on another stream)."""
        eps = _convert(np.atleast_1d(eps), np.float64)
        mp = _convert(np.atleast_1d(minpts), np.uint32)
        ds = (Dataset * 1)(Dataset(x_ptr, y_ptr, n, int(mbb_size), eps.ctypes.data,
                                   mp.ctypes.data, len(eps), labels_ptr))
        return self._call(ds, 1, precision, schedule, LOC_DEVICE, cells_per_eps, budget, False,
                          0, table, table_hash, entry_bytes, reuse, tile_cells, graph,
                          unit_candidates)

    def run_device_batch(self, items, mbb_size=70, precision="mixed", schedule="batched",
                         cells_per_eps=0, budget=0, streams=0, table="all", table_hash=False,
                         entry_bytes=0, reuse=True, tile_cells=0, graph=False,
                         unit_candidates=0):
        """Clusters several device-resident datasets in one call.  items:
        (x_ptr, y_ptr, n, eps, minpts, labels_ptr) tuples; each labels_ptr
        receives V*n uint32."""
        keep, dss = [], []
        for (xp, yp, n, eps, mp, lp) in items:
            eps = _convert(np.atleast_1d(eps), np.float64)
            mp = _convert(np.atleast_1d(mp), np.uint32)
            keep += [eps, mp]
            dss.append(Dataset(xp, yp, n, int(mbb_size), eps.ctypes.data, mp.ctypes.data,
                               len(eps), lp))
        arr = (Dataset * len(dss))(*dss)
        return self._call(arr, len(dss), precision, schedule, LOC_DEVICE, cells_per_eps, budget,
                          False, streams, table, table_hash, entry_bytes, reuse, tile_cells,
                          graph, unit_candidates)

    def _call(self, arr, nds, precision, schedule, location, cells_per_eps, budget, verbose,
              streams=0, table="all", table_hash=False, entry_bytes=0, reuse=True,
              tile_cells=0, graph=False, unit_candidates=0):
        o = Options()
        self.lib.vdb_default_options(ctypes.byref(o))
        o.precision = PRECISION[precision]
        o.schedule = SCHEDULE[schedule]
        o.location = location
        o.cells_per_eps = int(cells_per_eps)
        o.verbose = int(bool(verbose))
        o.table_budget_bytes = int(budget)
        o.streams = int(streams)
        o.table_rows = TABLE_ROWS[table]
        o.table_hash = int(bool(table_hash))
        o.table_entry_bytes = int(entry_bytes)
        o.no_reuse = 0 if reuse else 1
        o.tile_cells = int(tile_cells)
        o.graph = int(bool(graph))
        o.unit_candidates = int(unit_candidates)
        st = Stats()
        rc = self.lib.vdb_run_batch(self.h, arr, nds, ctypes.byref(o), ctypes.byref(st))
        if rc != VDB_OK:
            raise VDBError(rc, self.last_error())
        return st.as_dict()


def _import(fn, path, dt_a, dt_b):
    # first call counts, second call fills
    n = ctypes.c_uint32(0)
    rc = fn(os.fsencode(path), None, None, 0, ctypes.byref(n))
    if rc != VDB_OK:
        raise VDBError(rc, f"cannot read {path}")
    a = np.zeros(n.value, dt_a)
    b = np.zeros(n.value, dt_b)
    rc = fn(os.fsencode(path), a.ctypes.data, b.ctypes.data, n.value, ctypes.byref(n))
    if rc != VDB_OK:
        raise VDBError(rc, f"cannot read {path}")
    return a, b


def import_dataset(path):
    """(x, y) of a dataset file read as the reference's GPU prototype reads it
    (src/gpu/import_dataset.cpp:63-134): lines "longitude,latitude[,...]",
    x = the latitude mapped to [0, 180], y = the longitude."""
    return _import(load_library().vdb_import_dataset, path, np.float64, np.float64)


def import_variants(path):
    """(eps, minpts) of a variant file ("epsilon,minpts" lines), sorted by
    epsilon descending, then minpts ascending (src/gpu/import_dataset.cpp:41-49,
    232-262)."""
    return _import(load_library().vdb_import_variants, path, np.float64, np.uint32)


def version() -> str:
    return load_library().vdb_version().decode()
