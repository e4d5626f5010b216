"""ctypes front-end for the two CPU checkers.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.

* ``RestatedOracle`` loads ``oracle/_build/liborc_vdbscan.so`` (built from
  ``oracle/vdbscan_oracle.c``), a plain-C restatement of the reference's
  one-variant path (binDataset, src/main.cpp:459-605; filterCandidatesMPB and
  EuclidianDistance, src/DBScan.cpp:665-702; algDBScanParallel,
  src/DBScan.cpp:523-609).
* ``ReferenceLibrary`` loads ``oracle/_ref/libSharedVDBSCAN.so``, the
  reference's own CPU library compiled by ``oracle/build_ref.sh`` with the
  one-line missing-return fix.  Its entry point is the reference C ABI
  ``libVDBSCAN`` (src/main.cpp:50), bound with the argtypes of the reference's
  Python wrapper (python_package/vdbscan/variantdbscan.py:66-69).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import numpy.ctypeslib as npct

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_SO = os.path.join(HERE, "_build", "liborc_vdbscan.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libSharedVDBSCAN.so")

_d1 = npct.ndpointer(dtype=np.float64, ndim=1, flags="C_CONTIGUOUS")
_u1 = npct.ndpointer(dtype=np.uint32, ndim=1, flags="C_CONTIGUOUS")
_u64 = npct.ndpointer(dtype=np.uint64, ndim=1, flags="C_CONTIGUOUS")


def build_restated() -> str:
    subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    return ORC_SO


def build_reference() -> str | None:
    """Builds oracle/_ref from the reference checkout or the staged copy.
    Returns None when neither is available."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")],
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleError(RuntimeError):
    pass


class RestatedOracle:
    def __init__(self, path: str = ORC_SO):
        if not os.path.exists(path):
            build_restated()
        lib = ctypes.CDLL(path)
        lib.orc_visit_order.argtypes = [_d1, _d1, ctypes.c_uint32, _u1]
        lib.orc_visit_order.restype = ctypes.c_int
        lib.orc_visit_keys.argtypes = [_d1, _d1, ctypes.c_uint32, _u1]
        lib.orc_visit_keys.restype = ctypes.c_int
        lib.orc_eps_sq_threshold.argtypes = [ctypes.c_double]
        lib.orc_eps_sq_threshold.restype = ctypes.c_double
        lib.orc_neighbor_counts.argtypes = [_d1, _d1, ctypes.c_uint32, ctypes.c_double,
                                            ctypes.c_int, _u1,
                                            ctypes.POINTER(ctypes.c_uint64)]
        lib.orc_neighbor_counts.restype = ctypes.c_int
        lib.orc_neighbor_lists.argtypes = [_d1, _d1, ctypes.c_uint32, ctypes.c_double,
                                           ctypes.c_int, _u64, _u1]
        lib.orc_neighbor_lists.restype = ctypes.c_int
        lib.orc_neighbor_counts_bruteforce.argtypes = [_d1, _d1, ctypes.c_uint32,
                                                       ctypes.c_double, ctypes.c_int, _u1]
        lib.orc_neighbor_counts_bruteforce.restype = ctypes.c_int
        lib.orc_dbscan.argtypes = [_d1, _d1, ctypes.c_uint32, ctypes.c_double,
                                   ctypes.c_uint32, ctypes.c_int, _u1,
                                   ctypes.POINTER(ctypes.c_uint32)]
        lib.orc_dbscan.restype = ctypes.c_int
        lib.orc_dbscan_many.argtypes = [_d1, _d1, ctypes.c_uint32, _d1, _u1, ctypes.c_uint32,
                                        ctypes.c_int, _u1]
        lib.orc_dbscan_many.restype = ctypes.c_int
        lib.orc_table_hash.argtypes = [_d1, _d1, ctypes.c_uint32, ctypes.c_double, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_uint64)]
        lib.orc_table_hash.restype = ctypes.c_int
        self.lib = lib

    def visit_order(self, x, y):
        x, y = _f64(x), _f64(y)
        m = np.zeros(len(x), np.uint32)
        rc = self.lib.orc_visit_order(x, y, len(x), m)
        if rc:
            raise OracleError(f"orc_visit_order rc={rc}")
        return m

    def eps_threshold(self, eps: float) -> float:
        return self.lib.orc_eps_sq_threshold(float(eps))

    def neighbor_counts(self, x, y, eps, mbb=70, bruteforce=False):
        x, y = _f64(x), _f64(y)
        c = np.zeros(len(x), np.uint32)
        if bruteforce:
            rc = self.lib.orc_neighbor_counts_bruteforce(x, y, len(x), float(eps), mbb, c)
        else:
            tot = ctypes.c_uint64(0)
            rc = self.lib.orc_neighbor_counts(x, y, len(x), float(eps), mbb, c,
                                              ctypes.byref(tot))
        if rc:
            raise OracleError(f"orc_neighbor_counts rc={rc}")
        return c

    def neighbor_lists(self, x, y, eps, mbb=70):
        """CSR (offsets, neighbours) in input indices; rows unsorted."""
        x, y = _f64(x), _f64(y)
        c = self.neighbor_counts(x, y, eps, mbb)
        off = np.zeros(len(x) + 1, np.uint64)
        np.cumsum(c, out=off[1:])
        nb = np.zeros(int(off[-1]), np.uint32)
        rc = self.lib.orc_neighbor_lists(x, y, len(x), float(eps), mbb, off, nb)
        if rc:
            raise OracleError(f"orc_neighbor_lists rc={rc}")
        return off, nb

    def table_hash(self, x, y, eps, mbb=70) -> int:
        """Checksum of N(p) for every p (the library's vdb_stats.table_hash of
        one epsilon's table)."""
        x, y = _f64(x), _f64(y)
        h = ctypes.c_uint64(0)
        rc = self.lib.orc_table_hash(x, y, len(x), float(eps), mbb, ctypes.byref(h))
        if rc:
            raise OracleError(f"orc_table_hash rc={rc}")
        return h.value

    def dbscan(self, x, y, eps, minpts, mbb=70):
        x, y = _f64(x), _f64(y)
        lab = np.zeros(len(x), np.uint32)
        k = ctypes.c_uint32(0)
        rc = self.lib.orc_dbscan(x, y, len(x), float(eps), int(minpts), mbb, lab,
                                 ctypes.byref(k))
        if rc:
            raise OracleError(f"orc_dbscan rc={rc}")
        return lab

    def variants(self, x, y, eps, minpts, mbb=70):
        """(V, N) labels, each variant clustered on its own (orc_dbscan_many:
        counts shared per epsilon, variants labelled in parallel threads)."""
        x, y = _f64(x), _f64(y)
        eps = _f64(np.atleast_1d(eps))
        mp = np.ascontiguousarray(np.atleast_1d(minpts), dtype=np.uint32)
        lab = np.zeros(len(eps) * len(x), np.uint32)
        rc = self.lib.orc_dbscan_many(x, y, len(x), eps, mp, len(eps), mbb, lab)
        if rc:
            raise OracleError(f"orc_dbscan_many rc={rc}")
        return lab.reshape(len(eps), len(x))


class ReferenceLibrary:
    """The reference's own libVDBSCAN (src/main.cpp:50)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise OracleError(f"reference library not built: {path}")
        lib = ctypes.CDLL(path)
        lib.libVDBSCAN.restype = ctypes.c_int
        lib.libVDBSCAN.argtypes = [_d1, _d1, ctypes.c_uint, _d1, _u1, ctypes.c_uint,
                                   ctypes.c_int, _u1, ctypes.c_bool]
        self.lib = lib
        try:
            with open(os.path.join(os.path.dirname(path), "NSEARCHTHREADS")) as f:
                self.threads = int(f.read().strip())
        except OSError:
            self.threads = os.cpu_count() or 1

    def run(self, x, y, eps, minpts, mbb=70):
        """One libVDBSCAN call with all variants; (V, N) labels."""
        x, y = _f64(x), _f64(y)
        eps = _f64(np.atleast_1d(eps))
        mp = np.ascontiguousarray(np.atleast_1d(minpts), dtype=np.uint32)
        out = np.zeros(len(x) * len(eps), np.uint32)
        self.lib.libVDBSCAN(x, y, len(x), eps, mp, len(eps), mbb, out, False)
        return out.reshape(len(eps), len(x))

    def variants(self, x, y, eps, minpts, mbb=70):
        """(V, N) labels, one numVariants=1 call per variant (the standalone
        algDBScanParallel path, src/DBScan.cpp:523-609)."""
        return np.stack([self.run(x, y, [e], [m], mbb)[0] for e, m in zip(eps, minpts)])
