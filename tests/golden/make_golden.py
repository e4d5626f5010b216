"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run with VDB_REFERENCE_DIR naming a checkout of the reference sources:

    VDB_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py

Sources of truth:
  * reference_test_dataset.npz: the reference's own fixture pair
    src/test_dataset.csv + src/test_output.csv (225 points, variants
    eps=1.0/minpts=10 and eps=0.5/minpts=12 from src/c_test_prog.cpp:124-134).
  * every other case: labels produced by the reference CPU library
    (oracle/_ref/libSharedVDBSCAN.so, built by oracle/build_ref.sh) called with
    numVariants=1 per variant, i.e. the from-scratch path
    (src/DBScan.cpp:523-609).  The "multi" arrays hold the labels of one call
    with all variants (the reference's cluster-reuse path), kept for
    information only.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import ReferenceLibrary, RestatedOracle, build_reference  # noqa: E402
from variantdbscan_gb300 import synthetic as syn  # noqa: E402

REF = os.environ.get("VDB_REFERENCE_DIR", "")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("make_golden.py: set VDB_REFERENCE_DIR to a checkout of the reference sources")


def _save(name, **arrs):
    np.savez_compressed(os.path.join(HERE, name), **arrs)
    print("wrote", name, {k: getattr(v, "shape", v) for k, v in arrs.items()})


def _case(ref, x, y, eps, mp, mbb=70):
    eps = np.asarray(eps, np.float64)
    mp = np.asarray(mp, np.uint32)
    lab = ref.variants(x, y, eps, mp, mbb)
    return dict(x=np.asarray(x, np.float64), y=np.asarray(y, np.float64), eps=eps,
                minpts=mp, mbb=np.int32(mbb), labels=lab.astype(np.uint32))


def _adversarial(orc, ref, want=24, seed=7):
    """Small lattice sets (MBBsize 1-3) where the reference's neighbour relation
    is not symmetric between two core points of different components: the
    R-tree box test (src/RTree.h:1613-1625) rejects a pair that the distance
    test (src/DBScan.cpp:687) accepts in one direction only."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import connected_components
    rng = np.random.default_rng(seed)
    xs, ys, epss, mps, mbbs, labs, ns = [], [], [], [], [], [], []
    trial = 0
    while len(ns) < want and trial < 20000:
        trial += 1
        eps = float(rng.choice([0.05, 0.25, 0.5, 0.03]))
        n = int(rng.integers(20, 200))
        span = int(rng.integers(20, 120))
        k = rng.integers(-span, span, size=(n, 2))
        if rng.random() < 0.5:
            k[:, 1] = 0
        x = k[:, 0] / 100.0
        y = k[:, 1] / 100.0
        mbb = int(rng.choice([1, 1, 2, 3]))
        off, nb = orc.neighbor_lists(x, y, eps, mbb)
        rows = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
        a = csr_matrix((np.ones(len(nb)), (rows, nb)), shape=(n, n))
        cnt = np.diff(off)
        s = a.multiply(a.T)
        for mp in (1, 2, 3):
            core = cnt >= mp
            _, lab = connected_components(s[core][:, core], directed=False)
            r, c = a[core][:, core].nonzero()
            if (lab[r] != lab[c]).any():
                xs.append(x); ys.append(y); epss.append(eps); mps.append(mp)
                mbbs.append(mbb); ns.append(n)
                labs.append(ref.variants(x, y, [eps], [mp], mbb)[0])
                break
    off = np.zeros(len(ns) + 1, np.int64)
    off[1:] = np.cumsum(ns)
    return dict(offsets=off, x=np.concatenate(xs), y=np.concatenate(ys),
                eps=np.array(epss), minpts=np.array(mps, np.uint32),
                mbb=np.array(mbbs, np.int32), labels=np.concatenate(labs).astype(np.uint32))


def main():
    if build_reference() is None:
        sys.exit("reference library could not be built")
    ref = ReferenceLibrary()
    orc = RestatedOracle()

    ds = np.loadtxt(os.path.join(REF, "src", "test_dataset.csv"), delimiter=",")
    out = np.loadtxt(os.path.join(REF, "src", "test_output.csv"), delimiter=",")
    x, y = ds[:, 0].copy(), ds[:, 1].copy()
    eps = np.array([1.0, 0.5])
    mp = np.array([10, 12], np.uint32)
    multi = ref.run(x, y, eps, mp)
    assert (multi == out[:, 2:4].T).all(), "reference no longer reproduces test_output.csv"
    _save("reference_test_dataset.npz", x=x, y=y, eps=eps, minpts=mp, mbb=np.int32(70),
          labels=out[:, 2:4].T.astype(np.uint32), multi=multi)

    # the four collinear points of src/vtest.py, eps = sqrt(2) +- 0.01, minpts 2
    xv = np.array([3.0, 2.0, 8.0, 1.0])
    ev = np.array([np.sqrt(2) + 0.01, np.sqrt(2) - 0.01])
    _save("vtest.npz", **_case(ref, xv, xv.copy(), ev, [2, 2]))

    d = syn.single_variant(n=3000, seed=0)
    _save("single_variant_3k.npz", **_case(ref, d.x, d.y, [0.5, 0.5, 1.0, 2.0], [10, 4, 10, 30]))

    d = syn.variant_sweep(n=4000, seed=1)
    c = _case(ref, d.x, d.y, d.eps, d.minpts)
    c["multi"] = ref.run(d.x, d.y, d.eps, d.minpts)
    _save("variant_sweep_4k.npz", **c)

    d = syn.lattice_stress(n=4000, seed=3)
    _save("lattice_4k.npz", **_case(ref, d.x, d.y, [1.0, 2.0, 3.0, 5.0], [8, 32, 8, 32]))

    d = syn.lattice_stress(n=3000, seed=33)
    _save("lattice_4k_mbb1.npz", **_case(ref, d.x, d.y, [1.0, 2.0, 3.0], [4, 8, 16], mbb=1))

    # duplicates, negative coordinates (max initialised to DBL_MIN,
    # src/main.cpp:467-468), minpts 0 and 1, a zero and a negative epsilon
    rng = np.random.default_rng(11)
    xe = np.round(rng.uniform(-5, -1, 600), 1)
    ye = np.round(rng.uniform(-3, -2, 600), 1)
    _save("edge_negative_dupes.npz",
          **_case(ref, xe, ye, [0.15, 0.0, 0.3, -1.0, 0.2], [3, 2, 0, 0, 1]))

    _save("adversarial_asymmetric.npz", **_adversarial(orc, ref))


if __name__ == "__main__":
    main()
