"""Parity at the benchmark workloads' full sizes, at every epsilon.

* variant sweep, 2,000,000 points: for each of the four epsilons, the
  neighbour table built by the batched mixed-precision path has the restated
  oracle's table hash (rows, entries and one-way flags of every point) and the
  plain FP64 path's; the labels of the eps 0.1 and 0.2 variants equal the
  oracle's.
* lattice, 10,000,000 points on a 0.01 deg grid (many pairs exactly at eps):
  the eps 0.25 and 0.5 tables (row-chunked: they exceed device memory) have
  the oracle's hash and the FP64 path's; the eps 0.05 labels equal the
  oracle's.
* multi-dataset batch, 64 datasets: one batched mixed call against one plain
  FP64 call (labels and table hashes), and every dataset of at most 200,000
  points against the oracle.
* single variant, 50,000 points: the compiled reference library itself
  (libVDBSCAN with numVariants=1) gives the same labels.

The oracle is the C restatement of the reference's one-variant path
(oracle/vdbscan_oracle.c), pinned against the reference's fixtures by
tests/test_oracle_golden.py.
"""
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

MASK64 = (1 << 64) - 1


@pytest.fixture(scope="module")
def vdb():
    import variantdbscan_gb300 as v
    from variantdbscan_gb300 import build
    build.build()
    return v


@pytest.fixture(scope="module")
def ctx(vdb):
    c = vdb.Context()
    yield c
    c.close()


def _one(ctx, vdb, x, y, eps, mp, **kw):
    out, st = ctx.run([vdb.BatchItem(x, y, eps, mp)], **kw)
    return out[0], st


@pytest.fixture(scope="module")
def sweep():
    from variantdbscan_gb300 import synthetic as syn
    return syn.variant_sweep(n=2_000_000, seed=1)


@pytest.mark.parametrize("eps", [0.1, 0.2, 0.4, 0.8])
def test_variant_sweep_table_every_eps(ctx, vdb, orc, sweep, eps):
    d = sweep
    sel = np.flatnonzero(d.eps == eps)
    mixed, sm = _one(ctx, vdb, d.x, d.y, d.eps[sel], d.minpts[sel], table_hash=True)
    assert sm["tables"] == 1
    want = orc.table_hash(d.x, d.y, eps)
    assert sm["table_hash"] == want, f"eps {eps}: table differs from the oracle's"
    # the plain FP64 path builds the same table once per variant
    plain, sp = _one(ctx, vdb, d.x, d.y, d.eps[sel], d.minpts[sel], table_hash=True,
                     precision="fp64", schedule="plain")
    assert sp["tables"] == len(sel)
    assert sp["table_hash"] == (len(sel) * want) & MASK64
    assert sp["pairs"] == len(sel) * sm["pairs"]
    np.testing.assert_array_equal(mixed, plain)
    if eps <= 0.2:
        np.testing.assert_array_equal(mixed, orc.variants(d.x, d.y, d.eps[sel], d.minpts[sel]))


def test_variant_sweep_all_variants_one_call(ctx, vdb, sweep):
    # the bench's step (16 variants in one call) gives every variant the
    # labels of its own epsilon's call (checked against the oracle above),
    # and its four tables the same hashes
    d = sweep
    lab, st = _one(ctx, vdb, d.x, d.y, d.eps, d.minpts, table_hash=True)
    assert st["tables"] == 4
    total = 0
    for eps in (0.1, 0.2, 0.4, 0.8):
        sel = np.flatnonzero(d.eps == eps)
        part, sp = _one(ctx, vdb, d.x, d.y, d.eps[sel], d.minpts[sel], table_hash=True)
        np.testing.assert_array_equal(lab[sel], part, err_msg=f"eps {eps}")
        total += sp["table_hash"]
    assert st["table_hash"] == total & MASK64


@pytest.fixture(scope="module")
def lattice():
    from variantdbscan_gb300 import synthetic as syn
    return syn.lattice_stress(n=10_000_000, seed=3)


@pytest.mark.parametrize("eps", [0.25, 0.5])
def test_lattice_large_eps_tables(ctx, vdb, orc, lattice, eps):
    d = lattice
    sel = np.flatnonzero(d.eps == eps)
    mixed, sm = _one(ctx, vdb, d.x, d.y, d.eps[sel], d.minpts[sel], table_hash=True)
    assert sm["retested"] > 0
    fp64, sf = _one(ctx, vdb, d.x, d.y, d.eps[sel], d.minpts[sel], table_hash=True,
                    precision="fp64")
    assert sm["pairs"] == sf["pairs"]
    assert sm["table_hash"] == sf["table_hash"], f"eps {eps}: mixed differs from FP64"
    assert sm["table_hash"] == orc.table_hash(d.x, d.y, eps), f"eps {eps}: differs from oracle"
    np.testing.assert_array_equal(mixed, fp64)


def test_lattice_small_eps_labels_vs_oracle(ctx, vdb, orc, lattice):
    d = lattice
    sel = np.flatnonzero(d.eps == 0.05)
    lab, st = _one(ctx, vdb, d.x, d.y, d.eps[sel], d.minpts[sel], table_hash=True)
    assert st["table_hash"] == orc.table_hash(d.x, d.y, 0.05)
    np.testing.assert_array_equal(lab, orc.variants(d.x, d.y, d.eps[sel], d.minpts[sel]))


def test_multi_dataset_full_batch(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    dss = syn.multi_dataset(count=64, seed=2)
    items = [vdb.BatchItem(d.x, d.y, d.eps, d.minpts) for d in dss]
    mixed, sm = ctx.run(items, table_hash=True)
    plain, sp = ctx.run(items, table_hash=True, precision="fp64", schedule="plain")
    # one table per distinct epsilon (batched) against one per variant (plain)
    assert all(len(np.unique(d.eps)) == len(d.eps) for d in dss)
    assert sm["tables"] == sp["tables"] == sum(len(d.eps) for d in dss)
    assert sm["table_hash"] == sp["table_hash"] and sm["pairs"] == sp["pairs"]
    checked = 0
    for i, (d, a, b) in enumerate(zip(dss, mixed, plain)):
        np.testing.assert_array_equal(a, b, err_msg=f"dataset {i}")
        if d.n <= 200_000:
            np.testing.assert_array_equal(a, orc.variants(d.x, d.y, d.eps, d.minpts),
                                          err_msg=f"dataset {i} vs oracle")
            checked += 1
    assert checked >= 30


def test_single_variant_vs_compiled_reference(vdb):
    from oracle.oracle import REF_SO, ReferenceLibrary
    if not os.path.exists(REF_SO):
        pytest.skip("reference library not built")
    from variantdbscan_gb300 import synthetic as syn
    d = syn.single_variant()  # 50,000 points, eps 0.5, minpts 10
    ref = ReferenceLibrary()
    want = ref.variants(d.x, d.y, d.eps, d.minpts)
    got = vdb.VariantDBSCAN(d.eps, d.minpts, d.x, d.y)
    assert want.max() > 0
    np.testing.assert_array_equal(got, want[0])
