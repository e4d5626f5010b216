"""GPU parity tests: the CUDA path (through the C ABI) against the reference's
labels (golden fixtures made by the reference library) and the restated
oracle.  Labels must be identical values, not just the same partition."""
import numpy as np
import pytest

from golden_cases import CASES, adversarial, load

pytestmark = pytest.mark.gpu


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


def _run(ctx, vdb, x, y, eps, mp, mbb=70, **kw):
    out, st = ctx.run([vdb.BatchItem(x, y, eps, mp, mbb)], **kw)
    return out[0], st


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_golden_labels_per_variant(ctx, vdb, name, precision):
    c = load(name)
    mbb = int(c["mbb"])
    for v in range(len(c["eps"])):
        lab, _ = _run(ctx, vdb, c["x"], c["y"], [c["eps"][v]], [c["minpts"][v]], mbb,
                      precision=precision)
        np.testing.assert_array_equal(lab[0], c["labels"][v], err_msg=f"{name} v{v}")


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("schedule", ["batched", "plain"])
def test_golden_labels_all_variants_one_call(ctx, vdb, name, schedule):
    c = load(name)
    lab, _ = _run(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], int(c["mbb"]),
                  schedule=schedule)
    np.testing.assert_array_equal(lab, c["labels"])


def test_reference_abi_libVDBSCAN(vdb):
    # the reference's own entry point and wrapper semantics (variantdbscan.py:101-107)
    c = load("reference_test_dataset")
    res = vdb.VariantDBSCAN(c["eps"], c["minpts"], c["x"], c["y"])
    assert res.shape == (225, 2) and res.dtype == np.uint32
    np.testing.assert_array_equal(res.T, c["labels"])
    one = vdb.VariantDBSCAN([1.0], [10], c["x"], c["y"])
    assert one.shape == (225,)
    np.testing.assert_array_equal(one, c["labels"][0])


def test_vtest_known_answer(vdb):
    x = np.array([3, 2, 8, 1])
    res = vdb.VariantDBSCAN(np.array([np.sqrt(2) + 0.01, np.sqrt(2) - 0.01]),
                            np.array([2, 2]), x, x)
    np.testing.assert_array_equal(res, [[1, 0], [1, 0], [0, 0], [1, 0]])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_adversarial_one_way_edges(ctx, vdb, precision):
    for i, c in enumerate(adversarial()):
        lab, st = _run(ctx, vdb, c["x"], c["y"], [c["eps"]], [c["minpts"]], c["mbb"],
                       precision=precision)
        np.testing.assert_array_equal(lab[0], c["labels"], err_msg=f"case {i}")


@pytest.mark.parametrize("cpe", [1, 2, 3])
def test_grid_resolution_does_not_change_labels(ctx, vdb, cpe):
    c = load("variant_sweep_4k")
    lab, _ = _run(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], cells_per_eps=cpe)
    np.testing.assert_array_equal(lab, c["labels"])


def test_single_variant_full_size_vs_oracle(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    d = syn.single_variant()  # 50,000 points, eps 0.5, minpts 10
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts)
    want = orc.dbscan(d.x, d.y, d.eps[0], d.minpts[0])
    np.testing.assert_array_equal(lab[0], want)
    counts = orc.neighbor_counts(d.x, d.y, d.eps[0])
    assert st["pairs"] == int(counts.sum())


def test_variant_sweep_medium_vs_oracle(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts)
    want = orc.variants(d.x, d.y, d.eps, d.minpts)
    np.testing.assert_array_equal(lab, want)
    assert st["tables"] == 4
    assert st["clusters"] == int(sum(int(lab[v].max()) for v in range(len(d.eps))))


def test_lattice_medium_vs_oracle(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    d = syn.lattice_stress(n=100_000, seed=3)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts)
    want = orc.variants(d.x, d.y, d.eps, d.minpts)
    np.testing.assert_array_equal(lab, want)
    assert st["retested"] > 0


def test_lattice_mixed_equals_fp64_pairs(ctx, vdb):
    from variantdbscan_gb300 import synthetic as syn
    d = syn.lattice_stress(n=300_000, seed=3)
    a, sa = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, precision="mixed")
    b, sb = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, precision="fp64")
    assert sa["pairs"] == sb["pairs"]
    np.testing.assert_array_equal(a, b)


def test_multi_dataset_batch(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    dss = syn.multi_dataset(count=6, seed=2, n_lo=2000, n_hi=30000)
    items = [vdb.BatchItem(d.x, d.y, d.eps, d.minpts) for d in dss]
    outs, _ = ctx.run(items)
    for d, lab in zip(dss, outs):
        np.testing.assert_array_equal(lab, orc.variants(d.x, d.y, d.eps, d.minpts))


def test_edge_inputs(ctx, vdb):
    # one point at the origin: max initialised to DBL_MIN keeps the width positive
    lab, _ = _run(ctx, vdb, [0.0], [0.0], [1.0], [1])
    np.testing.assert_array_equal(lab, [[1]])
    # empty input
    lab, _ = _run(ctx, vdb, np.zeros(0), np.zeros(0), [1.0], [1])
    assert lab.shape == (1, 0)
    # zero-width box: the reference reports bins out of range
    with pytest.raises(vdb.VDBError) as e:
        _run(ctx, vdb, [1.0, 1.0, 1.0], [2.0, 3.0, 4.0], [1.0], [1])
    assert e.value.code == -2
    # NaN coordinate and MBBsize 0 are rejected
    with pytest.raises(vdb.VDBError) as e:
        _run(ctx, vdb, [1.0, np.nan], [2.0, 3.0], [1.0], [1])
    assert e.value.code == -1
    with pytest.raises(vdb.VDBError) as e:
        _run(ctx, vdb, [1.0, 2.0], [2.0, 3.0], [1.0], [1], mbb=0)
    assert e.value.code == -1
    # minpts above INT_MAX: the reference stores it in an int, no point is core
    lab, _ = _run(ctx, vdb, [1.0, 2.0], [2.0, 3.0], [5.0], [2**31 + 5])
    np.testing.assert_array_equal(lab, [[0, 0]])


def test_device_resident_call_matches_host_call(ctx, vdb):
    torch = pytest.importorskip("torch")
    c = load("variant_sweep_4k")
    xt = torch.tensor(c["x"], dtype=torch.float64, device="cuda")
    yt = torch.tensor(c["y"], dtype=torch.float64, device="cuda")
    lab = torch.zeros(len(c["eps"]) * len(c["x"]), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.run_device(xt.data_ptr(), yt.data_ptr(), len(c["x"]), c["eps"], c["minpts"],
                   lab.data_ptr())
    got = lab.cpu().numpy().view(np.uint32).reshape(len(c["eps"]), -1)
    np.testing.assert_array_equal(got, c["labels"])


@pytest.mark.parametrize("cpe", [2, 1])
def test_row_chunked_tables_match_whole_tables(ctx, vdb, cpe):
    # a table budget far below 4E forces row chunks of whole tiles; with one
    # cell per eps the cells are not cliques and every chunk is built twice
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    a, sa = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, cells_per_eps=cpe)
    b, sb = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, cells_per_eps=cpe,
                 budget=16 << 20)
    assert sb["pairs"] == sa["pairs"]
    assert sb["table_chunks"] > sb["tables"] and sa["table_chunks"] == sa["tables"]
    np.testing.assert_array_equal(a, b)


def test_row_chunked_lattice_vs_oracle(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    d = syn.lattice_stress(n=100_000, seed=3)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, budget=8 << 20)
    assert st["table_chunks"] > st["tables"]
    np.testing.assert_array_equal(lab, orc.variants(d.x, d.y, d.eps, d.minpts))


def test_row_chunked_adversarial(ctx, vdb):
    chunked_runs = 0
    for i, c in enumerate(adversarial()):
        args = (c["x"], c["y"], [c["eps"]], [c["minpts"]], c["mbb"])
        _, whole = _run(ctx, vdb, *args)
        for budget in (whole["pairs"], 2 * whole["pairs"], 4 * whole["pairs"] - 4):
            try:
                lab, st = _run(ctx, vdb, *args, budget=max(budget, 4))
            except vdb.VDBError as e:
                assert e.code == -4  # the rows of one tile exceed the budget
                continue
            np.testing.assert_array_equal(lab[0], c["labels"], err_msg=f"case {i}")
            chunked_runs += st["table_chunks"] > st["tables"]
    assert chunked_runs > 0


def test_concurrent_streams_match_one_stream(ctx, vdb):
    from variantdbscan_gb300 import synthetic as syn
    dss = syn.multi_dataset(count=9, seed=7, n_lo=2000, n_hi=40000)
    items = [vdb.BatchItem(d.x, d.y, d.eps, d.minpts) for d in dss]
    one, s1 = ctx.run(items, streams=1)
    many, s4 = ctx.run(items, streams=4)
    assert s1["pairs"] == s4["pairs"] and s1["tables"] == s4["tables"]
    for a, b in zip(one, many):
        np.testing.assert_array_equal(a, b)


def test_concurrent_batch_reports_a_failing_dataset(ctx, vdb):
    good = load("variant_sweep_4k")
    bad_x = np.array(good["x"], dtype=np.float64)
    bad_x[5] = np.nan
    items = [vdb.BatchItem(good["x"], good["y"], good["eps"], good["minpts"]) for _ in range(3)]
    items.insert(1, vdb.BatchItem(bad_x, good["y"], good["eps"], good["minpts"]))
    with pytest.raises(vdb.VDBError) as e:
        ctx.run(items, streams=3)
    assert e.value.code == -1
    # the context stays usable
    outs, _ = ctx.run(items[:1] + items[2:], streams=3)
    for lab in outs:
        np.testing.assert_array_equal(lab, good["labels"])


@pytest.mark.slow
def test_lattice_full_size_mixed_equals_fp64(ctx, vdb):
    # 10,000,000 points on a 0.01 deg lattice: for eps 0.05 and 0.1 the FP32
    # filter with FP64 band re-tests gives the FP64 path's tables and labels,
    # and the all-variant batched call (row-chunked tables for the large eps)
    # gives the same labels for those variants
    torch = pytest.importorskip("torch")
    from variantdbscan_gb300 import synthetic as syn
    d = syn.lattice_stress(n=10_000_000, seed=3)
    xt = torch.from_numpy(d.x).cuda()
    yt = torch.from_numpy(d.y).cuda()
    sel = np.flatnonzero(d.eps <= 0.1)
    n, k = d.n, len(sel)
    la = torch.zeros(k * n, dtype=torch.int32, device="cuda")
    lb = torch.zeros(k * n, dtype=torch.int32, device="cuda")
    lall = torch.zeros(len(d.eps) * n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    sa = ctx.run_device(xt.data_ptr(), yt.data_ptr(), n, d.eps[sel], d.minpts[sel],
                        la.data_ptr(), precision="mixed", table_hash=True)
    sb = ctx.run_device(xt.data_ptr(), yt.data_ptr(), n, d.eps[sel], d.minpts[sel],
                        lb.data_ptr(), precision="fp64", table_hash=True)
    ctx.run_device(xt.data_ptr(), yt.data_ptr(), n, d.eps, d.minpts, lall.data_ptr())
    torch.cuda.synchronize()
    assert sa["pairs"] == sb["pairs"] and sa["retested"] > 0
    assert sa["table_hash"] == sb["table_hash"]  # the same neighbour sets, row by row
    assert torch.equal(la, lb)
    assert torch.equal(lall.view(len(d.eps), n)[torch.as_tensor(sel, device="cuda")],
                       la.view(k, n))


@pytest.mark.slow
def test_variant_sweep_full_size_mixed_equals_fp64(ctx, vdb):
    # 2,000,000-point sweep, eps 0.1 variants: batched mixed == plain FP64
    torch = pytest.importorskip("torch")
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=2_000_000, seed=1)
    sel = np.flatnonzero(d.eps == 0.1)
    xt = torch.from_numpy(d.x).cuda()
    yt = torch.from_numpy(d.y).cuda()
    n, k = d.n, len(sel)
    la = torch.zeros(k * n, dtype=torch.int32, device="cuda")
    lb = torch.zeros(k * n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    sa = ctx.run_device(xt.data_ptr(), yt.data_ptr(), n, d.eps[sel], d.minpts[sel],
                        la.data_ptr(), table_hash=True)
    sb = ctx.run_device(xt.data_ptr(), yt.data_ptr(), n, d.eps[sel], d.minpts[sel],
                        lb.data_ptr(), precision="fp64", schedule="plain", table_hash=True)
    torch.cuda.synchronize()
    assert sb["pairs"] == k * sa["pairs"]
    # the plain path builds the same table once per variant
    assert sb["table_hash"] == (k * sa["table_hash"]) % (1 << 64)
    assert torch.equal(la, lb)


@pytest.mark.parametrize("name", ["variant_sweep_4k", "lattice_4k", "single_variant_3k"])
@pytest.mark.parametrize("entry_bytes", [0, 2])
def test_border_rows_table_gives_the_same_labels(ctx, vdb, name, entry_bytes):
    # VDB_TABLE_BORDER writes only the rows of points that are not core for
    # the largest minpts of their epsilon; the labels must not change (32-bit
    # entries by default in this mode, 16-bit on request)
    c = load(name)
    lab, st = _run(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], int(c["mbb"]),
                   table="border", entry_bytes=entry_bytes)
    np.testing.assert_array_equal(lab, c["labels"])
    assert st["compact_tables"] == (st["tables"] if entry_bytes == 2 else 0)


def test_border_rows_table_large_and_chunked(ctx, vdb, orc):
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    want = orc.variants(d.x, d.y, d.eps, d.minpts)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, table="border")
    np.testing.assert_array_equal(lab, want)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, table="border", budget=1 << 20)
    np.testing.assert_array_equal(lab, want)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, table="border", budget=1 << 20,
                   entry_bytes=2)
    np.testing.assert_array_equal(lab, want)
    # with one cell per eps the cells are not cliques: every row is written
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, table="border", cells_per_eps=1)
    np.testing.assert_array_equal(lab, want)


def test_border_rows_table_adversarial(ctx, vdb):
    for i, c in enumerate(adversarial()):
        lab, _ = _run(ctx, vdb, c["x"], c["y"], [c["eps"]], [c["minpts"]], c["mbb"],
                      table="border")
        np.testing.assert_array_equal(lab[0], c["labels"], err_msg=f"case {i}")


@pytest.mark.parametrize("cpe", [1, 2])
def test_reuse_across_variants_gives_from_scratch_labels(ctx, vdb, orc, cpe):
    # reuse (default): a variant's union-find starts from the larger minpts
    # before it at the same eps, and cell pairs of different components at a
    # larger eps are not searched; with one cell per eps the chained unions go
    # edge by edge through the table
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    a, sa = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, cells_per_eps=cpe)
    b, sb = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, cells_per_eps=cpe, reuse=False)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, orc.variants(d.x, d.y, d.eps, d.minpts))
    assert sb["reuse_skipped_pairs"] == 0
    if cpe == 2:
        # close epsilons: cells near the edge of one cluster and of another
        # that the larger epsilon keeps apart are not searched at the smaller
        eps = np.array([0.40, 0.38, 0.36, 0.34, 0.32])
        mp = np.full(5, 12, np.uint32)
        a, sa = _run(ctx, vdb, d.x, d.y, eps, mp)
        b, sb = _run(ctx, vdb, d.x, d.y, eps, mp, reuse=False)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, orc.variants(d.x, d.y, eps, mp))
        assert sa["reuse_skipped_pairs"] > 0 and sb["reuse_skipped_pairs"] == 0


def test_reuse_with_minpts_that_do_not_nest(ctx, vdb, orc):
    # components are taken from an earlier (larger) eps with the largest
    # minpts not above the variant's; row chunks keep one state per minpts
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=2)
    eps = np.array([0.8, 0.4, 0.4, 0.2, 0.1, 0.1, 0.25, 0.8])
    mp = np.array([30, 8, 64, 16, 4, 100, 3, 30], np.uint32)
    want = orc.variants(d.x, d.y, eps, mp)
    for kw in ({}, {"budget": 4 << 20}, {"cells_per_eps": 1}, {"table": "border"}):
        lab, st = _run(ctx, vdb, d.x, d.y, eps, mp, **kw)
        np.testing.assert_array_equal(lab, want, err_msg=str(kw))


@pytest.mark.parametrize("G", [1, 2, 4, 8, 16])
def test_every_tile_shape_gives_the_same_tables_and_labels(ctx, vdb, orc, G):
    # the tile shapes the autotuner can pick: same neighbour tables (hash),
    # same labels as the oracle, on a dense sweep and on sparse small datasets
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, tile_cells=G, table_hash=True)
    ref, sr = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, tile_cells=1, table_hash=True)
    assert st["table_hash"] == sr["table_hash"] and st["pairs"] == sr["pairs"]
    assert st["tables_by_tile_cells"][G.bit_length() - 1] == st["tables"]
    np.testing.assert_array_equal(lab, orc.variants(d.x, d.y, d.eps, d.minpts))
    c = load("variant_sweep_4k")
    lab, _ = _run(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], tile_cells=G)
    np.testing.assert_array_equal(lab, c["labels"])
    for dd in syn.multi_dataset(count=3, seed=9, n_lo=10_000, n_hi=20_000):
        lab, _ = _run(ctx, vdb, dd.x, dd.y, dd.eps, dd.minpts, tile_cells=G, budget=1 << 20)
        np.testing.assert_array_equal(lab, orc.variants(dd.x, dd.y, dd.eps, dd.minpts))


@pytest.mark.parametrize("unit", [1024, 2048, 4096])
def test_every_work_unit_size_gives_the_same_tables_and_labels(ctx, vdb, orc, unit):
    # work units of 1024 / 2048 / 4096 candidates (the library takes 1024
    # below 2^18 points, else 4096): same tables, one-way pairs and labels, in
    # both entry formats, whole and row-chunked, and with border rows only
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    want = orc.variants(d.x, d.y, d.eps, d.minpts)
    ref = None
    for kw in ({}, {"entry_bytes": 4}, {"budget": 1 << 20}, {"tile_cells": 8}):
        lab, st = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, unit_candidates=unit,
                       table_hash=True, **kw)
        np.testing.assert_array_equal(lab, want, err_msg=str(kw))
        if ref is None:
            ref = st
        assert st["table_hash"] == ref["table_hash"], kw
        assert st["asymmetric_pairs"] == ref["asymmetric_pairs"], kw
    lab, _ = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, unit_candidates=unit, table="border")
    np.testing.assert_array_equal(lab, want)
    _, big = _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, unit_candidates=4096, table_hash=True)
    assert big["table_hash"] == ref["table_hash"] and big["pairs"] == ref["pairs"]
    c = adversarial()[0]
    lab, _ = _run(ctx, vdb, c["x"], c["y"], [c["eps"]], [c["minpts"]], c["mbb"],
                  unit_candidates=unit)
    np.testing.assert_array_equal(lab[0], c["labels"])
    with pytest.raises(vdb.VDBError):
        _run(ctx, vdb, d.x, d.y, d.eps, d.minpts, unit_candidates=1000)


def test_autotuner_widens_tiles_on_sparse_grids(ctx, vdb, orc):
    # 200,000 points spread over the globe with a small eps: cells hold less
    # than one point, so one-cell tiles would leave most query slots of a warp
    # empty; the tuner picks groups of several cells (kept for the repeated
    # call), the labels do not change, and a dense sweep keeps one-cell tiles
    # at eps 0.8
    rng = np.random.default_rng(21)
    x = rng.uniform(0, 360, 200_000)
    y = rng.uniform(-90, 90, 200_000)
    eps, mp = [0.5, 0.2], [3, 2]
    lab, st = _run(ctx, vdb, x, y, eps, mp)
    assert st["tables_by_tile_cells"][0] == 0, st["tables_by_tile_cells"]
    np.testing.assert_array_equal(lab, orc.variants(x, y, eps, mp))
    assert st["worker_streams"] == 1
    lab2, st2 = _run(ctx, vdb, x, y, eps, mp)
    assert st2["tables_by_tile_cells"] == st["tables_by_tile_cells"]
    np.testing.assert_array_equal(lab2, lab)
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=400_000, seed=1)
    _, sd = _run(ctx, vdb, d.x, d.y, [0.8], [16])
    assert sd["tables_by_tile_cells"][0] == 1, sd["tables_by_tile_cells"]


def test_worker_streams_follow_the_work_split(ctx, vdb):
    from variantdbscan_gb300 import synthetic as syn
    dss = syn.multi_dataset(count=8, seed=4, n_lo=10_000, n_hi=12_000)
    items = [vdb.BatchItem(d.x, d.y, d.eps, d.minpts) for d in dss]
    _, st = ctx.run(items)
    assert st["worker_streams"] == 4   # eight datasets of similar work
    big = syn.variant_sweep(n=200_000, seed=1)
    items2 = [vdb.BatchItem(big.x, big.y, big.eps, big.minpts)] + items[:2]
    _, st2 = ctx.run(items2)
    assert st2["worker_streams"] == 1  # one dataset holds most of the work
    _, st3 = ctx.run(items, streams=2)
    assert st3["worker_streams"] == 2
