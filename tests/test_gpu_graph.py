"""Graph replay (vdb_options.graph): the first call of a shape runs directly
and captures its graph, later calls replay it.  Replayed labels, neighbour
tables and statistics must equal the direct call's; data that no longer
match the record fall back to the direct path with the same labels."""
import numpy as np
import pytest

from golden_cases import CASES, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vdb():
    import variantdbscan_gb300 as v
    from variantdbscan_gb300 import build
    build.build()
    return v


@pytest.fixture()
def ctx(vdb):
    c = vdb.Context()
    yield c
    c.close()


def _blobs(n, seed, centres=12, spread=0.35, box=20.0):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0, box, (centres, 2))
    k = rng.integers(0, centres, n)
    p = c[k] + rng.normal(0, spread, (n, 2))
    noise = rng.uniform(0, box, (n // 10, 2))
    p = np.vstack([p, noise])
    return np.ascontiguousarray(p[:, 0]), np.ascontiguousarray(p[:, 1])


EPS = [0.3, 0.15, 0.15, 0.08]
MP = [8, 4, 16, 3]


def _direct(ctx, vdb, x, y, eps=EPS, mp=MP, mbb=70, **kw):
    out, st = ctx.run([vdb.BatchItem(x, y, eps, mp, mbb)], table_hash=True, **kw)
    return out[0], st


def test_replay_equals_direct(ctx, vdb):
    x, y = _blobs(60_000, 1)
    ref, st0 = _direct(ctx, vdb, x, y)
    states = []
    for _ in range(4):
        lab, st = _direct(ctx, vdb, x, y, graph=True)
        np.testing.assert_array_equal(lab, ref)
        assert st["table_hash"] == st0["table_hash"]
        assert st["pairs"] == st0["pairs"]
        assert st["clusters"] == st0["clusters"]
        states.append(st["graph"])
        assert st["graph_checks"] > 0
    assert states == [vdb.GRAPH_CAPTURED] + [vdb.GRAPH_REPLAYED] * 3


@pytest.mark.parametrize("kw", [dict(precision="fp64"), dict(schedule="plain"),
                                dict(entry_bytes=4), dict(table="border"),
                                dict(reuse=False), dict(tile_cells=4)])
def test_replay_equals_direct_across_options(ctx, vdb, kw):
    x, y = _blobs(30_000, 2)
    ref, st0 = _direct(ctx, vdb, x, y, **kw)
    for want in (vdb.GRAPH_CAPTURED, vdb.GRAPH_REPLAYED, vdb.GRAPH_REPLAYED):
        lab, st = _direct(ctx, vdb, x, y, graph=True, **kw)
        np.testing.assert_array_equal(lab, ref)
        assert st["graph"] == want
        assert st["pairs"] == st0["pairs"]
        if kw.get("table") != "border":
            assert st["table_hash"] == st0["table_hash"]


@pytest.mark.parametrize("name", CASES)
def test_replay_of_reference_fixtures(ctx, vdb, name):
    c = load(name)
    args = (c["x"], c["y"], c["eps"], c["minpts"], int(c["mbb"]))
    for _ in range(3):
        out, st = ctx.run([vdb.BatchItem(*args)], graph=True)
        np.testing.assert_array_equal(out[0], c["labels"], err_msg=name)
        assert st["graph"] in (vdb.GRAPH_CAPTURED, vdb.GRAPH_REPLAYED, vdb.GRAPH_UNSUPPORTED)


def test_other_data_falls_back_and_is_recaptured(ctx, vdb):
    x, y = _blobs(40_000, 3)
    x2, y2 = _blobs(40_000, 4)
    x2 = x2 + 25.0  # same size, points outside the recorded box
    ref2, _ = _direct(ctx, vdb, x2, y2)
    assert _direct(ctx, vdb, x, y, graph=True)[1]["graph"] == vdb.GRAPH_CAPTURED
    assert _direct(ctx, vdb, x, y, graph=True)[1]["graph"] == vdb.GRAPH_REPLAYED
    lab, st = _direct(ctx, vdb, x2, y2, graph=True)
    assert st["graph"] == vdb.GRAPH_FALLBACK
    np.testing.assert_array_equal(lab, ref2)
    lab, st = _direct(ctx, vdb, x2, y2, graph=True)
    assert st["graph"] == vdb.GRAPH_CAPTURED
    np.testing.assert_array_equal(lab, ref2)
    lab, st = _direct(ctx, vdb, x2, y2, graph=True)
    assert st["graph"] == vdb.GRAPH_REPLAYED
    np.testing.assert_array_equal(lab, ref2)


def test_same_box_other_points(ctx, vdb):
    # the extremes stay, interior points move: the replay either passes its
    # checkpoints (sizes within the record) or falls back; labels are the
    # direct call's either way
    x, y = _blobs(50_000, 5)
    _direct(ctx, vdb, x, y, graph=True)
    rng = np.random.default_rng(6)
    keep = {int(np.argmin(x)), int(np.argmax(x)), int(np.argmin(y)), int(np.argmax(y))}
    seen = set()
    for trial, frac in enumerate([0.0, 0.001, 0.05, 0.3]):
        x2, y2 = x.copy(), y.copy()
        m = int(frac * len(x))
        idx = np.array([i for i in rng.choice(len(x), m + 8, replace=False) if i not in keep][:m],
                       dtype=np.int64)
        if len(idx):
            x2[idx] = rng.uniform(x.min(), x.max(), len(idx))
            y2[idx] = rng.uniform(y.min(), y.max(), len(idx))
        ref, st0 = _direct(ctx, vdb, x2, y2)
        lab, st = _direct(ctx, vdb, x2, y2, graph=True)
        np.testing.assert_array_equal(lab, ref, err_msg=f"trial {trial}")
        seen.add(st["graph"])
        if st["graph"] == vdb.GRAPH_REPLAYED:
            assert st["table_hash"] == st0["table_hash"]
    assert vdb.GRAPH_REPLAYED in seen


def test_points_inside_the_recorded_box_replay(ctx, vdb):
    # the graph serves other data of the same size inside the recorded box
    # (grid and error bounds are the record's, conservative for them) while
    # their sizes fit the buffers' headroom
    x, y = _blobs(50_000, 9)
    assert _direct(ctx, vdb, x, y, graph=True)[1]["graph"] == vdb.GRAPH_CAPTURED
    rng = np.random.default_rng(10)
    perm = rng.permutation(len(x))
    lo_x, hi_x, lo_y, hi_y = x.min(), x.max(), y.min(), y.max()
    jx = np.clip(x + rng.normal(0, 0.01, len(x)), lo_x, hi_x)
    jy = np.clip(y + rng.normal(0, 0.01, len(y)), lo_y, hi_y)
    shrink_x = lo_x + (x - lo_x) * 0.97
    for tag, (a, b) in {"permuted": (x[perm], y[perm]), "jittered": (jx, jy),
                        "shrunk": (shrink_x, y)}.items():
        a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
        ref, st0 = _direct(ctx, vdb, a, b)
        lab, st = _direct(ctx, vdb, a, b, graph=True)
        np.testing.assert_array_equal(lab, ref, err_msg=tag)
        assert st["graph"] == vdb.GRAPH_REPLAYED, tag
        assert st["table_hash"] == st0["table_hash"], tag
        assert st["pairs"] == st0["pairs"], tag


def test_multi_dataset_batch_graph(ctx, vdb):
    items = []
    for i, n in enumerate([20_000, 45_000, 5_000, 30_000, 1_000, 12_000]):
        x, y = _blobs(n, 10 + i, centres=4 + i)
        items.append(vdb.BatchItem(x, y, EPS[: 1 + i % 4], MP[: 1 + i % 4], 70))
    ref, st0 = ctx.run(items, table_hash=True)
    for want in (vdb.GRAPH_CAPTURED, vdb.GRAPH_REPLAYED, vdb.GRAPH_REPLAYED):
        out, st = ctx.run(items, table_hash=True, graph=True)
        assert st["graph"] == want
        assert st["table_hash"] == st0["table_hash"]
        for a, b in zip(out, ref):
            np.testing.assert_array_equal(a, b)


def test_device_buffers_replay(ctx, vdb):
    torch = pytest.importorskip("torch")
    x, y = _blobs(40_000, 7)
    ref, _ = _direct(ctx, vdb, x, y)
    dx = torch.tensor(x, device="cuda")
    dy = torch.tensor(y, device="cuda")
    lab = torch.zeros((len(EPS), len(x)), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for want in (vdb.GRAPH_CAPTURED, vdb.GRAPH_REPLAYED, vdb.GRAPH_REPLAYED):
        lab.zero_()
        torch.cuda.synchronize()
        st = ctx.run_device(dx.data_ptr(), dy.data_ptr(), len(x), EPS, MP, lab.data_ptr(),
                            graph=True)
        assert st["graph"] == want
        np.testing.assert_array_equal(lab.cpu().numpy().view(np.uint32), ref)


def test_page_locked_host_buffers_replay(ctx, vdb):
    # page-locked inputs and labels are copied straight by the replay;
    # pageable ones go through the graph's pinned buffers
    torch = pytest.importorskip("torch")
    x, y = _blobs(30_000, 11)
    ref, _ = _direct(ctx, vdb, x, y)
    px = torch.from_numpy(x).pin_memory().numpy()
    py = torch.from_numpy(y).pin_memory().numpy()
    plab = torch.zeros((len(EPS), len(x)), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    for want in (vdb.GRAPH_CAPTURED, vdb.GRAPH_REPLAYED, vdb.GRAPH_REPLAYED):
        plab[...] = 0
        out, st = ctx.run([vdb.BatchItem(px, py, EPS, MP, 70, labels=plab)], graph=True)
        assert st["graph"] == want
        np.testing.assert_array_equal(plab, ref)
    # the same call shape with pageable labels, then pageable inputs
    lab = np.zeros_like(plab)
    out, st = ctx.run([vdb.BatchItem(px, py, EPS, MP, 70, labels=lab)], graph=True)
    assert st["graph"] == vdb.GRAPH_REPLAYED
    np.testing.assert_array_equal(lab, ref)
    out, st = ctx.run([vdb.BatchItem(x.copy(), y.copy(), EPS, MP, 70, labels=plab)], graph=True)
    assert st["graph"] == vdb.GRAPH_REPLAYED
    np.testing.assert_array_equal(plab, ref)


def test_table_budget_that_fits_is_captured(ctx, vdb):
    # a table budget above the recorded table: captured, the headroom kept
    # within the budget
    x, y = _blobs(30_000, 12)
    ref, st0 = _direct(ctx, vdb, x, y)
    budget = st0["table_bytes"] + 4096
    ref_b, _ = _direct(ctx, vdb, x, y, budget=budget)
    np.testing.assert_array_equal(ref_b, ref)
    for want in (vdb.GRAPH_CAPTURED, vdb.GRAPH_REPLAYED):
        lab, st = _direct(ctx, vdb, x, y, budget=budget, graph=True)
        assert st["graph"] == want
        np.testing.assert_array_equal(lab, ref)


def test_paths_not_captured_run_directly(ctx, vdb):
    x, y = _blobs(20_000, 8)
    eps, mp = [0.2, -1.0], [5, 5]
    ref, _ = _direct(ctx, vdb, x, y, eps, mp)
    for _ in range(2):
        lab, st = _direct(ctx, vdb, x, y, eps, mp, graph=True)
        assert st["graph"] == vdb.GRAPH_UNSUPPORTED
        np.testing.assert_array_equal(lab, ref)
    # a table budget that forces row chunks
    ref, _ = _direct(ctx, vdb, x, y, budget=1 << 16)
    lab, st = _direct(ctx, vdb, x, y, graph=True, budget=1 << 16)
    assert st["graph"] == vdb.GRAPH_UNSUPPORTED
    np.testing.assert_array_equal(lab, ref)


def test_graph_cache_keeps_four_shapes(ctx, vdb):
    data = [_blobs(8_000 + 1000 * i, 20 + i) for i in range(6)]
    refs = [_direct(ctx, vdb, x, y)[0] for x, y in data]
    for (x, y), r in zip(data, refs):
        lab, st = _direct(ctx, vdb, x, y, graph=True)
        assert st["graph"] == vdb.GRAPH_CAPTURED
        np.testing.assert_array_equal(lab, r)
    # the last four shapes are kept, the first two were evicted
    for i in [2, 3, 4, 5, 0]:
        x, y = data[i]
        lab, st = _direct(ctx, vdb, x, y, graph=True)
        np.testing.assert_array_equal(lab, refs[i])
        assert st["graph"] == (vdb.GRAPH_REPLAYED if i >= 2 else vdb.GRAPH_CAPTURED)
