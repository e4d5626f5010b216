"""The neighbour tables themselves, not only the labels they lead to, against
the restated oracle: with table_hash set, the library reports the sum over
every table, row p and entry q of a 64-bit mix of (p, q), one-way entries
marked; the oracle computes the same sum from its own neighbour relation.
Equal sums mean equal neighbour sets for every point (up to 64-bit hash
collisions), whatever the precision, grid resolution or row chunking."""
import numpy as np
import pytest

from golden_cases import CASES, adversarial, load

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


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


def _stats(ctx, vdb, x, y, eps, mp, mbb=70, **kw):
    _, st = ctx.run([vdb.BatchItem(x, y, eps, mp, mbb)], table_hash=True, **kw)
    return st


def _oracle_hash(orc, x, y, eps_list, mbb=70):
    return sum(orc.table_hash(x, y, e, mbb) for e in eps_list) & M64


@pytest.mark.parametrize("name", [c for c in CASES if c != "vtest"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("entry_bytes", [0, 4])
def test_golden_tables(ctx, vdb, orc, name, precision, entry_bytes):
    # batched: one table per distinct epsilon; 16-bit entries (the default
    # where they fit) and 32-bit entries
    c = load(name)
    mbb = int(c["mbb"])
    st = _stats(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], mbb, precision=precision,
                entry_bytes=entry_bytes)
    assert st["table_hash"] == _oracle_hash(orc, c["x"], c["y"], np.unique(c["eps"]), mbb)
    if entry_bytes == 4:
        assert st["compact_tables"] == 0


def test_plain_schedule_builds_one_table_per_variant(ctx, vdb, orc):
    c = load("variant_sweep_4k")
    st = _stats(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], schedule="plain",
                precision="fp64")
    assert st["tables"] == len(c["eps"])
    assert st["table_hash"] == _oracle_hash(orc, c["x"], c["y"], c["eps"])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("entry_bytes", [0, 4])
def test_one_way_entries(ctx, vdb, orc, precision, entry_bytes):
    for i, c in enumerate(adversarial()):
        st = _stats(ctx, vdb, c["x"], c["y"], [c["eps"]], [c["minpts"]], c["mbb"],
                    precision=precision, entry_bytes=entry_bytes)
        want = orc.table_hash(c["x"], c["y"], c["eps"], c["mbb"])
        assert st["table_hash"] == want, f"case {i}"


@pytest.mark.parametrize("cpe", [1, 2, 3])
def test_lattice_medium_tables(ctx, vdb, orc, cpe):
    # many pairs at exactly eps: FP32 band re-tests decide them
    from variantdbscan_gb300 import synthetic as syn
    d = syn.lattice_stress(n=100_000, seed=3)
    st = _stats(ctx, vdb, d.x, d.y, d.eps, d.minpts, cells_per_eps=cpe)
    assert st["retested"] > 0 and st["compact_tables"] == st["tables"]
    assert st["table_hash"] == _oracle_hash(orc, d.x, d.y, np.unique(d.eps))


def test_sweep_medium_tables_whole_and_row_chunked(ctx, vdb, orc):
    # the table pass's multi-round units, carried segment ends and row chunks
    from variantdbscan_gb300 import synthetic as syn
    d = syn.variant_sweep(n=60_000, seed=1)
    want = _oracle_hash(orc, d.x, d.y, np.unique(d.eps))
    whole = _stats(ctx, vdb, d.x, d.y, d.eps, d.minpts)
    chunked = _stats(ctx, vdb, d.x, d.y, d.eps, d.minpts, budget=16 << 20)
    wide = _stats(ctx, vdb, d.x, d.y, d.eps, d.minpts, budget=16 << 20, entry_bytes=4)
    assert chunked["table_chunks"] > chunked["tables"]
    assert whole["compact_tables"] == whole["tables"] and wide["compact_tables"] == 0
    assert whole["entry_bytes"] == 2 * whole["pairs"] and wide["entry_bytes"] == 4 * wide["pairs"]
    assert whole["table_hash"] == want
    assert chunked["table_hash"] == want
    assert wide["table_hash"] == want


@pytest.mark.parametrize("entry_bytes", [0, 4])
def test_dense_tiles_with_many_units(ctx, vdb, orc, entry_bytes):
    # 34,000 points in one small blob: with eps 0.1 every tile has all of
    # them as candidates (9 work units per row), with eps 0.005 about 2,000
    rng = np.random.default_rng(7)
    x = 10.0 + rng.random(34_000) * 0.05
    y = 20.0 + rng.random(34_000) * 0.05
    st = _stats(ctx, vdb, x, y, [0.1, 0.005], [50, 10], entry_bytes=entry_bytes)
    assert st["tables"] == 2
    assert st["compact_tables"] == (2 if entry_bytes == 0 else 0)
    assert st["table_hash"] == _oracle_hash(orc, x, y, [0.1, 0.005])


def test_border_rows_mode_reports_no_hash(ctx, vdb):
    # tables that hold only the border rows are not hashed
    c = load("variant_sweep_4k")
    st = _stats(ctx, vdb, c["x"], c["y"], c["eps"], c["minpts"], table="border")
    assert st["table_hash"] == 0
