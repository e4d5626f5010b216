"""The allocation-free entry point vdb_run_noalloc, called through the C ABI.

It serves callers that may not allocate device memory during a call (all
device memory reserved up front, a framework's own allocator owning the heap,
or no room for the device-wide synchronisation of cudaMalloc/cudaFree): every
temporary lives in one fixed array inside the library.  Its labels must equal
those of the batched entry point vdb_run_batch exactly (labels are integers),
on consecutive calls that reuse the array left behind by the previous one.
This file is collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_POINTS = 65536
VDB_ERR_TOO_LARGE = -7
VDB_ERR_INVALID_ARG = -1


@pytest.fixture(scope="module")
def lib():
    import variantdbscan_gb300 as v
    from variantdbscan_gb300 import build
    build.build()
    lib = v.load_library()
    lib.vdb_run_noalloc.restype = ctypes.c_int
    lib.vdb_run_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                    ctypes.c_double, ctypes.c_uint32, ctypes.c_int32,
                                    ctypes.c_void_p, ctypes.c_void_p]
    return lib


def _batched(x, y, eps, minpts, mbb):
    import variantdbscan_gb300 as v
    ctx = v.Context()
    out, _ = ctx.run([v.BatchItem(x, y, [eps], [minpts], mbb)])
    ctx.close()
    return out[0][0]


def _noalloc(lib, torch, x, y, eps, minpts, mbb):
    xt = torch.tensor(x, dtype=torch.float64, device="cuda")
    yt = torch.tensor(y, dtype=torch.float64, device="cuda")
    lab = torch.full((len(x),), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.vdb_run_noalloc(xt.data_ptr(), yt.data_ptr(), len(x), float(eps), int(minpts),
                             int(mbb), lab.data_ptr(), None)
    assert rc == 0, rc
    return lab.cpu().numpy().view(np.uint32)


def test_noalloc_matches_batched_on_consecutive_calls(lib):
    torch = pytest.importorskip("torch")
    from variantdbscan_gb300 import synthetic as syn
    a = syn.single_variant(n=20_000, seed=0)
    b = syn.lattice_stress(n=12_000, seed=5)
    cases = [(a.x, a.y, 0.5, 10, 70), (b.x, b.y, 2.0, 4, 3), (a.x, a.y, 0.5, 10, 70)]
    for i, (x, y, eps, mp, mbb) in enumerate(cases):
        want = _batched(x, y, eps, mp, mbb)
        got = _noalloc(lib, torch, x, y, eps, mp, mbb)
        np.testing.assert_array_equal(got, want, err_msg=f"call {i}")
        assert want.max() > 0


def test_noalloc_matches_the_reference_fixtures(lib):
    # labels computed by the reference library itself: the golden cases one
    # variant at a time, and the cases whose pairs are accepted in one
    # direction only (MBBsize 1 to 3 on lattices)
    torch = pytest.importorskip("torch")
    from golden_cases import CASES, adversarial, load
    for name in CASES:
        c = load(name)
        for v in range(len(c["eps"])):
            eps = float(c["eps"][v])
            if not (0.0 <= eps < np.inf):
                # the entry point takes finite epsilons >= 0 only
                dummy = ctypes.c_void_p(16)
                rc = lib.vdb_run_noalloc(dummy, dummy, len(c["x"]), eps, int(c["minpts"][v]),
                                         int(c["mbb"]), dummy, None)
                assert rc == VDB_ERR_INVALID_ARG
                continue
            got = _noalloc(lib, torch, c["x"], c["y"], eps, c["minpts"][v], int(c["mbb"]))
            np.testing.assert_array_equal(got, c["labels"][v], err_msg=f"{name} v{v}")
    for i, c in enumerate(adversarial()):
        got = _noalloc(lib, torch, c["x"], c["y"], c["eps"], c["minpts"], c["mbb"])
        np.testing.assert_array_equal(got, c["labels"], err_msg=f"one-way case {i}")


def test_noalloc_coarse_grid_matches_the_oracle(lib, orc):
    # a small epsilon over the whole globe needs more cells than the array
    # holds: the grid is coarsened until it fits, its cells are no longer
    # cliques, and the labelling unites cores edge by edge from the table
    torch = pytest.importorskip("torch")
    from variantdbscan_gb300 import synthetic as syn
    d = syn.single_variant(n=20_000, seed=3)
    got = _noalloc(lib, torch, d.x, d.y, 0.3, 5, 70)
    want = orc.dbscan(d.x, d.y, 0.3, 5, 70)
    assert want.max() > 0
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got, _batched(d.x, d.y, 0.3, 5, 70))


def test_noalloc_table_beyond_the_array_then_a_normal_call(lib):
    # the largest n with an epsilon that makes the neighbour table far larger
    # than the array: the call refuses with VDB_ERR_TOO_LARGE after counting,
    # and the next call (which reuses the array) is still exact
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    x = rng.uniform(0.0, 10.0, MAX_POINTS)
    y = rng.uniform(0.0, 10.0, MAX_POINTS)
    xt = torch.tensor(x, dtype=torch.float64, device="cuda")
    yt = torch.tensor(y, dtype=torch.float64, device="cuda")
    lab = torch.zeros(MAX_POINTS, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.vdb_run_noalloc(xt.data_ptr(), yt.data_ptr(), MAX_POINTS, 5.0, 4, 70,
                             lab.data_ptr(), None)
    assert rc == VDB_ERR_TOO_LARGE
    got = _noalloc(lib, torch, x, y, 0.05, 4, 70)
    np.testing.assert_array_equal(got, _batched(x, y, 0.05, 4, 70))


def test_noalloc_on_a_caller_stream(lib):
    # the caller's stream: the call orders its work after what is queued there
    # and returns once that stream has finished
    torch = pytest.importorskip("torch")
    from variantdbscan_gb300 import synthetic as syn
    d = syn.single_variant(n=30_000, seed=4)
    want = _batched(d.x, d.y, 0.5, 10, 70)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        xt = torch.tensor(d.x, dtype=torch.float64, device="cuda")
        yt = torch.tensor(d.y, dtype=torch.float64, device="cuda")
        lab = torch.full((d.n,), -1, dtype=torch.int32, device="cuda")
    rc = lib.vdb_run_noalloc(xt.data_ptr(), yt.data_ptr(), d.n, 0.5, 10, 70, lab.data_ptr(),
                             ctypes.c_void_p(s.cuda_stream))
    assert rc == 0, rc
    np.testing.assert_array_equal(lab.cpu().numpy().view(np.uint32), want)


def test_noalloc_rejects_sizes_beyond_the_limit(lib):
    # rejected before any device work: the pointers are never dereferenced
    dummy = ctypes.c_void_p(16)
    rc = lib.vdb_run_noalloc(dummy, dummy, MAX_POINTS + 1, 0.5, 10, 70, dummy, None)
    assert rc == VDB_ERR_TOO_LARGE
