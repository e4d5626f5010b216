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


def test_noalloc_rejects_sizes_beyond_the_limit(lib):
    # rejected before any device work: the pointers are never dereferenced
    dummy = ctypes.c_void_p(16)
    rc = lib.vdb_run_noalloc(dummy, dummy, MAX_POINTS + 1, 0.5, 10, 70, dummy, None)
    assert rc == VDB_ERR_TOO_LARGE
