"""File ingest of the reference's GPU prototype (src/gpu/import_dataset.cpp):
vdb_import_dataset and vdb_import_variants, host code behind the C ABI,
checked against a numpy restatement of the same FP64 operations."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def vdb():
    import variantdbscan_gb300 as v
    from variantdbscan_gb300 import build
    build.build()
    v.load_library()
    return v


def _map_lat(lat):
    # src/gpu/import_dataset.cpp:84-98, operation by operation in FP64
    lat = np.asarray(lat, np.float64)
    pos = ((90.0 - lat) / 90.0) * 90.0
    neg = ((-lat) / 90.0) * 90.0 + 90.0
    return np.where(lat > 0.0, pos, neg)


def test_dataset_file(vdb, tmp_path):
    rng = np.random.default_rng(5)
    lon = rng.uniform(0, 360, 500)
    lat = rng.uniform(-90, 90, 500)
    lat[:4] = [0.0, 90.0, -90.0, 1e-300]
    tec = rng.uniform(0, 80, 500)
    p = tmp_path / "data.csv"
    with open(p, "w") as f:
        for i, (a, b, c) in enumerate(zip(lon, lat, tec)):
            f.write(f"{float(a)!r},{float(b)!r},{float(c)!r}\n")
            if i == 10:
                f.write("\n")  # blank lines are skipped
        f.write(f"{float(lon[0])!r},{float(lat[0])!r}")  # two fields, no newline at the end
    x, y = vdb.import_dataset(str(p))
    want_x = np.concatenate([_map_lat(lat), _map_lat(lat[:1])])
    want_y = np.concatenate([lon, lon[:1]])
    np.testing.assert_array_equal(x, want_x)
    np.testing.assert_array_equal(y, want_y)
    assert x.min() >= 0.0 and x.max() <= 180.0


def test_dataset_file_errors(vdb, tmp_path):
    p = tmp_path / "bad.csv"
    p.write_text("1.0,2.0\n3.0\n")
    with pytest.raises(vdb.VDBError) as e:
        vdb.import_dataset(str(p))
    assert e.value.code == -1
    with pytest.raises(vdb.VDBError):
        vdb.import_dataset(str(tmp_path / "missing.csv"))


def test_variant_file_sorted_like_the_prototype(vdb, tmp_path):
    p = tmp_path / "variants.csv"
    p.write_text("0.5,10\n1.0,4\n0.5,3\n\n2.0,7\n1.0,12\nnan,5\n0.25,0\n")
    eps, mp = vdb.import_variants(str(p))
    # epsilon descending, minpts ascending within an epsilon, NaN last
    np.testing.assert_array_equal(eps[:-1], [2.0, 1.0, 1.0, 0.5, 0.5, 0.25])
    assert np.isnan(eps[-1])
    np.testing.assert_array_equal(mp, [7, 4, 12, 3, 10, 0, 5])
    p.write_text("0.5,-3\n")
    with pytest.raises(vdb.VDBError):
        vdb.import_variants(str(p))


def test_counts_and_capacity(vdb, tmp_path):
    import ctypes
    p = tmp_path / "d.csv"
    p.write_text("1,2\n3,4\n5,6\n")
    lib = vdb.load_library()
    n = ctypes.c_uint32(0)
    assert lib.vdb_import_dataset(os.fsencode(str(p)), None, None, 0, ctypes.byref(n)) == 0
    assert n.value == 3
    x = np.zeros(2)
    y = np.zeros(2)
    rc = lib.vdb_import_dataset(os.fsencode(str(p)), x.ctypes.data, y.ctypes.data, 2,
                                ctypes.byref(n))
    assert rc == -5 and n.value == 3
    np.testing.assert_array_equal(y, [1.0, 3.0])


@pytest.mark.gpu
def test_command_line_matches_the_library(vdb, tmp_path):
    from golden_cases import load
    c = load("variant_sweep_4k")
    # a dataset file whose mapped coordinates are the fixture's: lat such that
    # the mapping returns x (lat = 90 - x for x < 90 is not exact in general,
    # so compare against the library on the imported coordinates instead)
    d = tmp_path / "d.csv"
    with open(d, "w") as f:
        for a, b in zip(c["x"], c["y"]):
            f.write(f"{float(a)!r},{float(b) - 90.0!r},1.0\n")
    vf = tmp_path / "v.csv"
    vf.write_text("".join(f"{float(e)!r},{int(m)}\n" for e, m in zip(c["eps"], c["minpts"])))
    out = tmp_path / "labels.csv"
    r = subprocess.run([sys.executable, "-m", "variantdbscan_gb300.cli", str(d), str(vf),
                        "--out", str(out)], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.loadtxt(out, delimiter=",", comments="#")
    x, y = vdb.import_dataset(str(d))
    eps, mp = vdb.import_variants(str(vf))
    want = vdb.VariantDBSCAN(eps, mp, x, y)
    np.testing.assert_array_equal(got[:, 0], x)
    np.testing.assert_array_equal(got[:, 1], y)
    np.testing.assert_array_equal(got[:, 2:].astype(np.uint32), want)
