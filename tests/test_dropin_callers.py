"""The reference's own callers of libVDBSCAN, unmodified, against the GB300
library.

* src/c_test_prog.cpp: the reference's C test program (dlopen check at :51,
  call at :141), compiled from a staged, unmodified copy and linked against
  variantdbscan_gb300/lib/libSharedVDBSCAN.so; its printed labels must equal
  src/test_output.csv.
* python_package/vdbscan/variantdbscan.py: the reference's Python wrapper,
  an unmodified copy in a package directory whose lib/ holds the GB300 library
  (placed by variantdbscan_gb300.install); it must return the reference's
  labels.

The staged copies come from oracle/build_ref.sh (oracle/_ref/callers/); the
tests skip when they are absent.
"""
import importlib.util
import os
import shutil
import subprocess

import numpy as np
import pytest

from golden_cases import CASES, load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CALLERS = os.path.join(ROOT, "oracle", "_ref", "callers")
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")

needs_callers = pytest.mark.skipif(
    not os.path.exists(os.path.join(CALLERS, "c_test_prog.cpp")),
    reason="staged reference callers missing (oracle/build_ref.sh with VDB_REFERENCE_DIR)")


def _build_c_test_prog(tmp_path):
    from variantdbscan_gb300 import build
    lib = build.build()
    exe = tmp_path / "c_test_prog"
    r = subprocess.run(["g++", "-O2", "-w", "-I", REF_SRC, os.path.join(CALLERS, "c_test_prog.cpp"),
                        "-L", os.path.dirname(lib), "-lSharedVDBSCAN", "-ldl", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, os.path.dirname(lib)


@needs_callers
def test_c_test_prog_builds_unmodified(tmp_path):
    # compile and link only (no GPU needed): the reference's prototype
    # (src/c_test_prog.h:26) resolves against the GB300 library
    exe, _ = _build_c_test_prog(tmp_path)
    assert exe.exists()


@needs_callers
def test_wrapper_package_layout(tmp_path):
    # the reference wrapper loads lib/libSharedVDBSCAN.so beside its own file
    from variantdbscan_gb300 import install
    fake = tmp_path / "fake.so"
    fake.write_bytes(b"\x7fELF")
    pkg = tmp_path / "vdbscan"
    pkg.mkdir()
    dst = install.place_library(str(pkg), str(fake))
    assert dst == str(pkg / "lib" / "libSharedVDBSCAN.so")
    assert open(dst, "rb").read() == b"\x7fELF"


@pytest.mark.gpu
@needs_callers
def test_reference_c_test_prog_unmodified(tmp_path):
    exe, libdir = _build_c_test_prog(tmp_path)
    run_dir = tmp_path / "run"
    run_dir.mkdir()
    shutil.copy(os.path.join(CALLERS, "test_dataset.csv"), run_dir / "test_dataset.csv")
    env = dict(os.environ, LD_LIBRARY_PATH=libdir + ":" + os.environ.get("LD_LIBRARY_PATH", ""))
    r = subprocess.run([str(exe)], cwd=run_dir, capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    # "\n%d, %f, %f, %d" per point and variant after each "Variant:" header
    # (src/c_test_prog.cpp:145-153)
    labels, cur = [], None
    for line in r.stdout.splitlines():
        if line.startswith("Variant:"):
            cur = []
            labels.append(cur)
            continue
        parts = [p.strip() for p in line.split(",")]
        if cur is not None and len(parts) == 4:
            cur.append(int(parts[3]))
    want = np.loadtxt(os.path.join(CALLERS, "test_output.csv"), delimiter=",")
    assert len(labels) == 2 and len(labels[0]) == len(want)
    np.testing.assert_array_equal(np.array(labels[0]), want[:, 2].astype(int))
    np.testing.assert_array_equal(np.array(labels[1]), want[:, 3].astype(int))


@pytest.mark.gpu
@needs_callers
def test_reference_python_wrapper_unmodified(tmp_path):
    from variantdbscan_gb300 import build, install
    lib = build.build()
    pkg = tmp_path / "vdbscan"
    pkg.mkdir()
    shutil.copy(os.path.join(CALLERS, "variantdbscan.py"), pkg / "variantdbscan.py")
    install.place_library(str(pkg), lib)
    spec = importlib.util.spec_from_file_location("ref_variantdbscan", pkg / "variantdbscan.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    for name in CASES:
        c = load(name)
        res = mod.VariantDBSCAN(c["eps"], c["minpts"], c["x"], c["y"], mbbsize=int(c["mbb"]))
        want = c["labels"].T if len(c["eps"]) > 1 else c["labels"][0]
        np.testing.assert_array_equal(res, want, err_msg=name)
