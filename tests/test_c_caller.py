"""A C program calls libVDBSCAN through include/vdbscan.h and the shared
library, the way the reference's C callers do (link against
libSharedVDBSCAN.so, host arrays in, retArr[v*n + i] out), and gets the labels
of the reference's own fixture."""
import os
import subprocess

import numpy as np
import pytest

from golden_cases import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_SRC = r"""
#include <stdio.h>
#include <stdlib.h>
#include "vdbscan.h"

int main(int argc, char **argv) {
    FILE *f = fopen(argv[1], "rb");
    unsigned int n, nv;
    if (!f || fread(&n, 4, 1, f) != 1 || fread(&nv, 4, 1, f) != 1) return 2;
    double *x = malloc(8 * n), *y = malloc(8 * n), *eps = malloc(8 * nv);
    unsigned int *mp = malloc(4 * nv), *ret = malloc(4 * (size_t)n * nv);
    if (fread(x, 8, n, f) != n || fread(y, 8, n, f) != n || fread(eps, 8, nv, f) != nv ||
        fread(mp, 4, nv, f) != nv) return 3;
    fclose(f);
    int rc = libVDBSCAN(x, y, n, eps, mp, nv, 70, ret, false);
    if (rc != 0) { fprintf(stderr, "rc %d\n", rc); return 4; }
    FILE *o = fopen(argv[2], "wb");
    fwrite(ret, 4, (size_t)n * nv, o);
    fclose(o);
    return 0;
}
"""


@pytest.mark.gpu
def test_c_program_links_and_matches_the_reference_fixture(tmp_path):
    from variantdbscan_gb300 import build
    lib = build.build()
    c = load("reference_test_dataset")
    n, nv = len(c["x"]), len(c["eps"])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, nv], np.uint32).tofile(f)
        np.asarray(c["x"], np.float64).tofile(f)
        np.asarray(c["y"], np.float64).tofile(f)
        np.asarray(c["eps"], np.float64).tofile(f)
        np.asarray(c["minpts"], np.uint32).tofile(f)
    src = tmp_path / "caller.c"
    src.write_text(C_SRC)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(lib)
    r = subprocess.run(["gcc", "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", libdir, "-lSharedVDBSCAN", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    env = dict(os.environ, LD_LIBRARY_PATH=libdir + ":" + os.environ.get("LD_LIBRARY_PATH", ""))
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.uint32).reshape(nv, n)
    np.testing.assert_array_equal(got, c["labels"])
