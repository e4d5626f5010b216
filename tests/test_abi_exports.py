"""The C-ABI library builds, loads and exports every symbol of include/vdbscan.h
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vdbscan.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from variantdbscan_gb300 import build
    return build.build()


def test_header_declares_reference_entry_point():
    names = declared_functions()
    assert "libVDBSCAN" in names
    assert "vdb_run_batch" in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True).stdout
    for name in declared_functions():
        assert re.search(rf"\bT {name}$", out, flags=re.M), name


def test_python_mirror_lists_exports(lib_path):
    import variantdbscan_gb300 as v
    assert sorted(v.EXPORTS) == declared_functions()


def test_header_compiles_as_c(tmp_path):
    c = tmp_path / "t.c"
    c.write_text('#include "vdbscan.h"\nint main(void){vdb_options o; (void)o; return 0;}\n')
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), "-c", str(c),
                        "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("cname,pyname", [("vdb_options", "Options"), ("vdb_stats", "Stats"),
                                          ("vdb_dataset", "Dataset")])
def test_python_structs_match_the_header(tmp_path, cname, pyname):
    # size and field offsets of the ctypes mirrors equal the C compiler's
    import variantdbscan_gb300 as v
    cls = getattr(v, pyname)
    fields = [f for f, _ in cls._fields_]
    body = "".join(f'printf("%zu\\n", offsetof({cname}, {f}));' for f in fields)
    c = tmp_path / "layout.c"
    c.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "vdbscan.h"\n'
                 f'int main(void){{printf("%zu\\n", sizeof({cname}));{body}return 0;}}\n')
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(t) for t in subprocess.run([str(exe)], capture_output=True,
                                          text=True).stdout.split()]
    assert got[0] == ctypes.sizeof(cls)
    assert got[1:] == [getattr(cls, f).offset for f in fields]


def test_python_constants_match_the_header(tmp_path):
    # the graph states and option values the Python mirror names
    import variantdbscan_gb300 as v
    names = {"VDB_GRAPH_NONE": v.GRAPH_NONE, "VDB_GRAPH_CAPTURED": v.GRAPH_CAPTURED,
             "VDB_GRAPH_REPLAYED": v.GRAPH_REPLAYED, "VDB_GRAPH_FALLBACK": v.GRAPH_FALLBACK,
             "VDB_GRAPH_UNSUPPORTED": v.GRAPH_UNSUPPORTED, "VDB_LOC_HOST": v.LOC_HOST,
             "VDB_LOC_DEVICE": v.LOC_DEVICE}
    body = "".join(f'printf("%d\\n", (int)({k}));' for k in names)
    c = tmp_path / "consts.c"
    c.write_text('#include <stdio.h>\n#include "vdbscan.h"\n'
                 f'int main(void){{{body}return 0;}}\n')
    exe = tmp_path / "consts"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(t) for t in subprocess.run([str(exe)], capture_output=True,
                                          text=True).stdout.split()]
    assert got == list(names.values())
