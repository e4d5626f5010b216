"""Places the GB300 library where the reference's Python wrapper loads it.

The reference's wrapper (python_package/vdbscan/variantdbscan.py:46,52) loads
``libSharedVDBSCAN`` from the ``lib/`` directory beside its own file, where
the reference's setup.py builds its CPU library (extension
``vdbscan.lib.libSharedVDBSCAN``).  Copying this build's library there turns an
installed reference package into a GB300 one without touching its Python code:

    python -m variantdbscan_gb300.install <directory of the vdbscan package>
"""
from __future__ import annotations

import os
import shutil
import sys

from . import LIB_PATH

LIB_NAME = "libSharedVDBSCAN.so"


def place_library(package_dir: str, lib_path: str = LIB_PATH) -> str:
    """Copies lib_path to <package_dir>/lib/libSharedVDBSCAN.so (replacing the
    reference's CPU library if one is there) and returns the new path."""
    if not os.path.isfile(lib_path):
        raise FileNotFoundError(f"{lib_path} is missing: build the library first")
    if not os.path.isdir(package_dir):
        raise NotADirectoryError(package_dir)
    dst_dir = os.path.join(package_dir, "lib")
    os.makedirs(dst_dir, exist_ok=True)
    dst = os.path.join(dst_dir, LIB_NAME)
    tmp = dst + ".tmp"
    shutil.copyfile(lib_path, tmp)
    os.replace(tmp, dst)
    return dst


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m variantdbscan_gb300.install <vdbscan package directory>")
    print(place_library(sys.argv[1]))
