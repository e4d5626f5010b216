"""Command line of the GPU prototype (src/gpu/main.cu:76-97): a dataset file
and a variant file in, labels out.

    python -m variantdbscan_gb300.cli <dataset file> <variant file> [--out labels.csv]

Both files are read as the prototype reads them (vdb_import_dataset,
vdb_import_variants); every variant is clustered in one vdb_run_batch call.
The output has one line per point: x, y, then one label per variant in the
sorted variant order (0 = noise).
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

import variantdbscan_gb300 as v


def main(argv=None) -> int:
    p = argparse.ArgumentParser(prog="variantdbscan_gb300.cli")
    p.add_argument("dataset")
    p.add_argument("variants")
    p.add_argument("--out", default="-", help="output CSV (default: standard output)")
    p.add_argument("--mbb", type=int, default=70, help="the reference's MBBsize")
    a = p.parse_args(argv)
    x, y = v.import_dataset(a.dataset)
    eps, mp = v.import_variants(a.variants)
    ctx = v.Context()
    try:
        (lab,), st = ctx.run([v.BatchItem(x, y, eps, mp, a.mbb)])
    finally:
        ctx.close()
    out = sys.stdout if a.out == "-" else open(a.out, "w")
    try:
        out.write("# " + " ".join(f"eps={e:g}/minpts={m}" for e, m in zip(eps, mp)) + "\n")
        cols = np.column_stack([x, y] + [lab[i] for i in range(len(eps))])
        for row in cols:
            out.write(f"{float(row[0])!r},{float(row[1])!r}," + ",".join(str(int(c)) for c in row[2:]) + "\n")
    finally:
        if out is not sys.stdout:
            out.close()
    print(f"{len(x)} points, {len(eps)} variants, {st['clusters']} clusters, "
          f"{st['ms_total']:.2f} ms", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
