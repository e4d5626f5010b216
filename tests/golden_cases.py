"""Loads the golden fixtures of tests/golden/ (made by make_golden.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES = ["reference_test_dataset", "vtest", "single_variant_3k", "variant_sweep_4k",
         "lattice_4k", "lattice_4k_mbb1", "edge_negative_dupes"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def adversarial():
    """List of single-variant cases (x, y, eps, minpts, mbb, labels)."""
    z = load("adversarial_asymmetric")
    off = z["offsets"]
    out = []
    for i in range(len(off) - 1):
        s, e = off[i], off[i + 1]
        out.append(dict(x=z["x"][s:e].copy(), y=z["y"][s:e].copy(), eps=float(z["eps"][i]),
                        minpts=int(z["minpts"][i]), mbb=int(z["mbb"][i]),
                        labels=z["labels"][s:e].copy()))
    return out
