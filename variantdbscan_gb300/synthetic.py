"""Seeded synthetic point sets with the shapes of the benchmark workloads.

Coordinates are 2-D FP64 degrees: lon in [0, 360), lat in [-90, 90].  Blob
points wrap in longitude and are clipped in latitude.  The reference papers
cluster a space-weather TEC dataset that is not distributed with the
reference; these generators stand in for it.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Dataset:
    x: np.ndarray
    y: np.ndarray
    eps: np.ndarray
    minpts: np.ndarray
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.x)


def _blobs(rng, n, nblobs, sig_lo, sig_hi, bg_frac, weights=None, lattice=None):
    nbg = int(round(n * bg_frac))
    nbl = n - nbg
    cx = rng.uniform(0.0, 360.0, nblobs)
    cy = rng.uniform(-90.0, 90.0, nblobs)
    sig = rng.uniform(sig_lo, sig_hi, nblobs)
    if weights is None:
        weights = np.full(nblobs, 1.0 / nblobs)
    which = rng.choice(nblobs, size=nbl, p=weights)
    bx = cx[which] + rng.standard_normal(nbl) * sig[which]
    by = cy[which] + rng.standard_normal(nbl) * sig[which]
    ux = rng.uniform(0.0, 360.0, nbg)
    uy = rng.uniform(-90.0, 90.0, nbg)
    x = np.concatenate([bx, ux])
    y = np.concatenate([by, uy])
    perm = rng.permutation(n)
    x = np.mod(x[perm], 360.0)
    y = np.clip(y[perm], -90.0, 90.0)
    if lattice is not None:
        steps = float(round(1.0 / lattice))
        x = np.rint(x * steps) / steps
        y = np.rint(y * steps) / steps
        x = np.where(x >= 360.0, x - 360.0, x)
    return np.ascontiguousarray(x), np.ascontiguousarray(y)


def single_variant(n: int = 50_000, seed: int = 0) -> Dataset:
    """Plain single-variant DBSCAN: 80% in 8 equal Gaussian blobs
    (sigma ~ U[0.5, 3] deg), 20% uniform; eps = 0.5 deg, minpts = 10."""
    rng = np.random.default_rng(seed)
    x, y = _blobs(rng, n, 8, 0.5, 3.0, 0.20)
    return Dataset(x, y, np.array([0.5]), np.array([10], np.uint32),
                   name=f"single_variant_n{n}")


def variant_sweep(n: int = 2_000_000, seed: int = 1) -> Dataset:
    """Variant sweep: 64 blobs (sigma ~ U[0.2, 2] deg, Dirichlet(1) weights)
    plus 10% uniform; 16 variants eps {0.1,0.2,0.4,0.8} x minpts {4,16,64,256}."""
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(64))
    x, y = _blobs(rng, n, 64, 0.2, 2.0, 0.10, weights=w)
    eps, mp = np.meshgrid([0.1, 0.2, 0.4, 0.8], [4, 16, 64, 256], indexing="ij")
    return Dataset(x, y, eps.ravel().astype(np.float64), mp.ravel().astype(np.uint32),
                   name=f"variant_sweep_n{n}")


def multi_dataset(count: int = 64, seed: int = 2, n_lo: int = 10_000,
                  n_hi: int = 1_000_000) -> list[Dataset]:
    """Uneven multi-dataset batch: point counts log-uniform in [n_lo, n_hi],
    4-32 blobs (sigma ~ U[0.2, 3]) plus 5-30% uniform; 4-12 variants each with
    eps log-uniform in [0.05, 1.5] and minpts uniform in [4, 128]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        nb = int(rng.integers(4, 33))
        bg = float(rng.uniform(0.05, 0.30))
        x, y = _blobs(rng, n, nb, 0.2, 3.0, bg)
        nv = int(rng.integers(4, 13))
        eps = np.exp(rng.uniform(np.log(0.05), np.log(1.5), nv))
        mp = rng.integers(4, 129, nv).astype(np.uint32)
        out.append(Dataset(x, y, eps, mp, name=f"multi_{i}_n{n}"))
    return out


def lattice_stress(n: int = 10_000_000, seed: int = 3) -> Dataset:
    """Mixed-precision boundary stress: coordinates on a 0.01 deg lattice, 70%
    in 256 blobs (sigma ~ U[0.05, 0.5] deg), 30% uniform; 8 variants
    eps {0.05,0.1,0.25,0.5} x minpts {8,32}."""
    rng = np.random.default_rng(seed)
    x, y = _blobs(rng, n, 256, 0.05, 0.5, 0.30, lattice=0.01)
    eps, mp = np.meshgrid([0.05, 0.1, 0.25, 0.5], [8, 32], indexing="ij")
    return Dataset(x, y, eps.ravel().astype(np.float64), mp.ravel().astype(np.uint32),
                   name=f"lattice_stress_n{n}")


def request_stream(count: int = 2000, seed: int = 4, n_lo: int = 10_000,
                   n_hi: int = 5_000_000):
    """Serving loop requests: (arrival offset in units of the mean gap, Dataset)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0, count)
    t = np.cumsum(gaps)
    reqs = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        nb = int(rng.integers(4, 33))
        bg = float(rng.uniform(0.05, 0.30))
        sub = np.random.default_rng([seed, i])
        x, y = _blobs(sub, n, nb, 0.2, 3.0, bg)
        nv = int(rng.integers(1, 33))
        eps = np.exp(rng.uniform(np.log(0.05), np.log(1.5), nv))
        mp = rng.integers(4, 129, nv).astype(np.uint32)
        reqs.append((float(t[i]), Dataset(x, y, eps, mp, name=f"req_{i}_n{n}")))
    return reqs
