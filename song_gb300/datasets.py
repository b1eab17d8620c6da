"""Seeded synthetic stand-ins for the workloads the reference measures on.

The reference's datasets (LIBSVM letter, SIFT1M, GIST1M, UQ_V; README.md:10-20)
are not available here; these generators produce vectors of the same shapes
and value ranges from Gaussian mixtures.  Seeds: base vectors 1, queries 2,
training queries 3, serving stream 4.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED_BASE, SEED_QUERY, SEED_TRAIN, SEED_SERVE = 1, 2, 3, 4


@dataclass(frozen=True)
class Workload:
    name: str
    n: int
    dim: int
    metric: str
    shift: int            # log2 of the adjacency row width
    search_degree: int    # out-edges kept per insertion (SEARCH_DEGREE)
    fixed_degree: int     # row capacity (FIXED_DEGREE)
    n_queries: int
    centers: int
    kind: str             # generator family


# degree-16 graph: FIXED_DEGREE 15, SHIFT 4, SEARCH_DEGREE 7; degree-32: 31, 5, 15.
SMALL = Workload("small-15k-16d-cos", 15_000, 16, "cos", 4, 7, 15, 5_000, 26, "unit")
SCALE = Workload("scale-1m-128d-l2", 1_000_000, 128, "l2", 5, 15, 31, 10_000, 1_000, "byte")
PRECISION = Workload("precision-1m-960d-cos", 1_000_000, 960, "cos", 5, 15, 31, 1_000, 500, "unit01")
LEARNED = Workload("learned-3m-256d-l2", 3_000_000, 256, "l2", 5, 15, 31, 10_000, 2_000, "normal")

WORKLOADS = {w.name: w for w in (SMALL, SCALE, PRECISION, LEARNED)}


def _centers(kind, k, dim, rng):
    if kind == "unit":
        return rng.uniform(-1.0, 1.0, size=(k, dim)).astype(np.float32)
    if kind == "byte":
        return rng.uniform(0.0, 255.0, size=(k, dim)).astype(np.float32)
    if kind == "unit01":
        return rng.uniform(0.0, 1.0, size=(k, dim)).astype(np.float32)
    if kind == "normal":
        return rng.standard_normal(size=(k, dim), dtype=np.float32)
    raise ValueError(kind)


def _finish(kind, x):
    if kind == "unit":
        np.clip(x, -1.0, 1.0, out=x)
    elif kind == "byte":
        np.rint(x, out=x)
        np.clip(x, 0.0, 255.0, out=x)
    elif kind == "unit01":
        np.clip(x, 0.0, 1.0, out=x)
    return x


def _sigma(kind):
    return {"unit": 0.15, "byte": 20.0, "unit01": 0.05, "normal": 0.3}[kind]


def mixture(kind, n, dim, k, seed, center_seed=SEED_BASE, chunk=1 << 18):
    """n vectors from the k-centre mixture of `kind`.  The centres always come
    from `center_seed`, so base and query sets share one mixture."""
    centers = _centers(kind, k, dim, np.random.default_rng(center_seed))
    rng = np.random.default_rng(seed)
    out = np.empty((n, dim), dtype=np.float32)
    sig = np.float32(_sigma(kind))
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        lab = rng.integers(0, k, size=b - a)
        noise = rng.standard_normal(size=(b - a, dim), dtype=np.float32)
        noise *= sig
        noise += centers[lab]
        out[a:b] = _finish(kind, noise)
    return out


def base_vectors(w: Workload, n=None):
    # The centre stream is drawn from a generator of its own (seed base+100) so
    # that base and query draws are independent of the centre draw.
    return mixture(w.kind, w.n if n is None else n, w.dim, w.centers, SEED_BASE, center_seed=SEED_BASE + 100)


def query_vectors(w: Workload, nq=None, seed=SEED_QUERY):
    return mixture(w.kind, w.n_queries if nq is None else nq, w.dim, w.centers, seed,
                   center_seed=SEED_BASE + 100)
