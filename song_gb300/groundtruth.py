"""FP64 brute-force exact k-nearest neighbours and recall.

Ranking follows the metrics of the search: L2 = squared Euclidean distance;
IP = negative inner product; COS = negative cosine similarity (the kernel's
-sign(q.x)(q.x)^2/|x|^2 orders a query's vectors the same way), with a
zero-norm base vector at distance 0, as in the kernel.

Candidates come from an FP64 matrix product (torch on the GPU when one is
present, numpy otherwise); the top k + `extra` of each query are then
re-scored element by element in FP64 and sorted, so the reported k-th distance
does not depend on the product's rounding.
"""
from __future__ import annotations

import numpy as np

METRIC_CODES = {"l2": 0, "ip": 1, "cos": 2}


def _code(metric):
    return METRIC_CODES[metric] if isinstance(metric, str) else int(metric)


def distances_fp64(data, queries, ids, metric, chunk=1024):
    """Exact distances of queries[i] to data[ids[i, j]] (ids may hold
    UINT64_MAX for empty slots, which get +inf)."""
    ids = np.asarray(ids)
    if ids.shape[0] > chunk:
        return np.concatenate([distances_fp64(data, queries[a:a + chunk], ids[a:a + chunk], metric, chunk)
                               for a in range(0, ids.shape[0], chunk)])
    m = _code(metric)
    ids = np.asarray(ids)
    valid = ids != np.uint64(0xFFFFFFFFFFFFFFFF) if ids.dtype == np.uint64 else ids >= 0
    safe = np.where(valid, ids, 0).astype(np.int64)
    x = data[safe].astype(np.float64)                      # nq x m x dim
    q = np.asarray(queries, dtype=np.float64)[:, None, :]
    if m == 0:
        d = ((x - q) ** 2).sum(-1)
    elif m == 1:
        d = -(x * q).sum(-1)
    else:
        dot = (x * q).sum(-1)
        xn = np.sqrt((x * x).sum(-1))
        qn = np.sqrt((q * q).sum(-1))
        with np.errstate(divide="ignore", invalid="ignore"):
            d = np.where(xn > 0, -dot / (xn * qn), 0.0)
    return np.where(valid, d, np.inf)


def _scores_numpy(data64, dn, q64, m):
    dot = q64 @ data64.T
    if m == 0:
        return dn[None, :] - 2.0 * dot
    if m == 1:
        return -dot
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(dn[None, :] > 0, -dot / np.sqrt(np.maximum(dn, 1e-300))[None, :], 0.0)


def exact_knn_fp64(data, queries, k, metric, extra=32, chunk=None, device=None):
    """Returns (ids int64 nq x k, kth float64 nq): the exact k nearest ids and
    the k-th smallest exact distance of each query."""
    m = _code(metric)
    data = np.ascontiguousarray(data, dtype=np.float32)
    queries = np.ascontiguousarray(queries, dtype=np.float32)
    n = data.shape[0]
    kk = min(n, k + extra)
    nq = queries.shape[0]
    cand = np.empty((nq, kk), dtype=np.int64)
    use_torch = False
    try:
        import torch
        use_torch = torch.cuda.is_available() if device is None else device == "cuda"
    except Exception:
        use_torch = False
    if use_torch:
        import torch
        dev = torch.device("cuda")
        X = torch.from_numpy(data).to(dev, dtype=torch.float64)
        dn = (X * X).sum(1)
        step = chunk or max(1, min(nq, int(2e9 // (8 * n))))
        for a in range(0, nq, step):
            Q = torch.from_numpy(queries[a:a + step]).to(dev, dtype=torch.float64)
            dot = Q @ X.T
            if m == 0:
                s = dn[None, :] - 2.0 * dot
            elif m == 1:
                s = -dot
            else:
                s = torch.where(dn[None, :] > 0, -dot / torch.sqrt(dn.clamp_min(1e-300))[None, :],
                                torch.zeros_like(dot))
            cand[a:a + step] = torch.topk(s, kk, dim=1, largest=False).indices.cpu().numpy()
            del dot, s, Q
        del X, dn
        torch.cuda.empty_cache()
    else:
        data64 = data.astype(np.float64)
        dn = (data64 * data64).sum(1)
        step = chunk or max(1, min(nq, int(2e8 // max(1, n))))
        for a in range(0, nq, step):
            s = _scores_numpy(data64, dn, queries[a:a + step].astype(np.float64), m)
            part = np.argpartition(s, kk - 1, axis=1)[:, :kk]
            cand[a:a + step] = part
    d = distances_fp64(data, queries, cand, m)
    order = np.lexsort((cand, d), axis=1)
    cand = np.take_along_axis(cand, order, 1)[:, :k]
    d = np.take_along_axis(d, order, 1)
    return cand, d[:, k - 1]


def recall(found, gt_ids, k):
    """|found[:, :k] & gt[:, :k]| / k, averaged over queries."""
    found = np.asarray(found)[:, :k].astype(np.int64)
    gt = np.asarray(gt_ids)[:, :k].astype(np.int64)
    hits = 0
    for f, g in zip(found, gt):
        hits += len(np.intersect1d(f, g))
    return hits / float(found.shape[0] * k)


def recall_tie_aware(found, data, queries, kth, metric, k):
    """Fraction of the first k returned ids whose exact distance is <= the
    exact k-th nearest distance (equal distances count as correct, which
    matters for integer-valued L2 data where ties are common).  An id
    returned twice in one row counts once: the reference's visited hash can
    lose an entry, and the search can then list that vertex again."""
    f = np.asarray(found)[:, :k]
    d = distances_fp64(data, queries, f, metric)
    ok = d <= kth[:, None] + 1e-12 * np.abs(kth[:, None])
    order = np.argsort(f, axis=1, kind="stable")
    fs = np.take_along_axis(f, order, 1)
    first = np.ones_like(fs, dtype=bool)
    first[:, 1:] = fs[:, 1:] != fs[:, :-1]
    distinct = np.empty_like(first)
    np.put_along_axis(distinct, order, first, 1)
    return float((ok & distinct).sum()) / float(f.shape[0] * k)
