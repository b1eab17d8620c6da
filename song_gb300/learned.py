"""Learned early exit: traces from the plain search, training on the GPU with
the library's own kernels, threshold selection, evaluation.

No counterpart in the reference (its search always runs to the pq_size
budget's finish rule, warp_astar_accelerator.h:191).  The network reads the
query's state after each hop and stops the search once it is confident that
the current top-k is already the final one; a query it never trusts runs the
plain search unchanged, so the plain search is both the fallback and, through
the labels, the reference the exit is trained against.

Label of a hop: "the top-k set after this hop equals the top-k set the plain
search returns" (the trace records how many times the top-k set has changed,
so a hop is positive when that count already equals the final count).

torch is used here only to hold device buffers and draw permutations; the
search, the tracing and the training run in libsong_gb300.so.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import TRACE_FIELDS, Index, mlp_init, mlp_train_device


@dataclass
class ExitModel:
    params: np.ndarray
    threshold: float
    min_hops: int
    every: int
    pq: int
    k: int
    info: dict = field(default_factory=dict)


def plain_stats(index: Index, dq, pq: int, k: int):
    """Device search with stats; returns (ids uint64 np, hops np, evals np)."""
    import torch
    nq = dq.shape[0]
    out = torch.empty((nq, k), dtype=torch.int64, device=dq.device)
    hops = torch.empty(nq, dtype=torch.int32, device=dq.device)
    evals = torch.empty(nq, dtype=torch.int32, device=dq.device)
    s = torch.cuda.current_stream()
    index.search_device(dq.data_ptr(), nq, pq, k, out.data_ptr(), hops.data_ptr(), evals.data_ptr(), s.cuda_stream)
    s.synchronize()
    return out.cpu().numpy().view(np.uint64), hops.cpu().numpy(), evals.cpu().numpy()


def trace_dataset(index: Index, queries: np.ndarray, pq: int, k: int, chunk: int = 4096,
                  max_samples_per_query: int = 0, seed: int = 0):
    """Runs the plain search with tracing; returns device tensors X (n x 5),
    y (n) of hop samples, and the plain ids of every query."""
    import torch
    rng = np.random.default_rng(seed)
    dq_all = torch.from_numpy(np.ascontiguousarray(queries, np.float32)).cuda()
    _, hops, _ = plain_stats(index, dq_all[: min(chunk, dq_all.shape[0])], pq, k)
    trace_hops = int(max(16, hops.max() * 2 + 16))
    xs, ys = [], []
    for a in range(0, dq_all.shape[0], chunk):
        dq = dq_all[a:a + chunk]
        nq = dq.shape[0]
        tr = torch.empty(nq * trace_hops * TRACE_FIELDS, dtype=torch.float32, device="cuda")
        fin = torch.empty(nq * 2, dtype=torch.int32, device="cuda")
        out = torch.empty((nq, k), dtype=torch.int64, device="cuda")
        s = torch.cuda.current_stream()
        index.trace_device(dq.data_ptr(), nq, pq, k, trace_hops, tr.data_ptr(), fin.data_ptr(), out.data_ptr(),
                           stream=s.cuda_stream)
        s.synchronize()
        tr = tr.view(nq, trace_hops, TRACE_FIELDS)
        fin = fin.view(nq, 2).long()
        h = torch.arange(trace_hops, device="cuda")[None, :]
        valid = h < fin[:, 1:2]
        if max_samples_per_query > 0:
            # keep a random subset of each query's hops (uniform over its hops)
            keep = torch.rand(valid.shape, device="cuda",
                              generator=torch.Generator(device="cuda").manual_seed(int(rng.integers(1 << 30))))
            frac = (max_samples_per_query / fin[:, 1:2].clamp_min(1).float()).clamp(max=1.0)
            valid = valid & (keep < frac)
        lab = (tr[:, :, 5] == fin[:, 0:1].float()).float()
        xs.append(tr[:, :, :5][valid].contiguous())
        ys.append(lab[valid].contiguous())
    return torch.cat(xs), torch.cat(ys)


def train(X, y, epochs: int = 6, batch: int = 8192, lr: float = 2e-3, neg_weight: float = 4.0,
          seed: int = 0):
    """Trains the network with the library's CUDA kernels.  Negative samples
    (top-k still changing) weigh `neg_weight`: a premature stop costs recall,
    a late one only time."""
    import torch
    n = X.shape[0]
    w = torch.where(y > 0.5, torch.ones_like(y), torch.full_like(y, neg_weight))
    params = torch.from_numpy(mlp_init(seed)).cuda()
    g = torch.Generator(device="cuda").manual_seed(seed)
    perm = torch.cat([torch.randperm(n, device="cuda", generator=g) for _ in range(epochs)]).to(torch.int32)
    losses = torch.zeros(epochs, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()
    t = time.time()
    mlp_train_device(X.data_ptr(), y.data_ptr(), w.data_ptr(), n, perm.data_ptr(), epochs, batch, lr,
                     params.data_ptr(), losses.data_ptr(), s.cuda_stream)
    s.synchronize()
    return params.cpu().numpy(), losses.cpu().numpy(), time.time() - t


def evaluate(index: Index, dq, pq: int, k: int, params=None, threshold=0.0, min_hops=8, every=1, max_hops=0):
    """Search with the exit (or a fixed hop budget, or neither); returns ids, hops, evals."""
    index.set_early_exit(params, threshold, min_hops, every) if params is not None else index.set_early_exit(None)
    index.set_hop_limit(max_hops)
    try:
        return plain_stats(index, dq, pq, k)
    finally:
        index.set_early_exit(None)
        index.set_hop_limit(0)


THRESHOLDS = [round(4.0 - 0.25 * i, 2) for i in range(23)]  # 4.0 .. -1.5


def fit(index: Index, train_queries: np.ndarray, pq: int, k: int, val_frac: float = 0.2,
        agreement: float = 0.995, min_hops: int = 8, every: int = 4, epochs: int = 6,
        max_samples_per_query: int = 256, seed: int = 0, data=None, metric=None,
        recall_slack: float = None, log=None) -> ExitModel:
    """Trace, train, and choose the threshold on held-out training queries.

    With `data`/`metric` and `recall_slack`, the chosen threshold is the most
    permissive one whose validation recall@k (tie-aware, against an FP64
    exact kNN) stays within `recall_slack` of the search without exit;
    otherwise the most permissive one that keeps the exit-free top-k on at
    least `agreement` of the validation queries."""
    import torch
    from . import groundtruth as GT
    nval = max(1, int(len(train_queries) * val_frac))
    tq, vq = train_queries[nval:], train_queries[:nval]
    t0 = time.time()
    X, y = trace_dataset(index, tq, pq, k, max_samples_per_query=max_samples_per_query, seed=seed)
    t_trace = time.time() - t0
    params, losses, t_train = train(X, y, epochs=epochs, seed=seed)
    dv = torch.from_numpy(np.ascontiguousarray(vq, np.float32)).cuda()
    # the exit-free search of the same kernel: a hop budget no query reaches
    base_ids, base_hops, _ = evaluate(index, dv, pq, k, max_hops=1 << 30)
    use_recall = data is not None and recall_slack is not None
    if use_recall:
        _, kth = GT.exact_knn_fp64(data, vq, k, metric)
        base_rec = GT.recall_tie_aware(base_ids, data, vq, kth, metric, k)
    best, curve = None, []
    for thr in THRESHOLDS:
        ids, hops, _ = evaluate(index, dv, pq, k, params, thr, min_hops, every)
        agree = float((np.sort(ids, axis=1) == np.sort(base_ids, axis=1)).all(axis=1).mean())
        row = [thr, round(agree, 4), round(float(hops.mean()), 2)]
        ok = agree >= agreement
        if use_recall:
            rec = GT.recall_tie_aware(ids, data, vq, kth, metric, k)
            row.append(round(rec, 4))
            ok = rec >= base_rec - recall_slack
        curve.append(row)
        if ok:
            best = row
        elif best is not None:
            break  # thresholds only get more permissive from here
    if best is None:
        best = curve[0]
    info = dict(samples=int(X.shape[0]), positive=float(y.mean().item()), trace_s=round(t_trace, 2),
                train_s=round(t_train, 2), losses=[round(float(v), 4) for v in losses],
                val_plain_hops=float(base_hops.mean()), threshold_curve=curve, chosen=best,
                val_recall_no_exit=round(base_rec, 4) if use_recall else None)
    if log:
        log("[learned] %s" % info)
    return ExitModel(params=params, threshold=best[0], min_hops=min_hops, every=every, pq=pq, k=k, info=info)
