"""FP64 brute-force k-NN and embedding quality metrics (test infrastructure only)."""
from __future__ import annotations

import numpy as np


def exact_knn(X: np.ndarray, k: int, queries: np.ndarray | None = None, metric: str = "euclidean",
              block: int = 2048):
    """Exact k nearest neighbours in float64, self excluded.

    Returns (indices, dists) for the query rows (all rows by default); dists
    are squared L2 for euclidean and 2(1 - cos) on L2-normalised rows for
    cosine -- the engine's published conventions.
    """
    X = np.asarray(X, dtype=np.float64)
    if metric == "cosine":
        nrm = np.linalg.norm(X, axis=1, keepdims=True)
        X = X / np.where(nrm > 0, nrm, 1.0)
    q = np.arange(X.shape[0]) if queries is None else np.asarray(queries)
    sq = np.einsum("ij,ij->i", X, X)
    idx = np.empty((len(q), k), dtype=np.int64)
    dst = np.empty((len(q), k), dtype=np.float64)
    for s in range(0, len(q), block):
        qq = q[s : s + block]
        d = sq[qq, None] + sq[None, :] - 2.0 * (X[qq] @ X.T)
        np.maximum(d, 0.0, out=d)
        d[np.arange(len(qq)), qq] = np.inf
        part = np.argpartition(d, k, axis=1)[:, :k]
        pd = np.take_along_axis(d, part, axis=1)
        order = np.argsort(pd, axis=1, kind="stable")
        idx[s : s + len(qq)] = np.take_along_axis(part, order, axis=1)
        dst[s : s + len(qq)] = np.take_along_axis(pd, order, axis=1)
    return idx, dst


def recall_at_k(approx: np.ndarray, exact: np.ndarray) -> float:
    """Mean over rows of |approx_row & exact_row| / k."""
    k = exact.shape[1]
    hits = 0
    for a, e in zip(approx, exact):
        hits += len(set(a[:k].tolist()) & set(e.tolist()))
    return hits / (k * len(exact))


def trustworthiness(X: np.ndarray, E: np.ndarray, n_neighbors: int = 15, sample: np.ndarray | None = None,
                    block: int = 1024) -> float:
    """Trustworthiness of embedding E w.r.t. X (Venna & Kaski), computed over
    the sample rows in blocks so no n x n matrix is formed."""
    X = np.asarray(X, dtype=np.float64)
    E = np.asarray(E, dtype=np.float64)
    n = X.shape[0]
    rows = np.arange(n) if sample is None else np.asarray(sample)
    k = n_neighbors
    sx = np.einsum("ij,ij->i", X, X)
    se = np.einsum("ij,ij->i", E, E)
    total = 0.0
    for s in range(0, len(rows), block):
        r = rows[s : s + block]
        dx = sx[r, None] + sx[None, :] - 2.0 * (X[r] @ X.T)
        dx[np.arange(len(r)), r] = -np.inf  # self ranks first
        rank_x = np.empty_like(dx, dtype=np.int64)
        order = np.argsort(dx, axis=1, kind="stable")
        rank_x[np.arange(len(r))[:, None], order] = np.arange(n)[None, :]
        de = se[r, None] + se[None, :] - 2.0 * (E[r] @ E.T)
        de[np.arange(len(r)), r] = -np.inf
        nn_e = np.argpartition(de, k + 1, axis=1)[:, : k + 1]
        for i in range(len(r)):
            nb = nn_e[i][nn_e[i] != r[i]][:k]
            rk = rank_x[i, nb]  # rank 0 is self
            total += np.sum(np.maximum(rk - k, 0))
    m = len(rows)
    return 1.0 - 2.0 / (m * k * (2.0 * n - 3.0 * k - 1.0)) * total
