"""Synthetic datasets, PCA, k-means, ground truth and .fvecs/.ivecs I/O.

The reference prepares its inputs with faiss (python/ivf.py: k-means ->
centroids + cluster ids on the raw vectors; python/pca.py: a mean-centred PCA
applied to base, queries and centroids).  faiss is not available here, so these
are plain numpy restatements with fixed seeds.  They produce the inputs for
both the GPU index and the CPU oracle, so parity never depends on them.

Generators (all float32, seeded):
  * gaussian_mixture: centres ~ N(0,1)^d, point = centre + N(0, sigma^2).
  * anisotropic: random orthogonal basis, per-axis variance ~ i^-alpha,
    rows normalised to unit length.
  * zipf_mixture: anisotropic centres with Zipf(s)-distributed cluster sizes;
    the component index is the IVF cluster id.
  * int_grid: the reference's own unit-test generator (unit_test/test_base.hpp:55-88):
    integers in [-8, 8], centroid 0 = 0, other centroids constant rows,
    cluster id = i % K.
"""
from __future__ import annotations

import numpy as np


# ---------------------------------------------------------------------------
# I/O in the reference's formats (saqlib/utils/IO.hpp:62-141, python/utils/io.py)
# ---------------------------------------------------------------------------
def write_fvecs(path, x: np.ndarray) -> None:
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    out = np.empty((n, d + 1), dtype=np.float32)
    out[:, 0] = np.frombuffer(np.int32(d).tobytes(), dtype=np.float32)[0]
    out[:, 1:] = x
    out.tofile(path)


def read_fvecs(path) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.int32)
    d = int(raw[0])
    return raw.reshape(-1, d + 1)[:, 1:].view(np.float32).copy()


def write_ivecs(path, x: np.ndarray) -> None:
    x = np.ascontiguousarray(x, dtype=np.int32)
    n, d = x.shape
    out = np.empty((n, d + 1), dtype=np.int32)
    out[:, 0] = d
    out[:, 1:] = x
    out.tofile(path)


def read_ivecs(path) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.int32)
    d = int(raw[0])
    return raw.reshape(-1, d + 1)[:, 1:].copy()


# ---------------------------------------------------------------------------
# Generators
# ---------------------------------------------------------------------------
def gaussian_mixture(n: int, d: int, n_centers: int, sigma: float = 0.5, seed: int = 0,
                     n_query: int = 0):
    rng = np.random.default_rng(seed)
    centers = rng.standard_normal((n_centers, d), dtype=np.float32)
    lab = rng.integers(0, n_centers, size=n)
    x = centers[lab] + sigma * rng.standard_normal((n, d), dtype=np.float32)
    q = None
    if n_query:
        lq = rng.integers(0, n_centers, size=n_query)
        q = centers[lq] + sigma * rng.standard_normal((n_query, d), dtype=np.float32)
    return x.astype(np.float32), (None if q is None else q.astype(np.float32))


def random_orthogonal(d: int, rng) -> np.ndarray:
    a = rng.standard_normal((d, d))
    q, r = np.linalg.qr(a)
    q *= np.sign(np.diag(r))[None, :]
    return q


def anisotropic(n: int, d: int, alpha: float = 0.8, seed: int = 0, n_query: int = 0):
    """Unit-norm rows with per-axis variance ~ i^-alpha in a random orthogonal basis."""
    rng = np.random.default_rng(seed)
    basis = random_orthogonal(d, rng).astype(np.float32)
    scale = (np.arange(1, d + 1, dtype=np.float64) ** (-alpha / 2)).astype(np.float32)

    def draw(m):
        z = rng.standard_normal((m, d), dtype=np.float32) * scale[None, :]
        v = z @ basis.T
        v /= np.linalg.norm(v, axis=1, keepdims=True) + 1e-30
        return v.astype(np.float32)

    x = draw(n)
    q = draw(n_query) if n_query else None
    return x, q


def zipf_sizes(n: int, k: int, s: float = 1.1) -> np.ndarray:
    """Cluster sizes proportional to rank^-s, summing exactly to n (largest first)."""
    w = np.arange(1, k + 1, dtype=np.float64) ** (-s)
    w /= w.sum()
    sizes = np.floor(w * n).astype(np.int64)
    rem = n - int(sizes.sum())
    frac = w * n - sizes
    order = np.argsort(-frac, kind="stable")
    sizes[order[:rem]] += 1
    return sizes


def int_grid(num_data: int, num_query: int, num_dim: int, num_centroids: int = 1, seed: int = 42):
    """Integer test data in the style of the reference unit tests (test_base.hpp:55-88).

    numpy's generator replaces std::mt19937, so the values differ from the
    reference's, but the structure (values in [-8, 8], zero centroid 0,
    constant-row centroids that repeat, cid = i % K) is the same.
    """
    rng = np.random.default_rng(seed)
    dpad = (num_dim + 63) // 64 * 64
    x = np.zeros((num_data, dpad), dtype=np.float32)
    x[:, :num_dim] = rng.integers(-8, 9, size=(num_data, num_dim))
    q = np.zeros((num_query, dpad), dtype=np.float32)
    q[:, :num_dim] = rng.integers(-8, 9, size=(num_query, num_dim))
    c = np.zeros((num_centroids, dpad), dtype=np.float32)
    for i in range(1, num_centroids):
        c[i, :num_dim] = float(rng.integers(-8, 9))
    cids = (np.arange(num_data) % num_centroids).astype(np.uint32)
    return x, q, c, cids


# ---------------------------------------------------------------------------
# PCA and k-means (restating python/pca.py and python/ivf.py without faiss)
# ---------------------------------------------------------------------------
def pca_fit(x: np.ndarray):
    """Mean and components (rows, descending eigenvalue) of a full-rank PCA."""
    x64 = x.astype(np.float64)
    mean = x64.mean(axis=0)
    xc = x64 - mean
    cov = xc.T @ xc / max(1, x.shape[0])
    w, v = np.linalg.eigh(cov)
    order = np.argsort(-w, kind="stable")
    comp = v[:, order].T
    return mean.astype(np.float32), comp.astype(np.float32), w[order]


def pca_apply(x: np.ndarray, mean: np.ndarray, comp: np.ndarray) -> np.ndarray:
    return ((x - mean[None, :]) @ comp.T).astype(np.float32)


def kmeans(x: np.ndarray, k: int, iters: int = 20, seed: int = 0, batch: int = 65536):
    """Lloyd's k-means (L2), seeded by k distinct random points; empty clusters keep their centre."""
    rng = np.random.default_rng(seed)
    n = x.shape[0]
    cent = x[rng.choice(n, size=k, replace=False)].astype(np.float32).copy()
    assign = np.zeros(n, dtype=np.int64)
    for _ in range(iters + 1):
        cn = (cent.astype(np.float64) ** 2).sum(1)
        for s in range(0, n, batch):
            xb = x[s:s + batch].astype(np.float64)
            d = cn[None, :] - 2.0 * xb @ cent.T.astype(np.float64)
            assign[s:s + batch] = np.argmin(d, axis=1)
        if _ == iters:
            break
        sums = np.zeros((k, x.shape[1]), dtype=np.float64)
        np.add.at(sums, assign, x.astype(np.float64))
        cnt = np.bincount(assign, minlength=k)
        nz = cnt > 0
        cent[nz] = (sums[nz] / cnt[nz, None]).astype(np.float32)
    return cent, assign.astype(np.uint32)


def assign_nearest(x: np.ndarray, cent: np.ndarray, batch: int = 65536) -> np.ndarray:
    cn = (cent.astype(np.float64) ** 2).sum(1)
    out = np.empty(x.shape[0], dtype=np.uint32)
    for s in range(0, x.shape[0], batch):
        xb = x[s:s + batch].astype(np.float64)
        out[s:s + batch] = np.argmin(cn[None, :] - 2.0 * xb @ cent.T.astype(np.float64), axis=1)
    return out


def ground_truth(x: np.ndarray, q: np.ndarray, k: int, shortlist: int = 200, batch: int = 256):
    """Exact FP64 top-k by L2: FP32 shortlist of `shortlist`, then FP64 re-rank."""
    n = x.shape[0]
    sl = min(shortlist, n)
    xn = (x.astype(np.float32) ** 2).sum(1)
    out = np.empty((q.shape[0], k), dtype=np.int64)
    for s in range(0, q.shape[0], batch):
        qb = q[s:s + batch]
        d = xn[None, :] - 2.0 * qb @ x.T
        cand = np.argpartition(d, sl - 1, axis=1)[:, :sl]
        for i in range(qb.shape[0]):
            c = cand[i]
            dd = ((x[c].astype(np.float64) - qb[i].astype(np.float64)) ** 2).sum(1)
            o = np.lexsort((c, dd))[:k]
            out[s + i] = c[o]
    return out


def recall_at_k(found: np.ndarray, gt: np.ndarray, k: int) -> float:
    hit = 0
    for f, g in zip(found, gt):
        hit += len(set(f[:k].tolist()) & set(g[:k].tolist()))
    return hit / (k * len(gt))
