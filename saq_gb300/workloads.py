"""Seeded synthetic workloads with the shapes of the SAQ benchmark configurations,
generated on the GPU (torch), plus exact ground truth.

Public datasets are not available, so each workload is a seeded stand-in with
the configuration's sizes and value distributions:

  zipf_aniso (10M x 1024, 16,384 clusters): unit-norm vectors with an
      anisotropic spectrum (random orthogonal basis, per-axis variance ~
      i^-alpha); cluster centres from the same spectrum, cluster sizes
      ~ rank^-1.1 (Zipf); point = normalise(centre + sigma * noise).  The
      cluster index is the IVF cluster id; centroids are the cluster means.
  PCA: mean-centred, components by descending eigenvalue (the reference's
      python/pca.py workflow), applied to base, queries and centroids.

  gaussian_mixture_ivf (100k x 960, 1,024 clusters): centres ~ N(0,1)^d,
      point = centre + N(0, sigma^2) per coordinate; PCA over the base set;
      IVF centroids from k-means (Lloyd, 20 iterations).
  aniso_ivf (1M x 1024, 4,096 clusters): unit-norm rows with per-axis
      variance ~ i^-alpha in a random orthogonal basis; PCA; k-means.

Queries follow the base distribution (their clusters drawn with the same
Zipf weights).  Ground truth is exact: an FP32 shortlist followed by an FP64
re-rank.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from .data import zipf_sizes


@dataclass
class Workload:
    name: str
    x: torch.Tensor          # n x d float32, cuda (PCA-transformed)
    q: torch.Tensor          # nq x d float32, cuda (PCA-transformed)
    centroids: torch.Tensor  # k x d float32, cuda
    cids: torch.Tensor       # n int64, cuda
    variance: np.ndarray     # d float32 (column variance of x)
    sizes: np.ndarray        # k cluster sizes


def _spectrum(d, alpha, dev):
    return torch.arange(1, d + 1, device=dev, dtype=torch.float64).pow(-alpha / 2).float()


def zipf_aniso(n: int, d: int, k: int, nq: int, s: float = 1.1, alpha: float = 0.8, sigma: float = 0.2,
               noise_alpha: float | None = None, seed: int = 0, device: str = "cuda",
               chunk: int = 1 << 20, query_clusters: str = "zipf") -> Workload:
    """Zipf-sized clusters of unit-norm vectors.  Centres follow the per-axis
    spectrum i^-alpha; the within-cluster noise follows i^-noise_alpha
    (default: the same spectrum).  Queries pick their cluster with the Zipf
    weights ("zipf") or uniformly ("uniform")."""
    torch.backends.cuda.matmul.allow_tf32 = False
    dev = torch.device(device)
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    q_, r_ = np.linalg.qr(rng.standard_normal((d, d)))
    basis = torch.as_tensor((q_ * np.sign(np.diag(r_))[None, :]).astype(np.float32), device=dev)
    scale = _spectrum(d, alpha, dev)
    nscale = _spectrum(d, alpha if noise_alpha is None else noise_alpha, dev)
    nscale = nscale * (scale.norm() / nscale.norm())
    centers = (torch.randn(k, d, generator=g, device=dev) * scale) @ basis.T
    centers = centers / centers.norm(dim=1, keepdim=True)
    sizes = zipf_sizes(n, k, s)
    labels = torch.repeat_interleave(torch.arange(k, device=dev), torch.as_tensor(sizes, device=dev))
    labels = labels[torch.randperm(n, generator=g, device=dev)]

    def draw(lab):
        out = torch.empty(lab.numel(), d, device=dev)
        for a in range(0, lab.numel(), chunk):
            b = min(lab.numel(), a + chunk)
            z = (torch.randn(b - a, d, generator=g, device=dev) * nscale) @ basis.T
            v = centers[lab[a:b]] + sigma * z
            out[a:b] = v / v.norm(dim=1, keepdim=True)
        return out

    x = draw(labels)
    w = torch.as_tensor(sizes / sizes.sum() if query_clusters == "zipf" else np.full(k, 1.0 / k), device=dev,
                        dtype=torch.float32)
    qlab = torch.multinomial(w, nq, replacement=True, generator=g)
    q = draw(qlab)
    # PCA (python/pca.py): covariance of a sample in FP32 GEMMs, eigendecomposition on the host in FP64
    samp = x[torch.randperm(n, generator=g, device=dev)[: min(n, 1 << 20)]]
    mean = samp.mean(0)
    xc = samp - mean
    cov = (xc.T @ xc / samp.shape[0]).double().cpu().numpy()
    evals, evecs = np.linalg.eigh(cov)
    comp = torch.as_tensor(evecs[:, np.argsort(-evals, kind="stable")].T.astype(np.float32), device=dev)
    del samp, xc
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        x[a:b] = (x[a:b] - mean) @ comp.T
    q = (q - mean) @ comp.T
    # IVF centroids: the generating centres in PCA coordinates
    cent = ((centers - mean) @ comp.T).contiguous()
    colsum = torch.zeros(d, device=dev, dtype=torch.float64)
    sumsq = torch.zeros(d, device=dev, dtype=torch.float64)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        colsum += x[a:b].sum(0, dtype=torch.float64)
        sumsq += (x[a:b] * x[a:b]).sum(0, dtype=torch.float64)
    var = (sumsq / n - (colsum / n) ** 2).float().cpu().numpy()
    return Workload(f"zipf_aniso_{n}x{d}_k{k}", x, q.contiguous(), cent, labels, var, sizes)


@torch.no_grad()
def kmeans(x: torch.Tensor, k: int, iters: int, seed: int = 0, chunk: int = 1 << 18):
    """Lloyd's k-means (L2) on the device, the role faiss plays in the reference's
    python/ivf.py: seeded by k distinct points, `iters` updates (FP64 sums, empty
    clusters keep their centre), then every point assigned to its nearest centre.
    Returns (centroids k x d float32, cluster id per point int64)."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n, d = x.shape
    g = torch.Generator(device=x.device)
    g.manual_seed(seed)
    cent = x[torch.randperm(n, generator=g, device=x.device)[:k]].clone()
    assign = torch.empty(n, dtype=torch.int64, device=x.device)

    def nearest():
        cn = (cent * cent).sum(1)
        for a in range(0, n, chunk):
            b = min(n, a + chunk)
            assign[a:b] = torch.argmin(cn[None, :] - 2.0 * x[a:b] @ cent.T, dim=1)
    for _ in range(iters):
        nearest()
        sums = torch.zeros(k, d, dtype=torch.float64, device=x.device)
        for a in range(0, n, chunk):
            b = min(n, a + chunk)
            sums.index_add_(0, assign[a:b], x[a:b].double())
        cnt = torch.bincount(assign, minlength=k)
        nz = cnt > 0
        cent[nz] = (sums[nz] / cnt[nz, None]).float()
    nearest()
    return cent.contiguous(), assign


def _pca(x: torch.Tensor, q: torch.Tensor, g: torch.Generator, chunk: int = 1 << 20):
    """Mean-centred full-rank PCA (python/pca.py): covariance of (a sample of) the
    base set, components by descending eigenvalue, applied in place to x and q."""
    n = x.shape[0]
    samp = x[torch.randperm(n, generator=g, device=x.device)[: min(n, 1 << 20)]]
    mean = samp.mean(0)
    xc = samp - mean
    cov = (xc.T @ xc / samp.shape[0]).double().cpu().numpy()
    evals, evecs = np.linalg.eigh(cov)
    comp = torch.as_tensor(evecs[:, np.argsort(-evals, kind="stable")].T.astype(np.float32), device=x.device)
    del samp, xc
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        x[a:b] = (x[a:b] - mean) @ comp.T
    return (q - mean) @ comp.T


def _column_variance(x: torch.Tensor, chunk: int = 1 << 20) -> np.ndarray:
    n, d = x.shape
    colsum = torch.zeros(d, device=x.device, dtype=torch.float64)
    sumsq = torch.zeros(d, device=x.device, dtype=torch.float64)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        colsum += x[a:b].sum(0, dtype=torch.float64)
        sumsq += (x[a:b].double() ** 2).sum(0)
    return (sumsq / n - (colsum / n) ** 2).float().cpu().numpy()


@torch.no_grad()
def gaussian_mixture_ivf(n: int = 100_000, d: int = 960, centers: int = 1024, sigma: float = 0.5, nq: int = 1000,
                         k: int = 1024, iters: int = 20, seed: int = 0, device: str = "cuda") -> Workload:
    """Gaussian mixture: centres ~ N(0,1)^d, point = centre + N(0, sigma^2) per
    coordinate, queries from the same mixture; PCA over the base set; k-means
    with k clusters for `iters` iterations gives the IVF centroids and ids."""
    torch.backends.cuda.matmul.allow_tf32 = False
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    ctr = torch.randn(centers, d, generator=g, device=dev)
    lab = torch.randint(0, centers, (n,), generator=g, device=dev)
    x = ctr[lab] + sigma * torch.randn(n, d, generator=g, device=dev)
    ql = torch.randint(0, centers, (nq,), generator=g, device=dev)
    q = ctr[ql] + sigma * torch.randn(nq, d, generator=g, device=dev)
    q = _pca(x, q, g)
    cent, cids = kmeans(x, k, iters, seed=seed + 1)
    sizes = torch.bincount(cids, minlength=k).cpu().numpy()
    return Workload(f"gmix_{n}x{d}_k{k}", x, q.contiguous(), cent, cids, _column_variance(x), sizes)


@torch.no_grad()
def aniso_ivf(n: int = 1_000_000, d: int = 1024, alpha: float = 0.8, nq: int = 10_000, k: int = 4096,
              iters: int = 10, seed: int = 0, device: str = "cuda", chunk: int = 1 << 20) -> Workload:
    """Unit-norm rows with per-axis variance ~ i^-alpha in a random orthogonal
    basis (queries from the same distribution); PCA; k-means with k clusters."""
    torch.backends.cuda.matmul.allow_tf32 = False
    dev = torch.device(device)
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    q_, r_ = np.linalg.qr(rng.standard_normal((d, d)))
    basis = torch.as_tensor((q_ * np.sign(np.diag(r_))[None, :]).astype(np.float32), device=dev)
    scale = _spectrum(d, alpha, dev)

    def draw(m):
        out = torch.empty(m, d, device=dev)
        for a in range(0, m, chunk):
            b = min(m, a + chunk)
            v = (torch.randn(b - a, d, generator=g, device=dev) * scale) @ basis.T
            out[a:b] = v / v.norm(dim=1, keepdim=True)
        return out
    x = draw(n)
    q = _pca(x, draw(nq), g)
    cent, cids = kmeans(x, k, iters, seed=seed + 1)
    sizes = torch.bincount(cids, minlength=k).cpu().numpy()
    return Workload(f"aniso_{n}x{d}_k{k}", x, q.contiguous(), cent, cids, _column_variance(x), sizes)


def rotations(plan, seed: int) -> np.ndarray:
    """Random orthogonal matrices (numpy, seeded), one per segment of `plan`,
    concatenated row-major: the rotations both builders are given, so that the
    GPU builder and the CPU oracle write the same index."""
    rng = np.random.default_rng(seed)
    mats = []
    for dim, _ in plan:
        a = rng.standard_normal((dim, dim))
        q_, r_ = np.linalg.qr(a)
        mats.append((q_ * np.sign(np.diag(r_))[None, :]).astype(np.float32).reshape(-1))
    return np.concatenate(mats)


@torch.no_grad()
def ground_truth(x: torch.Tensor, q: torch.Tensor, k: int, shortlist: int = 200, chunk: int = 1 << 21):
    """Exact FP64 top-k (L2) for each query: FP32 shortlist, FP64 re-rank."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = x.shape[0]
    best_d = torch.full((q.shape[0], shortlist), math.inf, device=q.device)
    best_i = torch.zeros((q.shape[0], shortlist), dtype=torch.int64, device=q.device)
    qn = (q * q).sum(1, keepdim=True)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        xb = x[a:b]
        d = qn - 2.0 * q @ xb.T + (xb * xb).sum(1)[None, :]
        vals, idx = torch.topk(d, min(shortlist, b - a), dim=1, largest=False)
        cat_d = torch.cat([best_d, vals], 1)
        cat_i = torch.cat([best_i, idx + a], 1)
        o = torch.topk(cat_d, shortlist, dim=1, largest=False).indices
        best_d = torch.gather(cat_d, 1, o)
        best_i = torch.gather(cat_i, 1, o)
    cand = x[best_i.reshape(-1)].double().reshape(q.shape[0], shortlist, -1)
    d64 = ((cand - q.double()[:, None, :]) ** 2).sum(-1)
    order = torch.argsort(d64, dim=1, stable=True)[:, :k]
    return torch.gather(best_i, 1, order).cpu().numpy()


def recall_at(found: np.ndarray, gt: np.ndarray, k: int) -> float:
    hit = 0
    for f, g_ in zip(found, gt):
        hit += len(set(f[:k].tolist()) & set(g_[:k].tolist()))
    return hit / (k * len(gt))
