"""Python mirror of the reference's IVF API (index/ivf.hpp) over the C ABI.

    ivf = IVF(n, num_dim, k, QuantizeConfig(...))      # IVF(n, dim, k, cfg)
    ivf.set_variance(vars)                              # IVF::set_variance
    ivf.construct(data, centroids, cluster_ids)         # IVF::construct
    ivf.save(path) / IVF.load(path)                     # IVF::save / IVF::load
    ids = ivf.search(query, topk, nprobe, SearcherConfig())   # IVF::search<L2Sqr>
    dist_list, fast, vars = ivf.estimate(query, nprobe)       # IVF::estimate<L2Sqr>

`search` accepts one query (the reference's signature) or a batch (nq x dim),
each answered exactly as an independent reference call.  Inputs may be numpy
arrays (host memory; the copies are part of the call) or CUDA torch tensors
(device memory, used in place).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N


@dataclass
class QuantizeConfig:
    """quantization/config.h:21-74 (QuantizeConfig with its QuantSingleConfig)."""
    avg_bits: float = 0.0
    seg_eqseg: int = 0
    enable_segmentation: bool = True
    use_compact_layout: bool = False
    random_rotation: bool = True
    caq_adj_rd_lmt: int = 6
    caq_adj_eps: float = 1e-8

    def to_c(self):
        return N.QuantizeConfig(self.avg_bits, self.seg_eqseg, int(self.enable_segmentation),
                                int(self.use_compact_layout), int(self.random_rotation), self.caq_adj_rd_lmt,
                                self.caq_adj_eps)


@dataclass
class SearcherConfig:
    """quantization/config.h:76-79."""
    searcher_vars_bound_m: float = 4.0
    dist_type: int = N.SAQG_DIST_L2

    def to_c(self):
        return N.SearcherConfig(self.searcher_vars_bound_m, self.dist_type)


def _is_cuda_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and bool(x.is_cuda)


def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(getattr(stream, "cuda_stream", stream))


class IVF:
    def __init__(self, n: int = 0, num_dim: int = 0, k: int = 0, cfg: QuantizeConfig | None = None):
        self.lib = N.load()
        self._h = C.c_void_p()
        self.num_data, self.num_dim, self.num_cen = n, num_dim, k
        self.cfg = cfg or QuantizeConfig()
        self._variance = None

    # -- lifecycle --------------------------------------------------------
    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.saqg_index_free(self._h)
            self._h = C.c_void_p()

    @classmethod
    def load(cls, path: str) -> "IVF":
        ivf = cls()
        N.check(ivf.lib.saqg_index_load(path.encode(), C.byref(ivf._h)))
        info = ivf.info()
        ivf.num_data, ivf.num_dim, ivf.num_cen = info["num_data"], info["num_dim"], info["num_clusters"]
        return ivf

    def save(self, path: str, format: str = "reference") -> None:
        """IVF::save in the reference's format, or format="v2" (checksummed device layout)."""
        if format == "v2":
            N.check(self.lib.saqg_index_save_v2(self._h, path.encode()))
        elif format == "reference":
            N.check(self.lib.saqg_index_save(self._h, path.encode()))
        else:
            raise ValueError(f"unknown index format {format!r}")

    def set_variance(self, vars_) -> None:
        self._variance = np.ascontiguousarray(vars_, np.float32).reshape(-1)

    def construct(self, data, centroids, cluster_ids, rotations=None, seed: int = 1) -> None:
        """IVF::construct.  `data` may be a numpy array or a CUDA torch tensor (used in place)."""
        if _is_cuda_tensor(data):
            data_t = data.contiguous()
            n, d = data_t.shape
            data_ptr, mem = data_t.data_ptr(), N.SAQG_MEM_DEVICE
        else:
            data_t = np.ascontiguousarray(data, np.float32)
            n, d = data_t.shape
            data_ptr, mem = data_t.ctypes.data, N.SAQG_MEM_HOST
        cent = np.ascontiguousarray(centroids, np.float32)
        cids = np.ascontiguousarray(cluster_ids, np.uint32).reshape(-1)
        if self._h.value:
            self.lib.saqg_index_free(self._h)
            self._h = C.c_void_p()
        cfg = self.cfg.to_c()
        rot = None if rotations is None else np.ascontiguousarray(rotations, np.float32)
        N.check(self.lib.saqg_index_construct(
            data_ptr, n, d, cent.ctypes.data, cent.shape[0], cids.ctypes.data, C.byref(cfg),
            None if self._variance is None else self._variance.ctypes.data,
            None if rot is None else rot.ctypes.data, seed, mem, C.byref(self._h)))
        self.num_data, self.num_dim, self.num_cen = n, d, cent.shape[0]

    def info(self) -> dict:
        inf = N.IndexInfo()
        N.check(self.lib.saqg_index_get_info(self._h, C.byref(inf)))
        S = inf.num_segments
        return dict(num_data=inf.num_data, num_dim=inf.num_dim, num_clusters=inf.num_clusters,
                    plan=[(inf.seg_dim[i], inf.seg_bits[i]) for i in range(S)], device_bytes=inf.device_bytes)

    # -- search -----------------------------------------------------------
    def search(self, query, topk, nprobe, searcher_cfg: SearcherConfig | None = None,
               return_dists: bool = False, out=None, stream=None):
        """IVF::search for one query or a batch.  `topk` / `nprobe` may be per-query
        sequences (rows are then max(topk) long, padded with id 0 / inf)."""
        cfg = (searcher_cfg or SearcherConfig()).to_c()
        if not (np.isscalar(topk) and np.isscalar(nprobe)):
            return self._search_mixed(query, topk, nprobe, cfg, return_dists, stream)
        if _is_cuda_tensor(query):
            import torch
            q = query.contiguous().view(-1, self.num_dim)
            nq = q.shape[0]
            ids, dists = out if out is not None else (
                torch.empty((nq, topk), dtype=torch.int32, device=q.device),
                torch.empty((nq, topk), dtype=torch.float32, device=q.device))
            N.check(self.lib.saqg_search(self._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), ids.data_ptr(),
                                         dists.data_ptr() if dists is not None else None, N.SAQG_MEM_DEVICE,
                                         _stream_ptr(stream)))
            return (ids, dists) if return_dists else ids
        q = np.ascontiguousarray(query, np.float32)
        single = q.ndim == 1
        q = q.reshape(-1, self.num_dim)
        nq = q.shape[0]
        ids = np.zeros((nq, topk), np.uint32)
        dists = np.zeros((nq, topk), np.float32)
        N.check(self.lib.saqg_search(self._h, q.ctypes.data, nq, topk, nprobe, C.byref(cfg), ids.ctypes.data,
                                     dists.ctypes.data, N.SAQG_MEM_HOST, _stream_ptr(stream)))
        if single:
            ids, dists = ids[0], dists[0]
        return (ids, dists) if return_dists else ids

    def _search_mixed(self, query, topk, nprobe, cfg, return_dists, stream):
        if _is_cuda_tensor(query):
            import torch
            q = query.contiguous().view(-1, self.num_dim)
            nq = q.shape[0]
        else:
            q = np.ascontiguousarray(query, np.float32).reshape(-1, self.num_dim)
            nq = q.shape[0]
        ks = np.broadcast_to(np.asarray(topk, np.int32), (nq,)).copy()
        nps = np.broadcast_to(np.asarray(nprobe, np.int32), (nq,)).copy()
        kmax = int(ks.max())
        if _is_cuda_tensor(query):
            ids = torch.empty((nq, kmax), dtype=torch.int32, device=q.device)
            dists = torch.empty((nq, kmax), dtype=torch.float32, device=q.device)
            N.check(self.lib.saqg_search_batch(self._h, q.data_ptr(), nq, nps.ctypes.data, ks.ctypes.data,
                                               int(nps.max()), kmax, C.byref(cfg), ids.data_ptr(), dists.data_ptr(),
                                               N.SAQG_MEM_DEVICE, _stream_ptr(stream), None))
        else:
            ids = np.zeros((nq, kmax), np.uint32)
            dists = np.zeros((nq, kmax), np.float32)
            N.check(self.lib.saqg_search_batch(self._h, q.ctypes.data, nq, nps.ctypes.data, ks.ctypes.data,
                                               int(nps.max()), kmax, C.byref(cfg), ids.ctypes.data, dists.ctypes.data,
                                               N.SAQG_MEM_HOST, _stream_ptr(stream), None))
        return (ids, dists) if return_dists else ids

    def search_tc(self, query, topk, nprobe, shortlist: int | None = None,
                  searcher_cfg: SearcherConfig | None = None, return_dists: bool = False,
                  return_approx: bool = False, stats: bool = False, stream=None):
        """Tensor-core form of a batched search (saqg_search_tc): the approximate
        distances of every probed vector come from one dense BF16 product per
        cluster on the tensor cores, the `shortlist` (default 4 * topk) smallest
        per query are re-ranked with the exact search's distance.  `topk` /
        `nprobe` may be per-query sequences (saqg_search_tc_batch; rows are then
        max(topk) long, padded with id 0 / FLT_MAX).  Returns ids [, dists]
        [, approx] [, stats dict]."""
        cfg = (searcher_cfg or SearcherConfig()).to_c()
        mixed = not (np.isscalar(topk) and np.isscalar(nprobe))
        st = N.TcStats()
        sp = C.byref(st) if stats else None
        if _is_cuda_tensor(query):
            import torch
            q = query.contiguous().view(-1, self.num_dim)
            nq = q.shape[0]
        else:
            q = np.ascontiguousarray(query, np.float32).reshape(-1, self.num_dim)
            nq = q.shape[0]
        if mixed:
            ks = np.broadcast_to(np.asarray(topk, np.int32), (nq,)).copy()
            nps = np.broadcast_to(np.asarray(nprobe, np.int32), (nq,)).copy()
            kmax, npmax = int(ks.max()), int(nps.max())
        else:
            kmax, npmax = int(topk), int(nprobe)
        L = int(shortlist if shortlist is not None else 4 * kmax)
        if _is_cuda_tensor(query):
            ids = torch.empty((nq, kmax), dtype=torch.int32, device=q.device)
            dists = torch.empty((nq, kmax), dtype=torch.float32, device=q.device)
            apx = torch.empty((nq, kmax), dtype=torch.float32, device=q.device)
            qp, ip, dp, ap, mem = q.data_ptr(), ids.data_ptr(), dists.data_ptr(), apx.data_ptr(), N.SAQG_MEM_DEVICE
        else:
            ids = np.zeros((nq, kmax), np.uint32)
            dists = np.zeros((nq, kmax), np.float32)
            apx = np.zeros((nq, kmax), np.float32)
            qp, ip, dp, ap, mem = q.ctypes.data, ids.ctypes.data, dists.ctypes.data, apx.ctypes.data, N.SAQG_MEM_HOST
        if mixed:
            N.check(self.lib.saqg_search_tc_batch(self._h, qp, nq, nps.ctypes.data, ks.ctypes.data, npmax, kmax, L,
                                                  C.byref(cfg), ip, dp, ap, mem, _stream_ptr(stream), sp))
        else:
            N.check(self.lib.saqg_search_tc(self._h, qp, nq, kmax, npmax, L, C.byref(cfg), ip, dp, ap, mem,
                                            _stream_ptr(stream), sp))
        out = [ids]
        if return_dists:
            out.append(dists)
        if return_approx:
            out.append(apx)
        if stats:
            out.append(st.as_dict())
        return out[0] if len(out) == 1 else tuple(out)

    def estimate(self, query, nprobe: int, searcher_cfg: SearcherConfig | None = None):
        """IVF::estimate: ([(id, accurate)], fast list, vars list) for every vector of the probed clusters."""
        cfg = (searcher_cfg or SearcherConfig()).to_c()
        q = np.ascontiguousarray(query, np.float32).reshape(-1)
        cap = max(1, self.num_data)
        ids = np.zeros(cap, np.uint32)
        acc = np.zeros(cap, np.float32)
        fast = np.zeros(cap, np.float32)
        var = np.zeros(cap, np.float32)
        cnt = C.c_int64()
        N.check(self.lib.saqg_estimate(self._h, q.ctypes.data, nprobe, C.byref(cfg), ids.ctypes.data,
                                       acc.ctypes.data, fast.ctypes.data, var.ctypes.data, cap, C.byref(cnt)))
        n = cnt.value
        return ids[:n], acc[:n], fast[:n], var[:n]


class Server:
    """Serving loop with continuous batching over an IVF (saqg_server_*): queries
    submitted one by one, batched on the device as slots and memory free up."""

    def __init__(self, index: IVF, max_batch: int = 4096, max_inflight: int = 2, max_topk: int = 100,
                 max_nprobe: int = 0, max_wait_us: int = 200, mem_budget_bytes: int = 0,
                 searcher_cfg: SearcherConfig | None = None, form: str = "exact", shortlist: int = 0):
        """form "exact": batches answered as saqg_search_batch (every answer the
        reference's); "tc": as saqg_search_tc_batch with `shortlist` (0: 8 x max_topk)."""
        self.index = index
        self.lib = index.lib
        cfg = N.ServerConfig(max_batch, max_inflight, max_topk, max_nprobe, max_wait_us,
                             (searcher_cfg or SearcherConfig()).searcher_vars_bound_m, mem_budget_bytes,
                             {"exact": N.SAQG_FORM_EXACT, "tc": N.SAQG_FORM_TC}[form], shortlist)
        self._h = C.c_void_p()
        N.check(self.lib.saqg_server_create(index._h, C.byref(cfg), C.byref(self._h)))

    def submit(self, query, nprobe: int, topk: int) -> int:
        q = np.ascontiguousarray(query, np.float32).reshape(-1)
        t = C.c_uint64()
        N.check(self.lib.saqg_server_submit(self._h, q.ctypes.data, int(nprobe), int(topk), C.byref(t)))
        return t.value

    def wait(self, ticket: int, topk: int, timeout_ms: int = -1):
        ids = np.zeros(topk, np.uint32)
        d = np.zeros(topk, np.float32)
        lat = C.c_double()
        N.check(self.lib.saqg_server_wait(self._h, ticket, ids.ctypes.data, d.ctypes.data, C.byref(lat), timeout_ms))
        return ids, d, lat.value

    def run_trace(self, queries, arrival_s, nprobe, topk):
        """Open-loop load from native code: query i submitted at arrival_s[i] seconds."""
        q = np.ascontiguousarray(queries, np.float32)
        n = q.shape[0]
        arr = np.ascontiguousarray(arrival_s, np.float64)
        nps = np.ascontiguousarray(np.broadcast_to(nprobe, (n,)), np.int32)
        ks = np.ascontiguousarray(np.broadcast_to(topk, (n,)), np.int32)
        row = int(ks.max())
        ids = np.zeros((n, row), np.uint32)
        d = np.full((n, row), np.inf, np.float32)
        lat = np.zeros(n, np.float64)
        N.check(self.lib.saqg_server_run_trace(self._h, q.ctypes.data, n, arr.ctypes.data, nps.ctypes.data,
                                               ks.ctypes.data, row, ids.ctypes.data, d.ctypes.data, lat.ctypes.data))
        return ids, d, lat

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(self.lib.saqg_server_get_stats(self._h, C.byref(st)))
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            N.check(self.lib.saqg_server_free(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def convert(src: str, dst: str, format: str = "v2") -> None:
    """Host-only conversion of an index file to `format` ("v2" or "reference")."""
    lib = N.load()
    fmt = {"v2": N.SAQG_FORMAT_V2, "reference": N.SAQG_FORMAT_REFERENCE}[format]
    N.check(lib.saqg_index_convert(src.encode(), dst.encode(), fmt))


def plan(variance, avg_bits: float, enable_segmentation: bool = True, seg_eqseg: int = 0):
    """SaqDataMaker::analyze_plan through the C ABI (host computation)."""
    lib = N.load()
    v = np.ascontiguousarray(variance, np.float32).reshape(-1)
    dims = np.zeros(64, np.int64)
    bits = np.zeros(64, np.int64)
    ns = C.c_int()
    N.check(lib.saqg_plan(v.ctypes.data, v.size, avg_bits, int(enable_segmentation), seg_eqseg, dims.ctypes.data,
                          bits.ctypes.data, 64, C.byref(ns)))
    return [(int(dims[i]), int(bits[i])) for i in range(ns.value)]


def plan_gpu(variance, avg_bits: float, enable_segmentation: bool = True, seg_eqseg: int = 0, stream=None):
    """SaqDataMaker::analyze_plan with the dynamic program on the GPU (the same plan
    as `plan`).  `variance` is a numpy array or a CUDA tensor."""
    lib = N.load()
    if _is_cuda_tensor(variance):
        v = variance.contiguous().float()
        ptr, mem, size = v.data_ptr(), N.SAQG_MEM_DEVICE, v.numel()
    else:
        v = np.ascontiguousarray(variance, np.float32).reshape(-1)
        ptr, mem, size = v.ctypes.data, N.SAQG_MEM_HOST, v.size
    dims = np.zeros(64, np.int64)
    bits = np.zeros(64, np.int64)
    ns = C.c_int()
    N.check(lib.saqg_plan_gpu(ptr, size, avg_bits, int(enable_segmentation), seg_eqseg, mem, _stream_ptr(stream),
                              dims.ctypes.data, bits.ctypes.data, 64, C.byref(ns)))
    return [(int(dims[i]), int(bits[i])) for i in range(ns.value)]


def caq_encode(resid, bits: int, centroid=None, rd_lmt: int = 6, eps: float = 1e-8):
    """CAQEncoder::encode_and_fac on the GPU for n residual vectors (host arrays)."""
    lib = N.load()
    r = np.ascontiguousarray(resid, np.float32)
    n, d = r.shape
    codes = np.zeros((n, d), np.int32)
    facs = np.zeros((n, 4), np.float32)
    c = None if centroid is None else np.ascontiguousarray(centroid, np.float32)
    N.check(lib.saqg_caq_encode(r.ctypes.data, n, d, bits, None if c is None else c.ctypes.data, rd_lmt, eps,
                                codes.ctypes.data, facs.ctypes.data, N.SAQG_MEM_HOST, None))
    return codes, facs
