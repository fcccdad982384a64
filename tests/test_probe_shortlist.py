"""Centroid ranking of batches through the GEMM shortlist.

Batches of at least 64 queries rank centroids from TF32 inner products plus an
error bound and evaluate the exact distance only on the shortlist; queries with
ties fall back to the full exact ranking.  Either way the probes, and hence
the search results, must equal the oracle's bit for bit (no tolerance).
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from saq_gb300 import data

pytestmark = pytest.mark.gpu


def _build(x, cent, cids, tmp_path, bits=4.0):
    from saq_gb300 import ivf
    rng = np.random.default_rng(11)
    var = O.colwise_var(x)
    plan = O.plan(var, bits, True, 0)
    rots = np.concatenate([data.random_orthogonal(d, rng).astype(np.float32).reshape(-1) for d, _ in plan])
    index = ivf.IVF(x.shape[0], x.shape[1], cent.shape[0], ivf.QuantizeConfig(avg_bits=bits))
    index.construct(x, cent, cids, rotations=rots)
    opath = str(tmp_path / "o.index")
    O.build_index(opath, x, cent, cids, bits, True, 0, rots)
    return index, O.OracleIndex(opath)


def _search_stats(index, q, topk, nprobe):
    from saq_gb300 import _native as N, ivf
    q = np.ascontiguousarray(q, np.float32)
    nq = q.shape[0]
    ids = np.zeros((nq, topk), np.uint32)
    d = np.zeros((nq, topk), np.float32)
    probes = np.zeros((nq, nprobe), np.uint32)
    st = N.SearchStats()
    cfg = ivf.SearcherConfig().to_c()
    N.check(index.lib.saqg_search_ex(index._h, q.ctypes.data, nq, topk, nprobe, C.byref(cfg), ids.ctypes.data,
                                     d.ctypes.data, N.SAQG_MEM_HOST, None, C.byref(st), probes.ctypes.data))
    return ids, d, probes, st


@pytest.mark.parametrize("dim,nc", [(128, 256), (192, 300), (256, 512)])
def test_shortlist_ranking_is_exact(dim, nc, tmp_path, monkeypatch):
    x, q = data.gaussian_mixture(12000, dim, 400, sigma=0.6, seed=4, n_query=160)
    cent, cids = data.kmeans(x, nc, iters=6, seed=1)
    index, oi = _build(x, cent, cids, tmp_path)
    topk, nprobe = 10, 16
    ids, d, probes, st = _search_stats(index, q, topk, nprobe)
    assert 0 < st.probe_exact < q.shape[0] * nc  # the shortlist served (most of) the batch
    oids, od = oi.search(q, topk, nprobe, with_dists=True)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    monkeypatch.setenv("SAQG_PROBE", "exact")
    ids2, d2, probes2, st2 = _search_stats(index, q, topk, nprobe)
    assert st2.probe_exact == q.shape[0] * nc
    assert np.array_equal(probes, probes2)
    assert np.array_equal(ids, ids2)


def test_shortlist_falls_back_on_ties(tmp_path):
    # integer data with constant-row centroids that repeat: exact distance ties
    x, q, cent, cids = data.int_grid(6000, 96, 64, num_centroids=40, seed=3)
    index, oi = _build(x, cent, cids, tmp_path)
    topk, nprobe = 20, 12
    ids, d, probes, st = _search_stats(index, q, topk, nprobe)
    oids, od = oi.search(q, topk, nprobe, with_dists=True)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    assert st.probe_exact >= 40  # at least one query took the full exact ranking
