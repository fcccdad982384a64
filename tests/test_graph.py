"""Graph-captured search: a launch of the captured graph returns exactly what
saqg_search returns for the queries currently in the bound buffer."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from saq_gb300 import data

pytestmark = pytest.mark.gpu


def _direct(index, q, topk, nprobe):
    import torch
    from saq_gb300 import _native as N, ivf
    ids = torch.empty((q.shape[0], topk), dtype=torch.int32, device="cuda")
    d = torch.empty((q.shape[0], topk), dtype=torch.float32, device="cuda")
    cfg = ivf.SearcherConfig().to_c()
    N.check(index.lib.saqg_search(index._h, q.data_ptr(), q.shape[0], topk, nprobe, C.byref(cfg), ids.data_ptr(),
                                  d.data_ptr(), N.SAQG_MEM_DEVICE, None))
    torch.cuda.synchronize()
    return ids.cpu().numpy(), d.cpu().numpy()


def _check_graph(index, qpool, nq, topk, nprobe):
    import torch
    from saq_gb300 import _native as N, ivf
    q = torch.from_numpy(np.ascontiguousarray(qpool[:nq])).cuda()
    ids = torch.empty((nq, topk), dtype=torch.int32, device="cuda")
    d = torch.empty((nq, topk), dtype=torch.float32, device="cuda")
    cfg = ivf.SearcherConfig().to_c()
    g = C.c_void_p()
    N.check(index.lib.saqg_search_graph_create(index._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), ids.data_ptr(),
                                               d.data_ptr(), None, C.byref(g)))
    try:
        for rnd in range(3):
            src = qpool[(rnd * nq) % max(1, qpool.shape[0] - nq):][:nq]
            q.copy_(torch.from_numpy(np.ascontiguousarray(src)).cuda())
            N.check(index.lib.saqg_search_graph_launch(g, None))
            torch.cuda.synchronize()
            want_ids, want_d = _direct(index, q, topk, nprobe)
            assert np.array_equal(ids.cpu().numpy(), want_ids), rnd
            assert np.array_equal(d.cpu().numpy().view(np.uint32), want_d.view(np.uint32)), rnd
    finally:
        N.check(index.lib.saqg_search_graph_free(g))


def test_graph_single_query_and_small_batch(golden_case):
    from saq_gb300 import ivf
    index = ivf.IVF.load(golden_case.index_path)
    qpool = np.concatenate([golden_case.q] * 4)
    _check_graph(index, qpool, 1, golden_case.topk, golden_case.nprobe)
    _check_graph(index, qpool, min(8, golden_case.q.shape[0]), golden_case.topk, golden_case.nprobe)


@pytest.mark.parametrize("defer", ["1", "1024"])
def test_graph_batch_with_shortlist_and_split_pass(defer, monkeypatch):
    from saq_gb300 import ivf
    monkeypatch.setenv("SAQG_DEFER_BLOCKS", defer)  # "1": every query through the split pass beside k_scan
    x, q = data.gaussian_mixture(12000, 128, 300, sigma=0.6, seed=6, n_query=300)
    cent, cids = data.kmeans(x, 160, iters=6, seed=2)
    index = ivf.IVF(x.shape[0], 128, 160, ivf.QuantizeConfig(avg_bits=4.0))
    index.construct(x, cent, cids, seed=5)
    _check_graph(index, q, 96, 10, 16)


def _mixture_index(tc=False):
    from saq_gb300 import ivf
    x, q = data.gaussian_mixture(12000, 128, 300, sigma=0.6, seed=6, n_query=300)
    cent, cids = data.kmeans(x, 160, iters=6, seed=2)
    index = ivf.IVF(x.shape[0], 128, 160, ivf.QuantizeConfig(avg_bits=6.0 if tc else 4.0,
                                                             enable_segmentation=not tc))
    index.construct(x, cent, cids, seed=5)
    return index, q


def test_autotune_keeps_the_answers():
    """The autotuner times every candidate shape, keeps the fastest, and later
    calls of that shape (which use it) return exactly what they returned before."""
    import torch
    from saq_gb300 import _native as N, ivf
    index, q = _mixture_index()
    qd = torch.from_numpy(np.ascontiguousarray(q[:128])).cuda()
    want_ids, want_d = _direct(index, qd, 10, 16)
    rep = N.TuneReport()
    cfg = ivf.SearcherConfig().to_c()
    N.check(index.lib.saqg_autotune(index._h, qd.data_ptr(), 128, 10, 16, 0, N.SAQG_FORM_EXACT, C.byref(cfg), None,
                                    C.byref(rep)))
    assert rep.form == N.SAQG_FORM_EXACT and rep.candidates >= 8
    assert 0 < rep.tuned_ms <= rep.default_ms
    ids, d = _direct(index, qd, 10, 16)
    assert np.array_equal(ids, want_ids)
    assert np.array_equal(d.view(np.uint32), want_d.view(np.uint32))


def _graph_ex(index, q, nq, topk, nprobe, form, npq=None, kq=None, shortlist=0, cap=0, autotune=0):
    import torch
    from saq_gb300 import _native as N, ivf
    ids = torch.empty((nq, topk), dtype=torch.int32, device="cuda")
    d = torch.empty((nq, topk), dtype=torch.float32, device="cuda")
    gc = N.GraphConfig(form, npq.data_ptr() if npq is not None else None, kq.data_ptr() if kq is not None else None,
                       shortlist, cap, autotune)
    cfg = ivf.SearcherConfig().to_c()
    g = C.c_void_p()
    rep = N.TuneReport()
    N.check(index.lib.saqg_search_graph_create_ex(index._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), C.byref(gc),
                                                  ids.data_ptr(), d.data_ptr(), None, C.byref(g), C.byref(rep)))
    return g, ids, d, rep


def test_graph_exact_form_uneven_nprobe_and_topk():
    """Per-query nprobe / topk in device arrays, rewritten between launches: each
    launch equals saqg_search_batch with the same arrays (rows padded past a
    query's own topk with id 0 / FLT_MAX)."""
    import torch
    from saq_gb300 import _native as N, ivf
    index, qpool = _mixture_index()
    nq, kmax, npmax = 64, 20, 32
    rng = np.random.default_rng(4)
    q = torch.from_numpy(np.ascontiguousarray(qpool[:nq])).cuda()
    npq = torch.full((nq,), npmax, dtype=torch.int32, device="cuda")
    kq = torch.full((nq,), kmax, dtype=torch.int32, device="cuda")
    g, ids, d, _ = _graph_ex(index, q, nq, kmax, npmax, N.SAQG_FORM_EXACT, npq, kq, autotune=1)
    try:
        for rnd in range(3):
            nps = rng.integers(1, npmax + 1, size=nq).astype(np.int32)
            ks = rng.choice([1, 10, 20], size=nq).astype(np.int32)
            npq.copy_(torch.from_numpy(nps))
            kq.copy_(torch.from_numpy(ks))
            q.copy_(torch.from_numpy(np.ascontiguousarray(qpool[nq * (rnd + 1):nq * (rnd + 2)])))
            N.check(index.lib.saqg_search_graph_launch(g, None))
            N.check(index.lib.saqg_search_graph_status(g, None))
            torch.cuda.synchronize()
            wi = torch.empty((nq, kmax), dtype=torch.int32, device="cuda")
            wd = torch.empty((nq, kmax), dtype=torch.float32, device="cuda")
            cfg = ivf.SearcherConfig().to_c()
            N.check(index.lib.saqg_search_batch(index._h, q.data_ptr(), nq, nps.ctypes.data, ks.ctypes.data, npmax,
                                                kmax, C.byref(cfg), wi.data_ptr(), wd.data_ptr(), N.SAQG_MEM_DEVICE,
                                                None, None))
            torch.cuda.synchronize()
            assert np.array_equal(ids.cpu().numpy(), wi.cpu().numpy()), rnd
            assert np.array_equal(d.cpu().numpy().view(np.uint32), wd.cpu().numpy().view(np.uint32)), rnd
    finally:
        N.check(index.lib.saqg_search_graph_free(g))


@pytest.mark.parametrize("uneven", [False, True])
def test_graph_tensor_core_form(uneven):
    """The tensor-core form captured with a candidate capacity: each launch equals
    a direct saqg_search_tc / saqg_search_tc_batch call on the same inputs."""
    import torch
    from saq_gb300 import _native as N, ivf
    index, qpool = _mixture_index(tc=True)
    nq, kmax, npmax, L = 48, 10, 24, 40
    rng = np.random.default_rng(9)
    q = torch.from_numpy(np.ascontiguousarray(qpool[:nq])).cuda()
    npq = torch.full((nq,), npmax, dtype=torch.int32, device="cuda") if uneven else None
    kq = torch.full((nq,), kmax, dtype=torch.int32, device="cuda") if uneven else None
    g, ids, d, rep = _graph_ex(index, q, nq, kmax, npmax, N.SAQG_FORM_TC, npq, kq, shortlist=L, autotune=1)
    assert rep.candidates >= 1
    cfg = ivf.SearcherConfig().to_c()
    try:
        for rnd in range(3):
            q.copy_(torch.from_numpy(np.ascontiguousarray(qpool[nq * (rnd + 1):nq * (rnd + 2)])))
            nps = rng.integers(1, npmax + 1, size=nq).astype(np.int32)
            ks = rng.choice([1, 5, 10], size=nq).astype(np.int32)
            if uneven:
                npq.copy_(torch.from_numpy(nps))
                kq.copy_(torch.from_numpy(ks))
            N.check(index.lib.saqg_search_graph_launch(g, None))
            N.check(index.lib.saqg_search_graph_status(g, None))
            got_i, got_d = ids.cpu().numpy().copy(), d.cpu().numpy().copy()
            wi = torch.empty((nq, kmax), dtype=torch.int32, device="cuda")
            wd = torch.empty((nq, kmax), dtype=torch.float32, device="cuda")
            if uneven:
                N.check(index.lib.saqg_search_tc_batch(index._h, q.data_ptr(), nq, nps.ctypes.data, ks.ctypes.data,
                                                       npmax, kmax, L, C.byref(cfg), wi.data_ptr(), wd.data_ptr(),
                                                       None, N.SAQG_MEM_DEVICE, None, None))
            else:
                N.check(index.lib.saqg_search_tc(index._h, q.data_ptr(), nq, kmax, npmax, L, C.byref(cfg),
                                                 wi.data_ptr(), wd.data_ptr(), None, N.SAQG_MEM_DEVICE, None, None))
            torch.cuda.synchronize()
            assert np.array_equal(got_i, wi.cpu().numpy()), rnd
            assert np.array_equal(got_d.view(np.uint32), wd.cpu().numpy().view(np.uint32)), rnd
    finally:
        N.check(index.lib.saqg_search_graph_free(g))


def test_graph_tensor_core_capacity_overflow_is_reported():
    """A launch whose batch needs more approximate distances than the graph's
    capacity writes nothing past its arrays and reports SAQG_ERR_NOMEM; a graph
    with room answers the same batch."""
    import torch
    from saq_gb300 import _native as N
    index, qpool = _mixture_index(tc=True)
    nq = 32
    q = torch.from_numpy(np.ascontiguousarray(qpool[:nq])).cuda()
    g, ids, d, _ = _graph_ex(index, q, nq, 10, 24, N.SAQG_FORM_TC, shortlist=40, cap=1000)
    try:
        N.check(index.lib.saqg_search_graph_launch(g, None))
        assert index.lib.saqg_search_graph_status(g, None) == 4  # SAQG_ERR_NOMEM
        assert b"capacity" in index.lib.saqg_last_error()
    finally:
        N.check(index.lib.saqg_search_graph_free(g))
    g, ids, d, _ = _graph_ex(index, q, nq, 10, 24, N.SAQG_FORM_TC, shortlist=40)
    try:
        N.check(index.lib.saqg_search_graph_launch(g, None))
        N.check(index.lib.saqg_search_graph_status(g, None))
    finally:
        N.check(index.lib.saqg_search_graph_free(g))
