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
