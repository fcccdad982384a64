"""The serving loop (continuous batching): every answer equals the same query
searched alone through the single-query drop-in, bit for bit, whichever batch
it landed in; batches form and run side by side."""
import numpy as np
import pytest

from saq_gb300 import data

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def index_and_queries():
    from saq_gb300 import ivf
    x, q = data.gaussian_mixture(120000, 128, 600, sigma=0.6, seed=9, n_query=300)
    cent, cids = data.kmeans(x, 256, iters=4, seed=4)
    index = ivf.IVF(x.shape[0], 128, 256, ivf.QuantizeConfig(avg_bits=4.0))
    index.construct(x, cent, cids, seed=3)
    return index, q


def _alone(index, q, k, npb):
    ids, d = index.search(q, int(k), int(npb), return_dists=True)
    return ids, d


def test_served_answers_equal_alone(index_and_queries):
    from saq_gb300 import ivf
    index, q = index_and_queries
    rng = np.random.default_rng(1)
    n = 300
    nps = rng.integers(8, 129, size=n).astype(np.int32)
    ks = rng.choice([10, 100], size=n).astype(np.int32)
    srv = ivf.Server(index, max_batch=48, max_inflight=2, max_topk=100, max_nprobe=256, max_wait_us=500)
    try:
        # a burst (all at once) then a paced tail
        arrival = np.concatenate([np.zeros(200), 0.002 + 0.0002 * np.arange(100)])
        ids, d, lat = srv.run_trace(q[:n], arrival, nps, ks)
        st = srv.stats()
    finally:
        srv.close()
    for i in range(n):
        aid, ad = _alone(index, q[i], ks[i], nps[i])
        assert np.array_equal(ids[i, :ks[i]], aid), i
        assert np.array_equal(d[i, :ks[i]].view(np.uint32), ad.view(np.uint32)), i
    assert st["completed"] == n and st["submitted"] == n
    assert st["batches"] < n and st["max_batch_seen"] > 1  # queries were batched
    assert st["max_inflight_seen"] == 2                     # and batches overlapped on the device
    assert np.all(lat > 0) and st["p99_ms"] >= st["p50_ms"] > 0


def test_submit_wait_and_admission_by_memory(index_and_queries):
    from saq_gb300 import ivf
    index, q = index_and_queries
    # a budget too small for two 48-query batches forces smaller ones
    srv = ivf.Server(index, max_batch=48, max_inflight=2, max_topk=10, max_nprobe=32, max_wait_us=0,
                     mem_budget_bytes=64 << 20)
    try:
        tickets = [srv.submit(q[i], 16, 10) for i in range(40)]
        got = [srv.wait(t, 10, timeout_ms=20000) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    for i, (ids, d, lat) in enumerate(got):
        aid, ad = _alone(index, q[i], 10, 16)
        assert np.array_equal(ids, aid)
        assert np.array_equal(d.view(np.uint32), ad.view(np.uint32))
    assert st["completed"] == 40


@pytest.fixture(scope="module")
def coded_index_and_queries():
    """An index whose every segment is coded (the tensor-core form needs it)."""
    from saq_gb300 import ivf
    x, q = data.gaussian_mixture(60000, 128, 400, sigma=0.6, seed=12, n_query=200)
    cent, cids = data.kmeans(x, 192, iters=4, seed=5)
    index = ivf.IVF(x.shape[0], 128, 192, ivf.QuantizeConfig(avg_bits=6.0, enable_segmentation=False))
    index.construct(x, cent, cids, seed=6)
    return index, q


def test_served_tensor_core_answers_equal_alone(coded_index_and_queries):
    """Tensor-core serving: every answer equals the same query searched alone by
    saqg_search_tc with the server's shortlist, bit for bit, whichever batch it
    landed in."""
    from saq_gb300 import ivf
    index, q = coded_index_and_queries
    rng = np.random.default_rng(2)
    n, L = 200, 200
    nps = rng.integers(4, 65, size=n).astype(np.int32)
    ks = rng.choice([10, 100], size=n).astype(np.int32)
    srv = ivf.Server(index, max_batch=40, max_inflight=2, max_topk=100, max_nprobe=64, max_wait_us=500, form="tc",
                     shortlist=L)
    try:
        arrival = np.concatenate([np.zeros(120), 0.002 + 0.0003 * np.arange(80)])
        ids, d, lat = srv.run_trace(q[:n], arrival, nps, ks)
        st = srv.stats()
    finally:
        srv.close()
    for i in range(n):
        aid, ad = index.search_tc(q[i], int(ks[i]), int(nps[i]), shortlist=L, return_dists=True)
        assert np.array_equal(ids[i, :ks[i]], aid[0]), i
        assert np.array_equal(d[i, :ks[i]].view(np.uint32), ad[0].view(np.uint32)), i
    assert st["completed"] == n and st["batches"] < n and st["max_batch_seen"] > 1
