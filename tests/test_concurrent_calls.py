"""Concurrent searches on one index (the reference's drivers call IVF::search
from a thread pool, src/test_qps.cpp:77-84): calls from several host threads,
each on its own stream, run on contexts leased from the index's pool and must
return exactly what the same calls return one after another."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _index_and_queries():
    from saq_gb300 import data, ivf
    x, q = data.gaussian_mixture(20000, 128, 200, sigma=0.6, seed=3, n_query=96)
    cent, cids = data.kmeans(x, 64, iters=5, seed=1)
    index = ivf.IVF(x.shape[0], 128, 64, ivf.QuantizeConfig(avg_bits=4.0))
    index.construct(x, cent, cids, seed=2)
    return index, q


@pytest.mark.parametrize("mem", ["host", "device"])
def test_threads_on_their_own_streams_match_sequential(mem):
    import torch
    index, q = _index_and_queries()
    want_ids, want_d = index.search(q, 10, 8, return_dists=True)
    nthreads, per = 8, q.shape[0] // 8
    got_ids = np.zeros_like(want_ids)
    got_d = np.zeros_like(want_d)
    errors = []

    def worker(t):
        try:
            st = torch.cuda.Stream()
            for rep in range(3):
                for i in range(t * per, (t + 1) * per):
                    if mem == "host":
                        ids, d = index.search(q[i], 10, 8, return_dists=True, stream=st)
                    else:
                        with torch.cuda.stream(st):
                            qd = torch.from_numpy(q[i:i + 1]).cuda(non_blocking=False)
                        ids_t, d_t = index.search(qd, 10, 8, return_dists=True, stream=st)
                        st.synchronize()
                        ids, d = ids_t.cpu().numpy()[0].view(np.uint32), d_t.cpu().numpy()[0]
                    got_ids[i], got_d[i] = ids, d
        except Exception as e:  # surfaced in the main thread
            errors.append(e)
    th = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    assert np.array_equal(got_ids, want_ids)
    assert np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32))
