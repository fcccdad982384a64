"""Edge cases against the oracle, bit for bit: empty clusters, topk beyond the
vectors probed (a pool that never fills: ids 0 / FLT_MAX), nprobe = every
cluster, topk = 1, one cluster, and no queries; in every scan form and through
the batch (shortlist) path."""
import numpy as np
import pytest

import oracle as O
from saq_gb300 import data

pytestmark = pytest.mark.gpu


def _build(x, cent, cids, tmp_path, bits=4.0, seg=True):
    from saq_gb300 import ivf
    rng = np.random.default_rng(21)
    plan = O.plan(O.colwise_var(x), bits, seg, 0)
    rots = np.concatenate([data.random_orthogonal(d, rng).astype(np.float32).reshape(-1) for d, _ in plan])
    index = ivf.IVF(x.shape[0], x.shape[1], cent.shape[0],
                    ivf.QuantizeConfig(avg_bits=bits, enable_segmentation=seg))
    index.construct(x, cent, cids, rotations=rots)
    opath = str(tmp_path / "o.index")
    O.build_index(opath, x, cent, cids, bits, seg, 0, rots)
    return index, O.OracleIndex(opath)


@pytest.fixture(scope="module")
def with_empty(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("edge")
    x, q = data.gaussian_mixture(3000, 128, 40, sigma=0.6, seed=13, n_query=80)
    cent, cids = data.kmeans(x, 10, iters=5, seed=5)
    far = np.full((2, 128), 50.0, np.float32)  # two clusters nobody is assigned to
    far[1] *= -1
    cent = np.concatenate([cent, far])
    return _build(x, cent, cids.astype(np.uint32), tmp) + (q,)


@pytest.mark.parametrize("mode", ["seq", "split", "warp", "ws"])
@pytest.mark.parametrize("topk,nprobe", [(1, 3), (10, 12), (2000, 2), (4000, 12)])
def test_against_oracle(with_empty, mode, topk, nprobe, monkeypatch):
    index, oi, q = with_empty
    monkeypatch.setenv("SAQG_SCAN_MODE", mode)
    qq = q[:12]
    ids, d = index.search(qq, topk, nprobe, return_dists=True)
    oids, od = oi.search(qq, topk, nprobe, with_dists=True)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))


def test_batch_path_with_empty_clusters(with_empty):
    index, oi, q = with_empty
    for topk, nprobe in [(10, 12), (500, 4)]:
        ids, d = index.search(q, topk, nprobe, return_dists=True)  # 80 queries: the shortlist path
        oids, od = oi.search(q, topk, nprobe, with_dists=True)
        assert np.array_equal(ids, oids)
        assert np.array_equal(d.view(np.uint32), od.view(np.uint32))


def test_one_cluster_and_no_queries(tmp_path):
    x, q = data.gaussian_mixture(700, 64, 5, sigma=0.5, seed=3, n_query=5)
    cent = x.mean(axis=0, keepdims=True).astype(np.float32)
    cids = np.zeros(x.shape[0], np.uint32)
    index, oi = _build(x, cent, cids, tmp_path, bits=6.0, seg=False)
    ids, d = index.search(q, 20, 1, return_dists=True)
    oids, od = oi.search(q, 20, 1, with_dists=True)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    empty = index.search(np.zeros((0, 64), np.float32), 10, 1)
    assert empty.shape == (0, 10)
