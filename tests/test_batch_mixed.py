"""Batches whose queries carry their own nprobe and k (the uneven batches of
the batching and serving forms).  Each query's answer must equal the oracle's
for that query alone, bit for bit, in every scan form; rows are padded to the
largest k with id 0 / inf."""
import numpy as np
import pytest

import oracle as O
from saq_gb300 import data

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    from saq_gb300 import ivf
    tmp = tmp_path_factory.mktemp("mixed")
    x, q = data.gaussian_mixture(12000, 128, 300, sigma=0.6, seed=6, n_query=120)
    cent, cids = data.kmeans(x, 160, iters=6, seed=2)
    rng = np.random.default_rng(3)
    plan = O.plan(O.colwise_var(x), 4.0, True, 0)
    rots = np.concatenate([data.random_orthogonal(d, rng).astype(np.float32).reshape(-1) for d, _ in plan])
    index = ivf.IVF(x.shape[0], 128, 160, ivf.QuantizeConfig(avg_bits=4.0))
    index.construct(x, cent, cids, rotations=rots)
    opath = str(tmp / "o.index")
    O.build_index(opath, x, cent, cids, 4.0, True, 0, rots)
    return index, O.OracleIndex(opath), q


@pytest.mark.parametrize("mode,defer", [(None, None), ("seq", "1"), ("seq", "0"), ("split", None), ("ws", "1"), ("ws", "0")])
@pytest.mark.parametrize("nq", [40, 120])
def test_mixed_nprobe_and_k(built, mode, defer, nq, monkeypatch):
    index, oi, q = built
    if mode:
        monkeypatch.setenv("SAQG_SCAN_MODE", mode)
    if defer:
        monkeypatch.setenv("SAQG_DEFER_BLOCKS", defer)
    rng = np.random.default_rng(nq)
    qq = q[:nq]
    nps = rng.integers(4, 41, size=nq).astype(np.int32)
    ks = rng.choice([10, 100], size=nq).astype(np.int32)
    ids, d = index.search(qq, ks, nps, return_dists=True)
    assert ids.shape == (nq, 100)
    for i in range(nq):
        oids, od = oi.search(qq[i:i + 1], int(ks[i]), int(nps[i]), with_dists=True)
        assert np.array_equal(ids[i, :ks[i]], oids[0]), i
        assert np.array_equal(d[i, :ks[i]].view(np.uint32), od[0].view(np.uint32)), i
        assert np.all(ids[i, ks[i]:] == 0) and np.all(np.isinf(d[i, ks[i]:]) | (d[i, ks[i]:] == np.float32(3.4028235e38)))


@pytest.mark.parametrize("mode,defer", [(None, None), ("seq", "1"), ("seq", "0"), ("ws", "0")])
def test_large_batch_heaviest_first(built, mode, defer, monkeypatch):
    """Batches of 1,024 queries and more launch the CTA scan heaviest query
    first; every answer must still be the oracle's, uniform and uneven shapes."""
    index, oi, q = built
    if mode:
        monkeypatch.setenv("SAQG_SCAN_MODE", mode)
    if defer:
        monkeypatch.setenv("SAQG_DEFER_BLOCKS", defer)
    rng = np.random.default_rng(11)
    nq = 1500
    qq = (q[rng.integers(0, q.shape[0], size=nq)] + rng.normal(0, 0.05, size=(nq, q.shape[1]))).astype(np.float32)
    ids, d = index.search(qq, 10, 24, return_dists=True)
    oids, od = oi.search(qq, 10, 24, with_dists=True)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    nps = rng.integers(4, 41, size=nq).astype(np.int32)
    ids, d = index.search(qq, 10, nps, return_dists=True)
    for i in range(0, nq, 7):
        oids, od = oi.search(qq[i:i + 1], 10, int(nps[i]), with_dists=True)
        assert np.array_equal(ids[i], oids[0]), i
        assert np.array_equal(d[i].view(np.uint32), od[0].view(np.uint32)), i


@pytest.mark.parametrize("mode,defer", [(None, None), ("seq", "1"), ("split", None)])
@pytest.mark.parametrize("budget_positions", [1, 300, 3000])
def test_record_space_exhausted(built, mode, defer, budget_positions, monkeypatch):
    """The split pass's record space holds only some of the queries it would take:
    the heaviest go first, the rest are answered by the CTA scan; every answer must
    still be the oracle's (uniform and uneven shapes)."""
    index, oi, q = built
    if mode:
        monkeypatch.setenv("SAQG_SCAN_MODE", mode)
    if defer:
        monkeypatch.setenv("SAQG_DEFER_BLOCKS", defer)
    # bytes per record position for the index's segments: 4 x the record words + the summary
    S = len(index.info()["plan"])
    words = (8 + (S + 1) + 32 + 32 * S + 3) & ~3
    monkeypatch.setenv("SAQG_SPLIT_RECORD_BYTES", str(budget_positions * (4 * words + 16)))
    rng = np.random.default_rng(budget_positions)
    nq = 90
    qq = q[:nq]
    ids, d = index.search(qq, 10, 20, return_dists=True)
    oids, od = oi.search(qq, 10, 20, with_dists=True)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    nps = rng.integers(4, 41, size=nq).astype(np.int32)
    ks = rng.choice([10, 100], size=nq).astype(np.int32)
    ids, d = index.search(qq, ks, nps, return_dists=True)
    for i in range(nq):
        oids, od = oi.search(qq[i:i + 1], int(ks[i]), int(nps[i]), with_dists=True)
        assert np.array_equal(ids[i, :ks[i]], oids[0]), i
        assert np.array_equal(d[i, :ks[i]].view(np.uint32), od[0].view(np.uint32)), i
