"""Tensor-core form of the batched search (saqg_search_tc).

The approximate distances come from the tensor cores; what the form returns is
checked against the oracle: every returned (id, distance) must be the oracle's
exact search distance for that vector (IVF::estimate's accurate distance for
one segment, bit for bit), and with a shortlist that holds every candidate the
answer must equal the oracle's top-k of those distances over all probed
vectors (ties: the later-scanned vector first).  With the default shortlist of
4 k, recall@10 against that full top-10 is measured and bounded."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN
from saq_gb300 import data

pytestmark = pytest.mark.gpu


def _build(tmp, bits, seg, d=256, n=8000, k=128, seed=11, eqseg=0):
    from saq_gb300 import ivf
    x, q = data.gaussian_mixture(n, d, 200, sigma=0.6, seed=seed, n_query=300)
    cent, cids = data.kmeans(x, k, iters=6, seed=2)
    rng = np.random.default_rng(5)
    plan = O.plan(O.colwise_var(x), float(bits), seg, eqseg)
    rots = np.concatenate([data.random_orthogonal(dd, rng).astype(np.float32).reshape(-1) for dd, _ in plan])
    index = ivf.IVF(n, d, k, ivf.QuantizeConfig(avg_bits=float(bits), enable_segmentation=seg,
                                                     seg_eqseg=eqseg))
    index.construct(x, cent, cids, rotations=rots)
    opath = str(tmp / f"tc_{bits}_{int(seg)}.index")
    O.build_index(opath, x, cent, cids, float(bits), seg, eqseg, rots)
    return index, O.OracleIndex(opath), q, plan


@pytest.fixture(scope="module", params=[6, 8, 4])
def built(request, tmp_path_factory):
    return _build(tmp_path_factory.mktemp("tc"), request.param, False)


def _full_topk(oi, q, nprobe, topk):
    """Oracle: top-k over every probed vector by the accurate distance, equal
    distances the later position first."""
    ids, acc, _, _ = oi.estimate(q, nprobe)
    order = sorted(range(len(acc)), key=lambda e: (np.float32(acc[e]), -e))[:topk]
    return ids[order], acc[order], dict(zip(ids.tolist(), acc.tolist())), len(acc)


@pytest.mark.parametrize("nq", [300, 20])
def test_full_shortlist_equals_oracle_topk(built, nq):
    index, oi, q, plan = built
    assert len(plan) == 1
    nprobe, topk = 3, 10
    ids, d = index.search_tc(q[:nq], topk, nprobe, shortlist=1024, return_dists=True)
    covered = 0
    for i in range(nq):
        oid, od, _, m = _full_topk(oi, q[i], nprobe, topk)
        if m > 1024:  # the shortlist does not hold every candidate of this query
            continue
        covered += 1
        assert np.array_equal(ids[i], oid), i
        assert np.array_equal(d[i].view(np.uint32), od.astype(np.float32).view(np.uint32)), i
    assert covered >= 0.8 * nq


def test_default_shortlist(built):
    index, oi, q, _ = built
    nprobe, topk = 16, 10
    ids, d, apx, st = index.search_tc(q, topk, nprobe, return_dists=True, return_approx=True, stats=True)
    hits, rel = 0, []
    for i in range(q.shape[0]):
        oid, od, accmap, _ = _full_topk(oi, q[i], nprobe, topk)
        for j in range(topk):  # every returned distance is the oracle's for that id
            assert accmap[int(ids[i, j])] == d[i, j], (i, j)
        assert np.all(np.diff(d[i]) >= 0)
        hits += len(set(ids[i].tolist()) & set(oid.tolist()))
        rel.extend(np.abs(apx[i] - d[i]) / np.maximum(np.abs(d[i]), 1e-6))
    recall = hits / (q.shape[0] * topk)
    assert recall >= 0.98, recall
    assert np.median(rel) < 2e-2, np.median(rel)
    assert st["pairs"] == q.shape[0] * nprobe and st["flops"] > 0 and st["ms_contract"] > 0


def test_batch_equals_single_queries(built):
    index, _, q, _ = built
    nprobe, topk = 12, 10
    ids, d = index.search_tc(q[:96], topk, nprobe, return_dists=True)
    for i in (0, 17, 95):
        si, sd = index.search_tc(q[i:i + 1], topk, nprobe, return_dists=True)
        assert np.array_equal(si[0], ids[i]) and np.array_equal(sd[0], d[i]), i


def test_uneven_batch_equals_single_queries(built):
    """Queries with their own nprobe and k in one call (saqg_search_tc_batch):
    each row equals that query searched alone with its own arguments and the
    same shortlist; rows are padded to the largest k with id 0 / FLT_MAX."""
    index, _, q, _ = built
    nq, L = 100, 48
    rng = np.random.default_rng(17)
    nps = rng.integers(2, 21, size=nq).astype(np.int32)
    ks = rng.choice([5, 10, 12], size=nq).astype(np.int32)
    ids, d = index.search_tc(q[:nq], ks, nps, shortlist=L, return_dists=True)
    assert ids.shape == (nq, 12)
    for i in range(0, nq, 9):
        si, sd = index.search_tc(q[i:i + 1], int(ks[i]), int(nps[i]), shortlist=L, return_dists=True)
        assert np.array_equal(si[0], ids[i, :ks[i]]) and np.array_equal(sd[0], d[i, :ks[i]]), i
        assert np.all(ids[i, ks[i]:] == 0) and np.all(d[i, ks[i]:] == np.float32(3.4028235e38)), i


def test_device_buffers_match_host(built):
    torch = pytest.importorskip("torch")
    index, _, q, _ = built
    ids, d = index.search_tc(q[:128], 10, 8, return_dists=True)
    qt = torch.as_tensor(q[:128], device="cuda")
    tids, td = index.search_tc(qt, 10, 8, return_dists=True)
    torch.cuda.synchronize()
    assert np.array_equal(tids.cpu().numpy().view(np.uint32), ids)
    assert np.array_equal(td.cpu().numpy(), d)


def test_multi_segment_distances_match_search(tmp_path):
    """Several coded segments: a returned id that the exact search also
    returns carries the exact search's distance bit for bit, and the answer is
    the top-10 of the estimator over every probed vector.  (The reference's
    multi-segment pruning by variance bounds is lossy: on this data its own
    search finds about 60% of that top-10, which the dense form recovers.)"""
    index, oi, q, plan = _build(tmp_path, 6, True, d=384, n=6000, k=64, seed=4, eqseg=3)
    assert len(plan) == 3 and all(b >= 1 for _, b in plan), plan
    nprobe, topk, nq = 8, 10, 120
    ids, d = index.search_tc(q[:nq], topk, nprobe, shortlist=200, return_dists=True)
    oids, od = oi.search(q[:nq], topk, nprobe, with_dists=True)
    common, full = 0, 0
    for i in range(nq):
        ref = dict(zip(oids[i].tolist(), od[i].tolist()))
        for j in range(topk):
            if int(ids[i, j]) in ref:
                common += 1
                assert np.float32(ref[int(ids[i, j])]) == d[i, j], (i, j)
        eids, acc, _, _ = oi.estimate(q[i], nprobe)  # sum of per-segment accurate distances
        full += len(set(ids[i].tolist()) & set(eids[np.argsort(acc, kind="stable")[:topk]].tolist()))
    assert common >= 0.5 * nq * topk
    assert full >= 0.97 * nq * topk, full / (nq * topk)


def test_rejects_uncoded_segments(golden_case_by_name):
    """An index with a 0-bit segment has no codes there to contract."""
    from saq_gb300 import _native as N, ivf
    z = np.load(os.path.join(GOLDEN, "aniso_b15_seg_0bit.npz"))
    assert any(int(b) == 0 for _, b in z["plan"])
    index = ivf.IVF.load(golden_case_by_name("aniso_b15_seg_0bit"))
    with pytest.raises(N.SaqgError, match="every segment coded"):
        index.search_tc(z["q"][:4], 10, 4)


@pytest.fixture(scope="module")
def with_empty(tmp_path_factory):
    """12 clusters, two of them empty and far away (as in test_edge_cases)."""
    from saq_gb300 import ivf
    tmp = tmp_path_factory.mktemp("tc_edge")
    x, q = data.gaussian_mixture(3000, 128, 40, sigma=0.6, seed=13, n_query=80)
    cent, cids = data.kmeans(x, 10, iters=5, seed=5)
    far = np.full((2, 128), 50.0, np.float32)
    far[1] *= -1
    cent = np.concatenate([cent, far])
    rng = np.random.default_rng(21)
    plan = O.plan(O.colwise_var(x), 6.0, False, 0)
    rots = np.concatenate([data.random_orthogonal(d, rng).astype(np.float32).reshape(-1) for d, _ in plan])
    index = ivf.IVF(x.shape[0], 128, cent.shape[0], ivf.QuantizeConfig(avg_bits=6.0, enable_segmentation=False))
    index.construct(x, cent, cids.astype(np.uint32), rotations=rots)
    opath = str(tmp / "o.index")
    O.build_index(opath, x, cent, cids.astype(np.uint32), 6.0, False, 0, rots)
    return index, O.OracleIndex(opath), q


@pytest.mark.parametrize("nq", [80, 6])
def test_edge_empty_clusters_and_unfilled_rows(with_empty, nq):
    """nprobe = every cluster (two empty), topk 1, and topk beyond the probed
    vectors (rows padded with id 0 / FLT_MAX); a query whose only probe is an
    empty cluster gets a row of padding."""
    index, oi, q = with_empty
    qq = q[:nq]
    for topk, nprobe, L in [(10, 12, 40), (1, 3, 4), (1000, 1, 1000)]:
        ids, d = index.search_tc(qq, topk, nprobe, shortlist=L, return_dists=True)
        for i in range(nq):
            oid, od, accmap, m = _full_topk(oi, qq[i], nprobe, topk)
            n = min(topk, m)
            for j in range(n):
                assert accmap[int(ids[i, j])] == d[i, j], (topk, nprobe, i, j)
            if m <= L:  # the shortlist holds every candidate: the oracle's top-k exactly
                assert np.array_equal(ids[i, :n], oid[:n]) and np.array_equal(d[i, :n], od[:n].astype(np.float32))
            assert np.all(ids[i, n:] == 0) and np.all(d[i, n:] == np.float32(3.4028235e38))
    far_q = np.full((1, 128), 50.0, np.float32)  # nearest centroid: an empty cluster
    ids, d = index.search_tc(far_q, 5, 1, return_dists=True)
    assert np.all(ids == 0) and np.all(d == np.float32(3.4028235e38))


def test_edge_one_cluster_and_no_queries(tmp_path):
    from saq_gb300 import ivf
    x, q = data.gaussian_mixture(700, 64, 5, sigma=0.5, seed=3, n_query=5)
    cent = x.mean(axis=0, keepdims=True).astype(np.float32)
    cids = np.zeros(x.shape[0], np.uint32)
    rng = np.random.default_rng(22)
    plan = O.plan(O.colwise_var(x), 6.0, False, 0)
    rots = np.concatenate([data.random_orthogonal(dd, rng).astype(np.float32).reshape(-1) for dd, _ in plan])
    index = ivf.IVF(x.shape[0], 64, 1, ivf.QuantizeConfig(avg_bits=6.0, enable_segmentation=False))
    index.construct(x, cent, cids, rotations=rots)
    opath = str(tmp_path / "one.index")
    O.build_index(opath, x, cent, cids, 6.0, False, 0, rots)
    oi = O.OracleIndex(opath)
    ids, d = index.search_tc(q, 20, 1, shortlist=1000, return_dists=True)
    for i in range(q.shape[0]):
        oid, od, _, _ = _full_topk(oi, q[i], 1, 20)
        assert np.array_equal(ids[i], oid) and np.array_equal(d[i], od.astype(np.float32)), i
    empty = index.search_tc(np.zeros((0, 64), np.float32), 10, 1)
    assert empty.shape == (0, 10)


def test_contraction_wait_timeout_is_reported_and_the_context_recovers(built, monkeypatch):
    """The contraction's bounded pipeline waits: with a 20 ms limit and one stage
    of CTA 0 that never fills (the test hooks SAQG_TEST_TC_WAIT_MS and
    SAQG_TEST_TC_SKIP_STAGE), the waits run out, the CTA drains and frees its
    tensor memory, and the call returns SAQG_ERR_INTERNAL; the next call on the
    same index returns the same answers as before, bit for bit."""
    index, _, q, _ = built
    nq, topk = 64, 10
    nprobe = index.num_cen  # every cluster: CTA 0 has work
    want_ids, want_d = index.search_tc(q[:nq], topk, nprobe, shortlist=40, return_dists=True)
    monkeypatch.setenv("SAQG_TEST_TC_WAIT_MS", "20")
    monkeypatch.setenv("SAQG_TEST_TC_SKIP_STAGE", "1")
    from saq_gb300._native import SaqgError
    with pytest.raises(SaqgError, match="timed out"):
        index.search_tc(q[:nq], topk, nprobe, shortlist=40, return_dists=True)
    monkeypatch.delenv("SAQG_TEST_TC_WAIT_MS")
    monkeypatch.delenv("SAQG_TEST_TC_SKIP_STAGE")
    ids, d = index.search_tc(q[:nq], topk, nprobe, shortlist=40, return_dists=True)
    assert np.array_equal(ids, want_ids)
    assert np.array_equal(np.asarray(d).view(np.uint32), np.asarray(want_d).view(np.uint32))
