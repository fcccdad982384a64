"""IVF::construct parity.

* CPU: the oracle's builder vs the reference's own construct (rotation off, so
  residuals are exact): variance, plan, ids, centroids, codes, factors and
  ex-codes all equal; the only bytes excluded are the ones the reference never
  initialises (tail lanes of a cluster's last block, ex factors of 0-bit
  segments, struct padding).
* GPU: the GPU builder vs the reference (same comparison) and vs the oracle
  with identical rotations (whole file byte-identical), then a search on the
  GPU-built index against the oracle.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from conftest import CONSTRUCT_CASES, GOLDEN
from saq_gb300 import data, index_format as F


def meaningful_equal(a: F.IndexFile, b: F.IndexFile):
    """Compare two parsed index files on every byte the reference initialises."""
    bad = []
    if a.variance.tobytes() != b.variance.tobytes():
        bad.append("variance")
    if F.plan_of(a) != F.plan_of(b):
        bad.append("plan")
    if a.centroids.tobytes() != b.centroids.tobytes():
        bad.append("centroids")
    S = len(a.segments)
    for ca, cb in zip(a.clusters, b.clusters):
        n = ca.num_vec
        nb = (n + 31) // 32
        valid = np.arange(nb * 32).reshape(nb, 32) < n
        if not np.array_equal(ca.ids, cb.ids):
            bad.append("ids")
        for s in range(S):
            if not np.array_equal(ca.centroids[s], cb.centroids[s]):
                bad.append("seg_centroid")
            bits = a.segments[s].bits
            if bits and not np.array_equal(ca.long_factors[:, s], cb.long_factors[:, s]):
                bad.append("long_factors")
        if S == 1:
            blk = ca.short_code.size // max(nb, 1)
            A, B = ca.short_code.reshape(nb, blk), cb.short_code.reshape(nb, blk)
            fa, fb = A[:, :256].copy().view(np.float32), B[:, :256].copy().view(np.float32)
            if not np.array_equal(fa[:, :32][valid], fb[:, :32][valid]):
                bad.append("onorm")
            if a.segments[0].bits and not np.array_equal(fa[:, 32:][valid], fb[:, 32:][valid]):
                bad.append("ip_cent_oa")
            full = n // 32
            if not np.array_equal(A[:full, 256:], B[:full, 256:]):
                bad.append("codes")
        else:
            fa, fb = ca.short_factors.reshape(nb, S, 64), cb.short_factors.reshape(nb, S, 64)
            for s in range(S):
                if not np.array_equal(fa[:, s, :32][valid], fb[:, s, :32][valid]):
                    bad.append("onorm")
                if a.segments[s].bits > 1 and not np.array_equal(fa[:, s, 32:][valid], fb[:, s, 32:][valid]):
                    bad.append("ip_cent_oa")
            full = n // 32
            blk = ca.short_code.size // max(nb, 1)
            if not np.array_equal(ca.short_code.reshape(nb, blk)[:full], cb.short_code.reshape(nb, blk)[:full]):
                bad.append("codes")
        if not np.array_equal(ca.long_code, cb.long_code):
            bad.append("long_code")
    return sorted(set(bad))


def load_case(name, tmp_path):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = json.loads(bytes(z["params"]).decode())
    ref_path = str(tmp_path / (name + ".index"))
    open(ref_path, "wb").write(z["index_bytes"].tobytes())
    return z, p, ref_path


@pytest.mark.parametrize("name", CONSTRUCT_CASES)
def test_oracle_construct_matches_reference(name, tmp_path):
    z, p, ref_path = load_case(name, tmp_path)
    out = str(tmp_path / "oracle.index")
    O.build_index(out, z["x"], z["centroids"], z["cids"], p["bits"], bool(p["seg"]), p["eqseg"], None)
    assert meaningful_equal(F.load(ref_path), F.load(out)) == []


@pytest.mark.gpu
@pytest.mark.parametrize("name", CONSTRUCT_CASES)
def test_gpu_construct_matches_reference(name, tmp_path):
    from saq_gb300 import ivf
    z, p, ref_path = load_case(name, tmp_path)
    cfg = ivf.QuantizeConfig(avg_bits=p["bits"], enable_segmentation=bool(p["seg"]), seg_eqseg=p["eqseg"],
                             random_rotation=False)
    index = ivf.IVF(z["x"].shape[0], z["x"].shape[1], z["centroids"].shape[0], cfg)
    index.construct(z["x"], z["centroids"], z["cids"])
    out = str(tmp_path / "gpu.index")
    index.save(out)
    assert meaningful_equal(F.load(ref_path), F.load(out)) == []


def _rotations(plan, seed):
    rng = np.random.default_rng(seed)
    mats = [data.random_orthogonal(d, rng).astype(np.float32) for d, _ in plan]
    return np.concatenate([m.reshape(-1) for m in mats])


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(4.0, True, 0, 256), (4.0, False, 0, 192), (1.5, True, 0, 256), (6.0, True, 0, 256),
                                  (10.0, True, 2, 128)])
def test_gpu_construct_matches_oracle_and_searches(case, tmp_path):
    from saq_gb300 import ivf
    bits, seg, eqseg, D = case
    x, q = data.anisotropic(3000, D, 0.8, seed=5, n_query=24)
    mean, comp, _ = data.pca_fit(x)
    x, q = data.pca_apply(x, mean, comp), data.pca_apply(q, mean, comp)
    cent, cids = data.kmeans(x, 12, iters=8, seed=2)
    var = O.colwise_var(x)
    plan = O.plan(var, bits, seg, eqseg)
    rots = _rotations(plan, 7)
    cfg = ivf.QuantizeConfig(avg_bits=bits, enable_segmentation=seg, seg_eqseg=eqseg)
    index = ivf.IVF(x.shape[0], D, 12, cfg)
    index.construct(x, cent, cids, rotations=rots)
    assert index.info()["plan"] == plan
    gpath, opath = str(tmp_path / "g.index"), str(tmp_path / "o.index")
    index.save(gpath)
    O.build_index(opath, x, cent, cids, bits, seg, eqseg, rots)
    assert open(gpath, "rb").read() == open(opath, "rb").read()
    oids, od = O.OracleIndex(opath).search(q, 10, 5, with_dists=True)
    for mode in ("seq", "split", "warp", "ws"):
        os.environ["SAQG_SCAN_MODE"] = mode
        try:
            ids, d = index.search(q, 10, 5, return_dists=True)
        finally:
            del os.environ["SAQG_SCAN_MODE"]
        assert np.array_equal(ids, oids), mode
        assert np.array_equal(d.view(np.uint32), od.view(np.uint32)), mode


@pytest.mark.gpu
@pytest.mark.parametrize("defer", ["1", "0"])
def test_batched_scan_with_deferred_queries(defer, tmp_path, monkeypatch):
    """Batch path: queries over the block budget go to the split pass (only the
    first 32 fit; the rest stay on the CTA scan).  Every answer must equal the
    oracle's, whichever path served it."""
    from saq_gb300 import ivf
    x, q = data.anisotropic(4000, 256, 0.8, seed=8, n_query=48)
    mean, comp, _ = data.pca_fit(x)
    x, q = data.pca_apply(x, mean, comp), data.pca_apply(q, mean, comp)
    cent, cids = data.kmeans(x, 10, iters=6, seed=3)
    var = O.colwise_var(x)
    plan = O.plan(var, 4.0, True, 0)
    rots = _rotations(plan, 9)
    index = ivf.IVF(x.shape[0], 256, 10, ivf.QuantizeConfig(avg_bits=4.0))
    index.construct(x, cent, cids, rotations=rots)
    opath = str(tmp_path / "o.index")
    O.build_index(opath, x, cent, cids, 4.0, True, 0, rots)
    monkeypatch.setenv("SAQG_SCAN_MODE", "seq")
    monkeypatch.setenv("SAQG_DEFER_BLOCKS", defer)
    for topk, nprobe in [(10, 4), (100, 10)]:
        ids, d = index.search(q, topk, nprobe, return_dists=True)
        oids, od = O.OracleIndex(opath).search(q, topk, nprobe, with_dists=True)
        assert np.array_equal(ids, oids)
        assert np.array_equal(d.view(np.uint32), od.view(np.uint32))


@pytest.mark.parametrize("case", [(4.0, True, 0, 256), (1.5, True, 0, 192), (9.0, False, 0, 128)])
def test_oracle_build_independent_of_threads(case, tmp_path):
    """The oracle's builder encodes vectors on many threads; the file must be the
    same for any thread count (every vector's arithmetic is independent)."""
    bits, seg, eqseg, D = case
    x, _ = data.anisotropic(2500, D, 0.8, seed=11)
    cent, cids = data.kmeans(x, 9, iters=3, seed=4)
    plan = O.plan(O.colwise_var(x), bits, seg, eqseg)
    rots = _rotations(plan, 13)
    files = []
    for th in (1, 3, 8):
        path = str(tmp_path / f"t{th}.index")
        O.build_index(path, x, cent, cids, bits, seg, eqseg, rots, threads=th)
        files.append(open(path, "rb").read())
    assert files[0] == files[1] == files[2]
