"""Parity at the sizes of the two single-query benchmark configurations.

* 100k x 960 Gaussian mixture (1,024 centres, sigma 0.5), PCA, k-means with
  1,024 clusters for 20 iterations; SAQ B=4 with segmentation; nprobe 32, k 10.
* 1M x 1024 unit-norm, per-axis variance i^-0.8, PCA, 4,096 k-means clusters;
  B in {1.5, 4} with and without segmentation (CAQ only); nprobe 16, 64, 128.

For each: the GPU builder and the CPU oracle's builder are given the same data,
centroids, ids, variance and rotations and must write byte-identical index
files (a NaN factor's sign bit aside, see _same_index); then 200 queries
are searched on the GPU (as one batch and one query per call, the plain
drop-in) and by the oracle, and ids and distances must be equal bit for bit.
The oracle is pinned to the reference by the golden fixtures.
"""
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

NQ = 200


def _build_both(wl, bits, seg, tmp, tag):
    from saq_gb300 import ivf, workloads
    var = wl.variance
    plan = O.plan(var, bits, seg, 0)
    rots = workloads.rotations(plan, seed=17)
    x = wl.x
    cent = wl.centroids.cpu().numpy()
    cids = wl.cids.cpu().numpy().astype(np.uint32)
    index = ivf.IVF(x.shape[0], x.shape[1], cent.shape[0],
                    ivf.QuantizeConfig(avg_bits=bits, enable_segmentation=seg))
    index.set_variance(var)
    index.construct(x, cent, cids, rotations=rots)
    assert index.info()["plan"] == plan
    gpath, opath = os.path.join(tmp, f"{tag}_gpu.index"), os.path.join(tmp, f"{tag}_oracle.index")
    index.save(gpath)
    O.build_index(opath, x.cpu().numpy(), cent, cids, bits, seg, 0, rots, variance=var)
    return index, gpath, opath


def _same_index(a, b):
    """Byte-identical files, except that a NaN factor may differ in its sign bit.

    A vector equal to its centroid (a one-vector cluster) has a zero residual;
    the reference's error factor is then 0 * sqrt(0/0 - 1) (caq_encoder.hpp:
    230-232), a NaN whose sign is the host's default NaN: negative on x86 (and on
    the GPU), positive on Arm.  Such NaNs compare equal here; every other byte
    must match."""
    from saq_gb300 import index_format as F
    if os.path.getsize(a) == os.path.getsize(b):
        with open(a, "rb") as fa, open(b, "rb") as fb:
            while True:
                x, y = fa.read(1 << 24), fb.read(1 << 24)
                if x != y:
                    break
                if not x:
                    return
    A, B = F.load(a), F.load(b)
    assert A.N == B.N and A.D == B.D and A.K == B.K
    assert A.centroids.tobytes() == B.centroids.tobytes()
    assert A.variance.tobytes() == B.variance.tobytes()
    assert A.quantize_cfg == B.quantize_cfg
    for sa, sb in zip(A.segments, B.segments):
        assert (sa.dim, sa.bits) == (sb.dim, sb.bits)
        assert (sa.P is None and sb.P is None) or sa.P.tobytes() == sb.P.tobytes()
    for ca, cb in zip(A.clusters, B.clusters):
        assert ca.num_vec == cb.num_vec
        for fld in ("ids", "short_factors", "short_code", "long_code"):
            assert np.ascontiguousarray(getattr(ca, fld)).tobytes() == np.ascontiguousarray(getattr(cb, fld)).tobytes()
        for x, y in zip(ca.centroids, cb.centroids):
            assert x.tobytes() == y.tobytes()
        fa, fb = ca.long_factors.view(np.uint32), cb.long_factors.view(np.uint32)
        nan = np.isnan(ca.long_factors)
        assert np.array_equal(nan, np.isnan(cb.long_factors))
        assert np.array_equal(fa[~nan], fb[~nan])


def _check_search(index, opath, q, nprobes, topk=10, single=True):
    oi = O.OracleIndex(opath)
    for nprobe in nprobes:
        oids, od = oi.search(q, topk, nprobe, threads=os.cpu_count() or 1, with_dists=True)
        ids, d = index.search(q, topk, nprobe, return_dists=True)
        assert np.array_equal(ids, oids), f"batch ids, nprobe {nprobe}"
        assert np.array_equal(d.view(np.uint32), od.view(np.uint32)), f"batch dists, nprobe {nprobe}"
        if single:
            for i in range(q.shape[0]):
                si, sd = index.search(q[i], topk, nprobe, return_dists=True)
                assert np.array_equal(si, oids[i]), f"single query {i}, nprobe {nprobe}"
                assert np.array_equal(sd.view(np.uint32), od[i].view(np.uint32)), f"single query {i}, nprobe {nprobe}"


@pytest.fixture(scope="module")
def c1_workload():
    import torch
    from saq_gb300 import workloads
    wl = workloads.gaussian_mixture_ivf(100_000, 960, 1024, 0.5, nq=NQ, k=1024, iters=20, seed=0)
    yield wl
    del wl
    torch.cuda.empty_cache()


def test_c1_gaussian_mixture_100k_x_960(c1_workload, tmp_path):
    wl = c1_workload
    assert wl.x.shape == (100_000, 960)
    index, gpath, opath = _build_both(wl, 4.0, True, str(tmp_path), "c1")
    _same_index(gpath, opath)
    q = wl.q[:NQ].cpu().numpy()
    _check_search(index, opath, q, [32])


@pytest.fixture(scope="module")
def c2_workload():
    import torch
    from saq_gb300 import workloads
    wl = workloads.aniso_ivf(1_000_000, 1024, 0.8, nq=NQ, k=4096, iters=8, seed=0)
    yield wl
    del wl
    torch.cuda.empty_cache()


@pytest.mark.parametrize("bits,seg", [(4.0, True), (4.0, False), (1.5, True), (1.5, False)])
def test_c2_aniso_1m_x_1024(c2_workload, bits, seg, tmp_path):
    import torch
    wl = c2_workload
    index, gpath, opath = _build_both(wl, bits, seg, str(tmp_path), f"c2_{bits}_{int(seg)}")
    _same_index(gpath, opath)
    q = wl.q[:NQ].cpu().numpy()
    _check_search(index, opath, q, [16, 64, 128], single=(bits == 4.0 and seg))
    del index
    torch.cuda.empty_cache()
