"""The reference unit test's acceptance for the cluster estimators
(unit_test/ut_cluster_estimator.cpp:148-160), on the oracle: synthetic integer
data in the style of test_base.hpp:55-88 (values in [-8, 8], one zero
centroid), 1,024 vectors x 768 dims, 16 queries, B = 4.  For every query the
average relative error of the accurate distance against the exact squared
distance is below 0.2, and every fast, accurate and variance-bound estimate is
non-negative.  The oracle reproduces the reference bit for bit and the GPU
reproduces the oracle bit for bit (tests/test_oracle_golden.py,
tests/test_gpu_parity.py), so the bound holds for all three."""
import numpy as np
import pytest

import oracle as O
from saq_gb300 import data


@pytest.mark.parametrize("seg,rotate", [(False, False), (False, True), (True, False)])
def test_relative_error_of_the_accurate_estimate(tmp_path, seg, rotate):
    x, q, cent, cids = data.int_grid(1024, 16, 768, num_centroids=1, seed=42)
    rots = None
    if rotate:
        rng = np.random.default_rng(7)
        plan = O.plan(O.colwise_var(x), 4.0, seg, 0)
        rots = np.concatenate([data.random_orthogonal(d, rng).astype(np.float32).reshape(-1) for d, _ in plan])
    path = str(tmp_path / "est.index")
    O.build_index(path, x, cent, np.asarray(cids, np.uint32), 4.0, seg, 0, rots)
    oi = O.OracleIndex(path)
    for i in range(q.shape[0]):
        ids, acc, fast, var = oi.estimate(q[i], 1)
        assert len(ids) == x.shape[0]
        true = ((x[ids].astype(np.float64) - q[i].astype(np.float64)) ** 2).sum(1)
        rel = np.abs(acc - true) / (true + 1e-18)
        assert rel.mean() < 0.2, (i, rel.mean())
        assert (acc >= 0).all() and (fast >= 0).all() and (var >= 0).all()
