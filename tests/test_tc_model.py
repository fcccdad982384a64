"""The tensor-core form's distance formula, checked on the CPU.

The contraction computes, per segment,
    |o|^2 + |r|^2 - 2 rescale (delta <r, u> + (delta/2 - 1) sum r)
with u the full B-bit code.  That is the reference's compAccurateDist with
the 1-bit part's u16 LUT replaced by the exact code.  The oracle's double
precision model of it (orc_tc_approx) must therefore agree with the reference's
accurate distance up to the LUT's quantisation, and rank the same top-10, on
every reference-built golden index whose segments are all coded."""
import numpy as np
import pytest

import oracle as O
from conftest import INDEX_CASES, GoldenCase


@pytest.mark.parametrize("name", INDEX_CASES)
def test_model_matches_reference_estimator(name, golden_dir):
    g = GoldenCase(name, golden_dir)
    if any(b == 0 for _, b in g.plan):
        pytest.skip("a 0-bit segment: the tensor-core form rejects such plans")
    oi = O.OracleIndex(g.index_path)
    for i in range(min(8, g.q.shape[0])):
        ia, acc, _, _ = oi.estimate(g.q[i], g.nprobe)
        it, apx = oi.tc_approx(g.q[i], g.nprobe)
        assert np.array_equal(ia, it)
        rel = np.abs(apx - acc) / np.maximum(np.abs(acc), 1e-9)
        assert np.median(rel) < 2e-5 and rel.max() < 1e-3, (i, np.median(rel), rel.max())
        k = min(10, len(acc))
        top_a = set(ia[np.argsort(acc, kind="stable")[:k]].tolist())
        top_t = set(it[np.argsort(apx, kind="stable")[:k]].tolist())
        assert len(top_a & top_t) >= k - 1, i
