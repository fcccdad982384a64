"""The segment planner on the GPU (saqg_plan_gpu): the reference's dynamic
program (SaqDataMaker::dynamic_programming, saq_data.hpp:147-227) with one
thread per state of a level.  Its plans must equal the reference's golden plans
and the host planner's on random and tie-heavy variances."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_device_plan_matches_reference_golden():
    from saq_gb300 import ivf
    z = np.load(os.path.join(GOLDEN, "plan.npz"))
    i = 0
    while f"c{i}_var" in z:
        p = ivf.plan_gpu(z[f"c{i}_var"], float(z[f"c{i}_avg_bits"]))
        assert p == [tuple(map(int, r)) for r in z[f"c{i}_plan"]], i
        i += 1
    assert i > 0


@pytest.mark.parametrize("dim", [64, 128, 448, 960, 1024, 1536])
@pytest.mark.parametrize("avg_bits", [1.0, 1.5, 2.0, 3.0, 4.0, 6.0, 8.0])
def test_device_plan_matches_host_planner(dim, avg_bits):
    from saq_gb300 import ivf
    rng = np.random.default_rng(dim * 100 + int(avg_bits * 10))
    variances = [
        (np.arange(1, dim + 1, dtype=np.float64) ** -0.8).astype(np.float32),           # decaying spectrum
        rng.gamma(0.5, 1.0, size=dim).astype(np.float32),                               # random
        np.ones(dim, np.float32),                                                        # all equal: ties
        np.repeat(rng.integers(1, 4, size=dim // 64), 64).astype(np.float32),          # equal blocks
        np.concatenate([np.full(dim // 2, 3.0), np.zeros(dim - dim // 2)]).astype(np.float32),  # zero tail
    ]
    for v in variances:
        assert ivf.plan_gpu(v, avg_bits) == ivf.plan(v, avg_bits), (dim, avg_bits)


def test_device_plan_from_device_memory_and_equal_segmentation():
    import torch
    from saq_gb300 import ivf
    v = (np.arange(1, 1025, dtype=np.float64) ** -1.0).astype(np.float32)
    assert ivf.plan_gpu(torch.from_numpy(v).cuda(), 4.0) == ivf.plan(v, 4.0)
    assert ivf.plan_gpu(v, 4.0, enable_segmentation=False) == [(1024, 4)]
    assert ivf.plan_gpu(v, 4.0, seg_eqseg=3) == ivf.plan(v, 4.0, seg_eqseg=3)
