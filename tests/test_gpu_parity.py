"""CUDA path vs the reference's golden outputs and the CPU oracle (bit-exact).

Tolerance: none.  Result ids, integer LUT work and every float distance are
compared bit for bit: the kernels reproduce the reference's operation order.
"""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def bits_eq(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))))


@pytest.fixture(scope="module")
def saqg():
    from saq_gb300 import ivf
    return ivf


@pytest.fixture(params=["seq", "split", "warp", "ws"])
def scan_mode(request, monkeypatch):
    """The exact scan implementations: CTA per query, split scan, warp per query,
    and CTA per query with the replay on its own warp (warp-specialised)."""
    monkeypatch.setenv("SAQG_SCAN_MODE", request.param)
    return request.param


def test_search_matches_reference(golden_case, saqg, scan_mode):
    idx = saqg.IVF.load(golden_case.index_path)
    ids, dists = idx.search(golden_case.q, golden_case.topk, golden_case.nprobe, return_dists=True)
    assert np.array_equal(ids, golden_case.z["search_ids"])
    oi = O.OracleIndex(golden_case.index_path)
    oids, od = oi.search(golden_case.q, golden_case.topk, golden_case.nprobe, with_dists=True)
    assert np.array_equal(ids, oids)
    assert bits_eq(dists, od)


def test_single_query_signature(golden_case, saqg, scan_mode):
    idx = saqg.IVF.load(golden_case.index_path)
    for i in range(min(3, golden_case.q.shape[0])):
        ids = idx.search(golden_case.q[i], golden_case.topk, golden_case.nprobe)
        assert ids.shape == (golden_case.topk,)
        assert np.array_equal(ids, golden_case.z["search_ids"][i])


def test_estimate_matches_reference(golden_case, saqg):
    z = golden_case.z
    idx = saqg.IVF.load(golden_case.index_path)
    off = 0
    for i, n in enumerate(z["est_count"].astype(int)):
        ids, acc, fast, var = idx.estimate(golden_case.q[i], golden_case.nprobe)
        assert len(ids) == n
        assert np.array_equal(ids, z["est_ids"][off:off + n])
        assert bits_eq(acc, z["est_acc"][off:off + n])
        assert bits_eq(fast, z["est_fast"][off:off + n])
        assert bits_eq(var, z["est_vars"][off:off + n])
        off += n


def test_save_roundtrip_is_byte_identical(golden_case, saqg, tmp_path):
    idx = saqg.IVF.load(golden_case.index_path)
    out = str(tmp_path / "rt.index")
    idx.save(out)
    assert open(out, "rb").read() == open(golden_case.index_path, "rb").read()


def test_search_device_tensors(golden_case, saqg):
    torch = pytest.importorskip("torch")
    idx = saqg.IVF.load(golden_case.index_path)
    q = torch.from_numpy(golden_case.q).cuda()
    ids, dists = idx.search(q, golden_case.topk, golden_case.nprobe, return_dists=True)
    torch.cuda.synchronize()
    assert np.array_equal(ids.cpu().numpy().view(np.uint32), golden_case.z["search_ids"])


@pytest.mark.parametrize("bits", [1, 2, 3, 4, 5, 6, 7, 8, 9, 13])
def test_caq_encoder_matches_reference(bits, saqg):
    z = np.load(os.path.join(GOLDEN, "encode.npz"))
    r, cen = z[f"b{bits}_resid"], z[f"b{bits}_centroid"]
    codes, facs = saqg.caq_encode(r, bits, cen)
    assert np.array_equal(codes, z[f"b{bits}_codes"])
    ref = z[f"b{bits}_facs"]
    assert bits_eq(facs[:, [0, 2, 3]], ref[:, [0, 2, 3]])
    if bits > 1:
        assert bits_eq(facs[:, 1], ref[:, 1])


def test_errors_are_reported(golden_case, saqg):
    from saq_gb300._native import SaqgError
    idx = saqg.IVF.load(golden_case.index_path)
    with pytest.raises(SaqgError):
        idx.search(golden_case.q, golden_case.topk, idx.num_cen + 1)
    with pytest.raises(SaqgError):
        saqg.IVF.load(golden_case.index_path + ".missing")
