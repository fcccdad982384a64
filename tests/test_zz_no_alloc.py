"""saqg_search_static: the search entry point that allocates nothing.

Its scratch is a static device array shared by every call, so each case makes
two calls in a row and both must return exactly what saqg_search returns on the
same device inputs (ids equal, distances bit for bit: the tolerance of every
parity test here is none).  Device free memory must not move across a call
after the first.  Collected last, so it runs both after the other GPU tests
and, alone, in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _as_u32(t):
    return t.cpu().numpy().view(np.uint32)


def _bits(t):
    return t.cpu().numpy().view(np.uint32)


def test_static_search_matches_search_twice(golden_case):
    torch = pytest.importorskip("torch")
    from saq_gb300 import _native as N, ivf
    lib = N.load()
    idx = ivf.IVF.load(golden_case.index_path)
    cfg = ivf.SearcherConfig().to_c()
    q = torch.from_numpy(np.ascontiguousarray(golden_case.q)).cuda()
    nq, topk, nprobe = q.shape[0], golden_case.topk, golden_case.nprobe
    stream = torch.cuda.current_stream().cuda_stream

    ref_ids = torch.empty((nq, topk), dtype=torch.int32, device="cuda")
    ref_d = torch.empty((nq, topk), dtype=torch.float32, device="cuda")
    N.check(lib.saqg_search(idx._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), ref_ids.data_ptr(),
                            ref_d.data_ptr(), N.SAQG_MEM_DEVICE, stream))
    torch.cuda.synchronize()
    assert np.array_equal(_as_u32(ref_ids), golden_case.z["search_ids"])

    outs = [(torch.full((nq, topk), -1, dtype=torch.int32, device="cuda"),
             torch.full((nq, topk), float("nan"), dtype=torch.float32, device="cuda")) for _ in range(2)]
    torch.cuda.synchronize()
    free_before = None
    for call, (ids, d) in enumerate(outs):
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        N.check(lib.saqg_search_static(idx._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), ids.data_ptr(),
                                       d.data_ptr(), stream))
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        assert np.array_equal(_as_u32(ids), _as_u32(ref_ids)), f"call {call}"
        assert np.array_equal(_bits(d), _bits(ref_d)), f"call {call}"


def test_static_search_rejects_batches_beyond_its_scratch(golden_case):
    torch = pytest.importorskip("torch")
    from saq_gb300 import _native as N, ivf
    lib = N.load()
    idx = ivf.IVF.load(golden_case.index_path)
    info = idx.info()
    # a lower bound of the bytes one query needs (padded dim >= dim, >= 1 segment)
    per_query = 12 * info["num_clusters"] + 4 * golden_case.nprobe + 4 * info["num_dim"]
    nq = N.SAQG_STATIC_SCRATCH_BYTES // per_query + 16
    q = torch.zeros((nq, info["num_dim"]), dtype=torch.float32, device="cuda")
    ids = torch.zeros((nq, golden_case.topk), dtype=torch.int32, device="cuda")
    rc = lib.saqg_search_static(idx._h, q.data_ptr(), nq, golden_case.topk, golden_case.nprobe, None,
                                ids.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert rc == 1  # SAQG_ERR_INVALID
    assert b"static maximum" in lib.saqg_last_error()


def _static_bytes(nq, K, nprobe, dtot, S):
    """Scratch bytes of a call (the header's formula: each term rounded up to 16, + 64)."""
    a16 = lambda x: (x + 15) // 16 * 16  # noqa: E731
    return a16(4 * nq * K) + a16(8 * nq * K) + a16(4 * nq * nprobe) + a16(4 * nq * dtot) + a16(4 * nq * S) + 64


def test_static_search_at_its_largest_batch(golden_case_by_name):
    """The largest batch whose scratch fits the static array ends its last
    scratch region within the array: it must run and equal saqg_search bit for
    bit; one query more must be rejected before any work."""
    torch = pytest.importorskip("torch")
    from saq_gb300 import _native as N, ivf
    lib = N.load()
    idx = ivf.IVF.load(golden_case_by_name("aniso_b4_seg"))
    info = idx.info()
    K, D = info["num_clusters"], info["num_dim"]
    dtot, S = sum(d for d, _ in info["plan"]), len(info["plan"])
    topk, nprobe = 10, min(4, K)
    lo, hi = 1, 1
    while _static_bytes(hi, K, nprobe, dtot, S) <= N.SAQG_STATIC_SCRATCH_BYTES:
        lo, hi = hi, hi * 2
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if _static_bytes(mid, K, nprobe, dtot, S) <= N.SAQG_STATIC_SCRATCH_BYTES:
            lo = mid
        else:
            hi = mid
    nq = lo
    assert _static_bytes(nq + 1, K, nprobe, dtot, S) > N.SAQG_STATIC_SCRATCH_BYTES
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    q = torch.randn((nq + 1, D), generator=g, device="cuda")
    cfg = ivf.SearcherConfig().to_c()
    stream = torch.cuda.current_stream().cuda_stream
    ref_ids = torch.empty((nq, topk), dtype=torch.int32, device="cuda")
    ref_d = torch.empty((nq, topk), dtype=torch.float32, device="cuda")
    N.check(lib.saqg_search(idx._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), ref_ids.data_ptr(),
                            ref_d.data_ptr(), N.SAQG_MEM_DEVICE, stream))
    ids = torch.full((nq + 1, topk), -1, dtype=torch.int32, device="cuda")
    d = torch.full((nq + 1, topk), float("nan"), dtype=torch.float32, device="cuda")
    for call in range(2):
        N.check(lib.saqg_search_static(idx._h, q.data_ptr(), nq, topk, nprobe, C.byref(cfg), ids.data_ptr(),
                                       d.data_ptr(), stream))
        torch.cuda.synchronize()
        assert np.array_equal(_as_u32(ids[:nq]), _as_u32(ref_ids)), f"call {call}"
        assert np.array_equal(_bits(d[:nq]), _bits(ref_d)), f"call {call}"
    rc = lib.saqg_search_static(idx._h, q.data_ptr(), nq + 1, topk, nprobe, C.byref(cfg), ids.data_ptr(),
                                d.data_ptr(), stream)
    assert rc == 1 and b"static maximum" in lib.saqg_last_error()


def test_static_search_rejects_host_pointers(golden_case_by_name):
    """Host memory passed as queries or results is reported (SAQG_ERR_INVALID),
    never handed to a kernel."""
    torch = pytest.importorskip("torch")
    from saq_gb300 import _native as N, ivf
    lib = N.load()
    idx = ivf.IVF.load(golden_case_by_name("aniso_b4_seg"))
    D = idx.info()["num_dim"]
    qh = np.zeros((2, D), np.float32)
    ih = np.zeros((2, 10), np.uint32)
    qd = torch.zeros((2, D), dtype=torch.float32, device="cuda")
    idd = torch.zeros((2, 10), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.saqg_search_static(idx._h, qh.ctypes.data, 2, 10, 2, None, idd.data_ptr(), None, stream)
    assert rc == 1 and b"queries must be device memory" in lib.saqg_last_error()
    rc = lib.saqg_search_static(idx._h, qd.data_ptr(), 2, 10, 2, None, ih.ctypes.data, None, stream)
    assert rc == 1 and b"ids must be device memory" in lib.saqg_last_error()
    N.check(lib.saqg_search_static(idx._h, qd.data_ptr(), 2, 10, 2, None, idd.data_ptr(), None, stream))
    torch.cuda.synchronize()
