"""Pins the CPU oracle against golden vectors produced by the reference itself."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN


def bits_eq(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return np.array_equal(a.view(np.uint32), b.view(np.uint32)) or (
        a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b)))))


def test_search_ids(golden_case):
    oi = O.OracleIndex(golden_case.index_path)
    ids = oi.search(golden_case.q, golden_case.topk, golden_case.nprobe)
    assert np.array_equal(ids, golden_case.z["search_ids"])


def test_estimate_bit_exact(golden_case):
    z = golden_case.z
    oi = O.OracleIndex(golden_case.index_path)
    off = 0
    for i, n in enumerate(z["est_count"].astype(int)):
        ids, acc, fast, var = oi.estimate(golden_case.q[i], golden_case.nprobe)
        assert len(ids) == n
        assert np.array_equal(ids, z["est_ids"][off:off + n])
        assert bits_eq(acc, z["est_acc"][off:off + n])
        assert bits_eq(fast, z["est_fast"][off:off + n])
        assert bits_eq(var, z["est_vars"][off:off + n])
        off += n


def test_probe_rotation_lut_sums(golden_case):
    z = golden_case.z
    oi = O.OracleIndex(golden_case.index_path)
    plan = golden_case.plan
    dims = [d for d, _ in plan]
    nprobe = golden_case.nprobe
    nq = z["dump_probe_ids"].size // nprobe
    pid = z["dump_probe_ids"].reshape(nq, nprobe)
    pd = z["dump_probe_d"].reshape(nq, nprobe)
    rotq = z["dump_rotq"].reshape(nq, sum(dims))
    prune = z["dump_prune"].reshape(nq, len(dims))
    from saq_gb300 import index_format
    idx = index_format.load(golden_case.index_path)
    so = lo = uo = 0
    for i in range(nq):
        ids, d = oi.probe(golden_case.q[i], nprobe)
        assert np.array_equal(ids, pid[i]) and bits_eq(d, pd[i])
        r, p = oi.query_prep(golden_case.q[i], dims)
        assert bits_eq(r, rotq[i]) and bits_eq(p, prune[i])
        for c in pid[i]:
            nb = (idx.clusters[c].num_vec + 31) // 32
            for s, (dim, b) in enumerate(plan):
                lut, scal, sums, _ = oi.lut(golden_case.q[i], int(c), s, dim, nb)
                assert bits_eq(scal, z["dump_scal"][so:so + 5])
                so += 5
                if b == 0:
                    continue
                n = dim // 4 * 16
                assert np.array_equal(lut, z["dump_lut"][lo:lo + n])
                lo += n
                assert np.array_equal(sums, z["dump_sums"][uo:uo + nb * 32])
                uo += nb * 32
    assert so == z["dump_scal"].size and lo == z["dump_lut"].size and uo == z["dump_sums"].size


@pytest.mark.parametrize("bits", [1, 2, 3, 4, 5, 6, 7, 8, 9, 13])
def test_encoder_and_packing(bits):
    z = np.load(os.path.join(GOLDEN, "encode.npz"))
    r, cen = z[f"b{bits}_resid"], z[f"b{bits}_centroid"]
    codes, facs = O.caq_encode(r, bits, cen)
    assert np.array_equal(codes, z[f"b{bits}_codes"])
    ref = z[f"b{bits}_facs"]
    assert bits_eq(facs[:, [0, 2, 3]], ref[:, [0, 2, 3]])
    if bits > 1:
        assert bits_eq(facs[:, 1], ref[:, 1])
        low = (codes & ((1 << (bits - 1)) - 1)).astype(np.uint16)
        for i in range(r.shape[0]):
            packed = O.pack_excode(low[i], bits - 1)
            assert np.array_equal(packed, z[f"b{bits}_long"][i])
            assert np.array_equal(O.unpack_excode(packed, r.shape[1], bits - 1), low[i])
    # first FastScan block: top bit of every dimension, MSB-first bytes, kPerm0 interleave
    D = r.shape[1]
    top = ((codes[:32] >> (bits - 1)) & 1).astype(np.uint8)
    sc = np.packbits(top, axis=1)
    assert np.array_equal(O.pack_block(sc, D), z[f"b{bits}_blocks"][256:256 + 4 * D])


def test_planner():
    z = np.load(os.path.join(GOLDEN, "plan.npz"))
    i = 0
    while f"c{i}_var" in z:
        plan = O.plan(z[f"c{i}_var"], float(z[f"c{i}_avg_bits"]))
        assert plan == [tuple(map(int, r)) for r in z[f"c{i}_plan"]]
        i += 1
    assert i >= 8
