"""Index file v2: conversion from and to the reference format (host only, no
GPU), corruption detection, and search on a v2-loaded index (GPU)."""
import struct

import numpy as np
import pytest

from conftest import INDEX_CASES, CONSTRUCT_CASES
from saq_gb300 import ivf
from saq_gb300._native import SaqgError


def _v2_sections(path):
    b = open(path, "rb").read()
    assert b[:8] == b"SAQGIDX2"
    version, hdr = struct.unpack_from("<II", b, 8)
    n, d, k, s, compact, nvar = struct.unpack_from("<6Q", b, 16)
    at = 16 + 48 + 32 + s * 40
    (nsec,) = struct.unpack_from("<Q", b, at)
    secs = [struct.unpack_from("<IIQQQ", b, at + 8 + 32 * i) for i in range(nsec)]
    return version, hdr, (n, d, k, s), secs, len(b)


@pytest.mark.parametrize("name", INDEX_CASES + CONSTRUCT_CASES)
def test_reference_v2_round_trip_is_byte_identical(golden_case_by_name, name, tmp_path):
    src = golden_case_by_name(name)
    v2, back = str(tmp_path / "x.v2"), str(tmp_path / "back.index")
    ivf.convert(src, v2, "v2")
    ivf.convert(v2, back, "reference")
    assert open(back, "rb").read() == open(src, "rb").read()
    version, hdr, (n, d, k, s), secs, size = _v2_sections(v2)
    assert version == 2 and size % 4096 == 0
    assert all(off % 4096 == 0 for _, _, off, _, _ in secs)
    # v2 -> v2 is stable too
    v2b = str(tmp_path / "y.v2")
    ivf.convert(v2, v2b, "v2")
    assert open(v2b, "rb").read() == open(v2, "rb").read()


def test_v2_corruption_is_detected(golden_case_by_name, tmp_path):
    src = golden_case_by_name(INDEX_CASES[0])
    v2 = str(tmp_path / "x.v2")
    ivf.convert(src, v2, "v2")
    raw = bytearray(open(v2, "rb").read())
    _, hdr, _, secs, _ = _v2_sections(v2)
    for pos in (secs[-1][2] + 5, 40):  # a byte of the last section, then of the header
        bad = bytearray(raw)
        bad[pos] ^= 0x40
        p = str(tmp_path / f"bad{pos}.v2")
        open(p, "wb").write(bytes(bad))
        with pytest.raises(SaqgError, match="checksum"):
            ivf.convert(p, str(tmp_path / "out.index"), "reference")
    trunc = str(tmp_path / "trunc.v2")
    open(trunc, "wb").write(bytes(raw[: secs[-1][2] + 3]))
    with pytest.raises(SaqgError):
        ivf.convert(trunc, str(tmp_path / "out2.index"), "reference")


@pytest.mark.gpu
def test_search_on_v2_index_matches_reference(golden_case, tmp_path):
    v2 = str(tmp_path / "x.v2")
    ivf.convert(golden_case.index_path, v2, "v2")
    idx = ivf.IVF.load(v2)
    ids = idx.search(golden_case.q, golden_case.topk, golden_case.nprobe)
    assert np.array_equal(ids, golden_case.z["search_ids"])
    # save from the device in both formats
    out_v2, out_ref = str(tmp_path / "d.v2"), str(tmp_path / "d.index")
    idx.save(out_v2, format="v2")
    idx.save(out_ref)
    assert open(out_v2, "rb").read() == open(v2, "rb").read()
    assert open(out_ref, "rb").read() == open(golden_case.index_path, "rb").read()
