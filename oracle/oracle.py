"""ctypes wrapper for the CPU oracle (oracle/saq_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by `__graft_entry__.smoke()` and by
the CPU-baseline leg of bench.py, as the checker.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_lib = None

f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
L = C.c_long


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        l = C.CDLL(LIB_PATH)
        l.orc_eigen_sum.restype = C.c_float
        l.orc_eigen_sum.argtypes = [f32p, L]
        l.orc_eigen_sqnorm.restype = C.c_float
        l.orc_eigen_sqnorm.argtypes = [f32p, L]
        l.orc_eigen_sqdist.restype = C.c_float
        l.orc_eigen_sqdist.argtypes = [f32p, f32p, L]
        l.orc_gemv_rowvec.argtypes = [f32p, f32p, L, f32p]
        l.orc_excode_ip.restype = C.c_float
        l.orc_excode_ip.argtypes = [f32p, u8p, L, C.c_int]
        l.orc_pack_excode.argtypes = [u16p, L, C.c_int, u8p]
        l.orc_unpack_excode.argtypes = [u8p, L, C.c_int, u16p]
        l.orc_pack_block.argtypes = [u8p, L, u8p]
        l.orc_colwise_var.argtypes = [f32p, L, L, f32p]
        l.orc_plan.restype = C.c_int
        l.orc_plan.argtypes = [f32p, L, C.c_float, C.c_int, C.c_int, i64p, i64p, C.c_int]
        l.orc_caq_encode.restype = C.c_int
        l.orc_caq_encode.argtypes = [f32p, L, L, C.c_int, C.c_void_p, C.c_int, C.c_float, i32p, f32p]
        l.orc_index_load.restype = C.c_void_p
        l.orc_index_load.argtypes = [C.c_char_p]
        l.orc_index_free.argtypes = [C.c_void_p]
        l.orc_index_info.argtypes = [C.c_void_p, C.POINTER(L), C.POINTER(L), C.POINTER(L), C.POINTER(L)]
        l.orc_probe.argtypes = [C.c_void_p, f32p, L, u32p, f32p]
        l.orc_query_prep.argtypes = [C.c_void_p, f32p, C.c_float, f32p, f32p]
        l.orc_lut.argtypes = [C.c_void_p, f32p, L, C.c_int, u16p, f32p, i32p, f32p]
        l.orc_search.argtypes = [C.c_void_p, f32p, L, L, L, C.c_float, u32p, C.c_void_p, C.c_int]
        l.orc_estimate.restype = L
        l.orc_estimate.argtypes = [C.c_void_p, f32p, L, C.c_float, u32p, f32p, f32p, f32p, L]
        l.orc_tc_approx.restype = L
        l.orc_tc_approx.argtypes = [C.c_void_p, f32p, L, C.c_float, u32p, f64p, L]
        l.orc_build_index.restype = C.c_int
        l.orc_build_index.argtypes = [f32p, L, L, f32p, L, u32p, C.c_float, C.c_int, C.c_int, C.c_int, C.c_float,
                                      C.c_int, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
        _lib = l
    return _lib


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def eigen_sum(x):
    x = _f32(x)
    return float(np.float32(lib().orc_eigen_sum(x, x.size)))


def eigen_sqnorm(x):
    x = _f32(x)
    return float(np.float32(lib().orc_eigen_sqnorm(x, x.size)))


def gemv_rowvec(q, P):
    q, P = _f32(q), _f32(P)
    out = np.empty(q.size, np.float32)
    lib().orc_gemv_rowvec(q, P, q.size, out)
    return out


def excode_ip(q, code_bytes, ex_bits):
    q = _f32(q)
    return np.float32(lib().orc_excode_ip(q, np.ascontiguousarray(code_bytes, np.uint8), q.size, ex_bits))


def pack_excode(values, ex_bits):
    v = np.ascontiguousarray(values, np.uint16)
    D = v.size
    out = np.zeros(D * ex_bits // 8, np.uint8)
    lib().orc_pack_excode(v, D, ex_bits, out)
    return out


def unpack_excode(code_bytes, D, ex_bits):
    out = np.zeros(D, np.uint16)
    lib().orc_unpack_excode(np.ascontiguousarray(code_bytes, np.uint8), D, ex_bits, out)
    return out


def pack_block(short_codes, D):
    out = np.zeros(4 * D, np.uint8)
    lib().orc_pack_block(np.ascontiguousarray(short_codes, np.uint8), D, out)
    return out


def colwise_var(x):
    x = _f32(x)
    out = np.empty(x.shape[1], np.float32)
    lib().orc_colwise_var(x, x.shape[0], x.shape[1], out)
    return out


def plan(var, avg_bits, enable_seg=True, eqseg=0):
    var = _f32(var)
    dims = np.zeros(64, np.int64)
    bits = np.zeros(64, np.int64)
    n = lib().orc_plan(var, var.size, avg_bits, int(enable_seg), eqseg, dims, bits, 64)
    return [(int(dims[i]), int(bits[i])) for i in range(n)]


def caq_encode(resid, bits, cent_unrot=None, rdlmt=6, eps=1e-8):
    r = _f32(resid)
    n, D = r.shape
    codes = np.zeros((n, D), np.int32)
    facs = np.zeros((n, 4), np.float32)
    c = None if cent_unrot is None else _f32(cent_unrot)
    lib().orc_caq_encode(r, n, D, bits, None if c is None else c.ctypes.data, rdlmt, eps, codes, facs)
    return codes, facs


def build_index(path, data, centroids, cids, avg_bits, enable_seg=True, eqseg=0, rotations=None, variance=None,
                rdlmt=6, eps=1e-8, threads=0):
    """IVF::construct + IVF::save with the given rotations (concatenated per segment; None = no rotation).
    threads <= 0: every host thread (the file is the same for any thread count)."""
    x = _f32(data)
    c = _f32(centroids)
    v = None if variance is None else _f32(variance)
    r = None if rotations is None else _f32(rotations)
    rc = lib().orc_build_index(x, x.shape[0], x.shape[1], c, c.shape[0], np.ascontiguousarray(cids, np.uint32),
                               avg_bits, int(enable_seg), eqseg, rdlmt, eps, int(r is not None),
                               None if v is None else v.ctypes.data, None if r is None else r.ctypes.data,
                               path.encode(), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle build failed ({rc})")


class OracleIndex:
    """A reference-format index held by the oracle."""

    def __init__(self, path: str):
        self.h = lib().orc_index_load(path.encode())
        if not self.h:
            raise IOError(f"oracle could not load {path}")
        N, D, K, S = L(), L(), L(), L()
        lib().orc_index_info(self.h, C.byref(N), C.byref(D), C.byref(K), C.byref(S))
        self.N, self.D, self.K, self.S = N.value, D.value, K.value, S.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_index_free(self.h)
            self.h = None

    def probe(self, q, nprobe):
        ids = np.zeros(nprobe, np.uint32)
        d = np.zeros(nprobe, np.float32)
        lib().orc_probe(self.h, _f32(q), nprobe, ids, d)
        return ids, d

    def query_prep(self, q, dims, m=4.0):
        rot = np.zeros(sum(dims), np.float32)
        pr = np.zeros(len(dims), np.float32)
        lib().orc_query_prep(self.h, _f32(q), m, rot, pr)
        return rot, pr

    def lut(self, q, cid, seg, dim, nblocks):
        lut = np.zeros(dim // 4 * 16, np.uint16)
        scal = np.zeros(5, np.float32)
        sums = np.zeros(nblocks * 32, np.int32)
        fast = np.zeros(nblocks * 32, np.float32)
        lib().orc_lut(self.h, _f32(q), cid, seg, lut, scal, sums, fast)
        return lut, scal, sums, fast

    def search(self, q, topk, nprobe, m=4.0, threads=1, with_dists=False):
        q = _f32(q).reshape(-1, self.D)
        ids = np.zeros((q.shape[0], topk), np.uint32)
        d = np.zeros((q.shape[0], topk), np.float32) if with_dists else None
        lib().orc_search(self.h, q, q.shape[0], topk, nprobe, m, ids, None if d is None else d.ctypes.data, threads)
        return (ids, d) if with_dists else ids

    def tc_approx(self, q, nprobe, m=4.0, cap=None):
        """Model of the tensor-core form's approximate distance (exact codes, double):
        (ids, approx) for every vector of the probed clusters, in estimate's order."""
        cap = cap or self.N
        ids = np.zeros(cap, np.uint32)
        apx = np.zeros(cap, np.float64)
        n = lib().orc_tc_approx(self.h, _f32(q), nprobe, m, ids, apx, cap)
        return ids[:n], apx[:n]

    def estimate(self, q, nprobe, m=4.0, cap=None):
        cap = cap or self.N
        ids = np.zeros(cap, np.uint32)
        acc = np.zeros(cap, np.float32)
        fast = np.zeros(cap, np.float32)
        var = np.zeros(cap, np.float32)
        n = lib().orc_estimate(self.h, _f32(q), nprobe, m, ids, acc, fast, var, cap)
        return ids[:n], acc[:n], fast[:n], var[:n]


# ---------------------------------------------------------------- reference
def ref_available() -> bool:
    return os.path.exists(REF_DRIVER)


def run_ref(*args) -> str:
    r = subprocess.run([REF_DRIVER, *map(str, args)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_driver {args[0]} failed ({r.returncode}): {r.stderr[-2000:]}")
    return r.stdout
