"""ctypes binding of the C ABI in include/saqg.h.

The library is loaded from the package's own _lib/ directory (built by
saq_gb300/build.py).  There is no fallback: if the shared library or a CUDA
device is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

SAQG_MEM_HOST = 0
SAQG_MEM_DEVICE = 1
SAQG_STATIC_SCRATCH_BYTES = 16 << 20
SAQG_FORMAT_REFERENCE = 0
SAQG_FORMAT_V2 = 1
SAQG_DIST_L2 = 1

I64 = C.c_int64


class QuantizeConfig(C.Structure):
    _fields_ = [("avg_bits", C.c_float), ("seg_eqseg", C.c_int), ("enable_segmentation", C.c_int),
                ("use_compact_layout", C.c_int), ("random_rotation", C.c_int), ("caq_adj_rd_lmt", C.c_int),
                ("caq_adj_eps", C.c_float)]


class SearcherConfig(C.Structure):
    _fields_ = [("searcher_vars_bound_m", C.c_float), ("dist_type", C.c_int)]


class IndexInfo(C.Structure):
    _fields_ = [("num_data", I64), ("num_dim", I64), ("num_clusters", I64), ("num_segments", C.c_int32),
                ("seg_dim", C.c_int32 * 16), ("seg_bits", C.c_int32 * 16), ("device_bytes", I64)]


class SearchStats(C.Structure):
    _fields_ = [("ms_probe", C.c_float), ("ms_qprep", C.c_float), ("ms_scan", C.c_float), ("ms_total", C.c_float),
                ("probes", I64), ("blocks", I64), ("vectors", I64), ("reranked", I64), ("speculative", I64),
                ("fast_bytes", I64), ("rerank_bytes", I64), ("ms_split", C.c_float),
                ("ms_split_first", C.c_float), ("ms_split_spec", C.c_float), ("ms_split_replay", C.c_float),
                ("probe_exact", I64), ("probe_full", I64), ("probe_full_ties", I64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class TcStats(C.Structure):
    _fields_ = [("ms_probe", C.c_float), ("ms_pairs", C.c_float), ("ms_contract", C.c_float),
                ("ms_select", C.c_float), ("ms_rerank", C.c_float), ("pairs", I64), ("candidates", I64),
                ("tiles", I64), ("flops", I64), ("mma_flops", I64), ("code_bytes", I64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class TuneReport(C.Structure):
    _fields_ = [("form", C.c_int), ("scan_mode", C.c_int), ("defer_blocks", C.c_int), ("first_blocks", C.c_int),
                ("pairs_per_chunk", C.c_int), ("spec_levels", C.c_int), ("candidates", C.c_int),
                ("default_ms", C.c_float),
                ("tuned_ms", C.c_float)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class GraphConfig(C.Structure):
    _fields_ = [("form", C.c_int), ("nprobe_per_query", C.c_void_p), ("topk_per_query", C.c_void_p),
                ("shortlist", I64), ("candidate_capacity", I64), ("autotune", C.c_int)]


SAQG_FORM_EXACT = 0
SAQG_FORM_TC = 1


class SaqgError(RuntimeError):
    pass


_lib = None

class ServerConfig(C.Structure):
    _fields_ = [("max_batch", C.c_int32), ("max_inflight", C.c_int32), ("max_topk", C.c_int32),
                ("max_nprobe", C.c_int32), ("max_wait_us", C.c_int32), ("searcher_vars_bound_m", C.c_float),
                ("mem_budget_bytes", I64), ("form", C.c_int32), ("shortlist", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", I64), ("completed", I64), ("batches", I64), ("admission_shrinks", I64),
                ("max_batch_seen", C.c_int32), ("max_inflight_seen", C.c_int32), ("mean_batch", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS = {
    "saqg_version": (C.c_int, []),
    "saqg_last_error": (C.c_char_p, []),
    "saqg_kernel_launches": (I64, []),
    "saqg_index_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "saqg_index_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "saqg_index_save_v2": (C.c_int, [C.c_void_p, C.c_char_p]),
    "saqg_index_convert": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int]),
    "saqg_index_free": (C.c_int, [C.c_void_p]),
    "saqg_index_get_info": (C.c_int, [C.c_void_p, C.POINTER(IndexInfo)]),
    "saqg_index_construct": (C.c_int, [C.c_void_p, I64, I64, C.c_void_p, I64, C.c_void_p, C.POINTER(QuantizeConfig),
                                       C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]),
    "saqg_search": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, C.POINTER(SearcherConfig), C.c_void_p,
                              C.c_void_p, C.c_int, C.c_void_p]),
    "saqg_search_ex": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, C.POINTER(SearcherConfig), C.c_void_p,
                                 C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "saqg_search_batch": (C.c_int, [C.c_void_p, C.c_void_p, I64, C.c_void_p, C.c_void_p, I64, I64,
                                    C.POINTER(SearcherConfig), C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                    C.c_void_p]),
    "saqg_search_static": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, C.POINTER(SearcherConfig), C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
    "saqg_search_tc": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, I64, C.POINTER(SearcherConfig), C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(TcStats)]),
    "saqg_search_tc_batch": (C.c_int, [C.c_void_p, C.c_void_p, I64, C.c_void_p, C.c_void_p, I64, I64, I64,
                                       C.POINTER(SearcherConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.POINTER(TcStats)]),
    "saqg_search_graph_create": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, C.POINTER(SearcherConfig),
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "saqg_search_graph_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "saqg_search_graph_free": (C.c_int, [C.c_void_p]),
    "saqg_server_create": (C.c_int, [C.c_void_p, C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "saqg_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_uint64)]),
    "saqg_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                   C.c_int32]),
    "saqg_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    "saqg_server_run_trace": (C.c_int, [C.c_void_p, C.c_void_p, I64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                        C.c_void_p, C.c_void_p, C.c_void_p]),
    "saqg_server_free": (C.c_int, [C.c_void_p]),
    "saqg_estimate": (C.c_int, [C.c_void_p, C.c_void_p, I64, C.POINTER(SearcherConfig), C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, I64, C.POINTER(I64)]),
    "saqg_plan": (C.c_int, [C.c_void_p, I64, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                            C.POINTER(C.c_int)]),
    "saqg_autotune": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, I64, C.c_int, C.c_void_p, C.c_void_p,
                                C.c_void_p]),
    "saqg_search_graph_create_ex": (C.c_int, [C.c_void_p, C.c_void_p, I64, I64, I64, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "saqg_search_graph_status": (C.c_int, [C.c_void_p, C.c_void_p]),
    "saqg_plan_gpu": (C.c_int, [C.c_void_p, I64, C.c_float, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "saqg_caq_encode": (C.c_int, [C.c_void_p, I64, I64, C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_void_p,
                                  C.c_void_p, C.c_int, C.c_void_p]),
}


def lib_path() -> str:
    return LIB


def load(build_if_missing: bool = False):
    """Load libsaqg.so (optionally building it first); raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        if not build_if_missing:
            raise SaqgError(f"native library {LIB} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        from .build import build
        build()
    l = C.CDLL(LIB)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args
    _lib = l
    return l


def check(rc: int) -> None:
    if rc != 0:
        msg = _lib.saqg_last_error().decode(errors="replace") if _lib else "unknown"
        raise SaqgError(f"saqg error {rc}: {msg}")
