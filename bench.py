"""Benchmark of the SAQ search hot path on one GB300 (or N replicas).

Workload (default): 10M x 1024 unit-norm vectors, anisotropic spectrum, PCA,
16,384 clusters with Zipf(1.1) sizes, SAQ B=4 with segmentation, k=10, the
smallest nprobe that reaches recall@10 >= 0.95 against exact FP64 ground truth.

  value   batched QPS of the exact form (saqg_search): one call answers a batch
          of 4096 queries already in HBM, every answer bit-identical to an
          independent IVF::search call; the L2 cache is flushed between steps.
  e2e     the same batch through the C ABI with host buffers: host->device copy
          of the queries and device->host copy of ids + distances inside the
          timed region.
  roofline  the exact form's scan phase: compulsory bytes (each distinct probed
          cluster's codes once + every re-rank) / its CUDA-event duration (from
          calls with statistics, outside the timed steps).
  batched_tc  the batched tensor-core form (saqg_search_tc, a stated-recall
          variant: dense contraction, shortlist, exact re-rank) with the
          contraction's roofline on the codes' own (packed) bytes.
  plain   the plain single-query drop-in: one query per call (QPS, p50, p99).
  c1, c2  the single-query configurations: 100k x 960 Gaussian mixture (nprobe
          32) and 1M x 1024 anisotropic (B 1.5 / 4, with and without
          segmentation, nprobe 16-128): plain QPS, p50 / p99, recall@10 against
          FP64, GPU encode vectors/s, and the CPU oracle's search and encode
          rates on the same data beside them.
  cpu_baseline  the CPU oracle (a port of the reference's search) on the host
          cores, on a bounded sample of the same queries and index.

--impl reference times the CPU implementation alone on an index that the CPU
oracle's builder writes (same data, plan and rotations, so the same file; this
process never loads the GPU library) and prints its line with
"impl": "reference".  Multi-GPU (--gpus N via torchrun) runs N independent
replicas (the search has no exchange step): value = all ranks' queries / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "QPS at recall@10≥0.95 (10M×1024, B=4): batched vs plain GPU; p99 ms; HBM %"
NPROBE_GRID = [16, 24, 32, 48, 64, 96, 128, 160, 192, 256]
CACHE_VERSION = 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--dim", type=int, default=1024)
    ap.add_argument("--clusters", type=int, default=16384)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--topk", type=int, default=10)
    ap.add_argument("--bits", type=float, default=4.0)
    ap.add_argument("--gt-queries", type=int, default=1000)
    ap.add_argument("--plain-queries", type=int, default=256)
    ap.add_argument("--target-recall", type=float, default=0.95)
    ap.add_argument("--cache", default=os.path.join(tempfile.gettempdir(), "saqg_bench_cache"))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--sigma", type=float, default=0.2)
    ap.add_argument("--noise-alpha", type=float, default=1.6)
    ap.add_argument("--query-clusters", default="uniform", choices=["uniform", "zipf"])
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[20000, 50000, 100000, 200000])
    ap.add_argument("--serve-seconds", type=float, default=0.3)
    ap.add_argument("--tc-shortlist", type=int, default=40)
    ap.add_argument("--only", default="all", choices=["all", "precision", "c1", "c2", "kernels"],
                    help="precision / c1 / c2: only that leg's measurements (its own JSON line); kernels: the "
                         "workload at --n / --clusters, two exact batched calls then two tensor-core calls and "
                         "nothing else (the command the kernel profiles capture)")
    ap.add_argument("--configs", type=int, default=1, help="0: skip the c1 / c2 legs in the full run")
    ap.add_argument("--c2-n", type=int, default=1_000_000)
    ap.add_argument("--c2-queries", type=int, default=400, help="single queries timed per (B, seg, nprobe)")
    ap.add_argument("--c1-queries", type=int, default=1000)
    ap.add_argument("--precision-bits", type=int, nargs="*", default=[6, 8])
    ap.add_argument("--precision-n", type=int, default=1_000_000)
    ap.add_argument("--precision-dim", type=int, default=1536)
    ap.add_argument("--precision-clusters", type=int, default=4096)
    ap.add_argument("--precision-nprobe", type=int, default=32)
    ap.add_argument("--precision-batches", type=int, nargs="*", default=[256, 2048])
    return ap.parse_args()


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def time_calls(torch, fn, flush, steps, warmup=2):
    """Mean ms of `fn` on the current stream (CUDA events, L2 flushed before each call)."""
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    ms = []
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.mean(ms)), ms


def overlap(a_ids, b_ids, k):
    hit = 0
    for x, y in zip(a_ids, b_ids):
        hit += len(set(x[:k].tolist()) & set(y[:k].tolist()))
    return hit / (k * len(a_ids))


def exact_dists(torch, x, q, ids):
    """FP64 squared L2 from each query to each of its returned ids."""
    with torch.no_grad():
        idx = torch.as_tensor(ids.astype(np.int64), device=x.device)
        v = x[idx.reshape(-1)].double().reshape(ids.shape[0], ids.shape[1], -1)
        return ((v - q.double()[:, None, :]) ** 2).sum(-1).cpu().numpy()


def precision_leg(a, torch, flush, log):
    """Precision form: B=6 / 8 CAQ codes at 1M x 1536 (spectrum i^-1), the
    ex-code contraction on the tensor cores (saqg_search_tc) beside the FP32
    CUDA-core search (saqg_search) on the same batches."""
    import ctypes as C
    from saq_gb300 import _native as N, ivf, workloads
    t0 = time.time()
    nmax = max(a.precision_batches)
    wl = workloads.zipf_aniso(a.precision_n, a.precision_dim, a.precision_clusters, nq=nmax, s=0.0, alpha=1.0,
                              sigma=a.sigma, noise_alpha=1.0, seed=1, query_clusters="uniform")
    gt = workloads.ground_truth(wl.x, wl.q, 10)
    log(f"precision workload generated in {time.time() - t0:.1f}s")
    peak_tf, peak_tf_kind = bf16_peak()
    hbm, hbm_kind = peaks()
    out = {"workload": f"{a.precision_n // 1_000_000}M x {a.precision_dim}, unit-norm, spectrum i^-1, "
                       f"{a.precision_clusters} clusters (equal sizes), CAQ (no segmentation), k=10, "
                       f"nprobe {a.precision_nprobe}, shortlist {a.tc_shortlist}",
           "operands": "codes BF16 (exact integers), queries BF16, FP32 accumulation in TMEM (tcgen05.mma kind::f16)",
           "configs": []}
    for bits in a.precision_bits:
        # the rotation (one orthogonal matrix per segment, as the reference's Rotator
        # draws at index set-up) is made before the timed build, as for the other legs
        rots = workloads.rotations(ivf.plan(wl.variance, float(bits), False), ROT_SEED)
        t0 = time.time()
        index = ivf.IVF(a.precision_n, a.precision_dim, a.precision_clusters,
                        ivf.QuantizeConfig(avg_bits=float(bits), enable_segmentation=False))
        index.set_variance(wl.variance)
        index.construct(wl.x, wl.centroids.cpu().numpy(), wl.cids.cpu().numpy().astype(np.uint32), rotations=rots)
        torch.cuda.synchronize()
        build_s = time.time() - t0
        lib = index.lib
        cfg = {"bits": bits, "encode_vectors_per_s": a.precision_n / build_s, "plan": index.info()["plan"],
               "batches": []}
        log(f"precision B={bits}: index built in {build_s:.1f}s")
        for B in a.precision_batches:
            q = wl.q[:B].contiguous()
            ids_tc = torch.empty((B, 10), dtype=torch.int32, device="cuda")
            d_tc = torch.empty((B, 10), dtype=torch.float32, device="cuda")
            ap_tc = torch.empty((B, 10), dtype=torch.float32, device="cuda")
            st = N.TcStats()
            scfg = ivf.SearcherConfig().to_c()
            sptr = C.c_void_p(torch.cuda.current_stream().cuda_stream)

            def tc(with_stats=False):
                N.check(lib.saqg_search_tc(index._h, q.data_ptr(), B, 10, a.precision_nprobe, a.tc_shortlist,
                                           C.byref(scfg), ids_tc.data_ptr(), d_tc.data_ptr(), ap_tc.data_ptr(),
                                           N.SAQG_MEM_DEVICE, sptr, C.byref(st) if with_stats else None))
            ids_c = torch.empty((B, 10), dtype=torch.int32, device="cuda")
            d_c = torch.empty((B, 10), dtype=torch.float32, device="cuda")

            def core():
                N.check(lib.saqg_search(index._h, q.data_ptr(), B, 10, a.precision_nprobe, C.byref(scfg),
                                        ids_c.data_ptr(), d_c.data_ptr(), N.SAQG_MEM_DEVICE, sptr))
            ms_tc, _ = time_calls(torch, tc, flush, 5)
            ms_core, _ = time_calls(torch, core, flush, 5)
            cst = N.SearchStats()
            flush.zero_()
            N.check(lib.saqg_search_ex(index._h, q.data_ptr(), B, 10, a.precision_nprobe, C.byref(scfg),
                                       ids_c.data_ptr(), d_c.data_ptr(), N.SAQG_MEM_DEVICE, sptr, C.byref(cst), None))
            core_stages = {"ms_probe": cst.ms_probe, "ms_qprep": cst.ms_qprep, "ms_scan": cst.ms_scan,
                           "probe_full": cst.probe_full, "probe_full_ties": cst.probe_full_ties,
                           "probe_exact": cst.probe_exact}
            flush.zero_()
            tc(True)
            torch.cuda.synchronize()
            it = ids_tc.cpu().numpy().view(np.uint32)
            ic = ids_c.cpu().numpy().view(np.uint32)
            dt = d_tc.cpu().numpy()
            apx = ap_tc.cpu().numpy()
            ex = exact_dists(torch, wl.x, q, it)
            rel_est = np.abs(dt.astype(np.float64) - ex) / np.maximum(ex, 1e-12)
            rel_apx = np.abs(apx.astype(np.float64) - ex) / np.maximum(ex, 1e-12)
            rel_apx_est = np.abs(apx.astype(np.float64) - dt) / np.maximum(np.abs(dt.astype(np.float64)), 1e-12)
            s = st.as_dict()
            tflops = s["flops"] / (s["ms_contract"] / 1e3) / 1e12
            row = {"batch": B, "tc_qps": B / (ms_tc / 1e3), "tc_ms": ms_tc, "core_qps": B / (ms_core / 1e3),
                   "core_ms": ms_core, "tc_over_core": ms_core / ms_tc,
                   "recall@10_tc_vs_core": overlap(it, ic, 10),
                   "recall@10_tc_vs_fp64": workloads.recall_at(it, gt[:B], 10),
                   "recall@10_core_vs_fp64": workloads.recall_at(ic, gt[:B], 10),
                   "dist_rel_err_vs_fp64": {"median": float(np.median(rel_est)), "p99": float(np.percentile(rel_est, 99)),
                                            "note": "returned distances (the exact search's estimator) vs FP64 |x-q|^2"},
                   "tc_approx_rel_err_vs_fp64": {"median": float(np.median(rel_apx)),
                                                 "p99": float(np.percentile(rel_apx, 99))},
                   "tc_approx_rel_err_vs_fp32_estimator": {"median": float(np.median(rel_apx_est)),
                                                           "p99": float(np.percentile(rel_apx_est, 99))},
                   "stages_ms": {k: s[k] for k in ("ms_probe", "ms_pairs", "ms_contract", "ms_select", "ms_rerank")},
                   "core_stages": core_stages,
                   "contract_roofline": {"tensor_tflops": tflops, "tensor_peak": peak_tf, "tensor_frac": tflops / peak_tf,
                                         "tensor_peak_kind": peak_tf_kind,
                                         "issued_tflops": s["mma_flops"] / (s["ms_contract"] / 1e3) / 1e12,
                                         "code_gbs": s["code_bytes"] / (s["ms_contract"] / 1e3) / 1e9,
                                         "hbm_peak": hbm, "hbm_frac": s["code_bytes"] / (s["ms_contract"] / 1e3) / 1e9 / hbm,
                                         "flops": s["flops"], "code_bytes": s["code_bytes"], "tiles": s["tiles"]}}
            cfg["batches"].append(row)
            log(f"precision B={bits} batch {B}: tc {row['tc_qps']:.0f} q/s, core {row['core_qps']:.0f} q/s, "
                f"recall tc/core {row['recall@10_tc_vs_core']:.4f}, contract {s['ms_contract']:.3f} ms "
                f"({tflops:.1f} TF/s, {row['contract_roofline']['code_gbs']:.0f} GB/s)")
        out["configs"].append(cfg)
        del index
        torch.cuda.empty_cache()
    del wl
    torch.cuda.empty_cache()
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in csv.reader(io.StringIO(getattr(self, "out", ""))):
            if len(row) < 9:
                continue
            try:
                sm.append(float(row[1]))
                smax.append(float(row[2]))
            except ValueError:
                continue
            for nm, v in zip(names, row[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cache_paths(a, builder):
    """Per-box cache of the built index; `builder` is "gpu" (this library) or
    "oracle" (the CPU oracle's builder, used by the reference arm).  Both write
    the same bytes from the same data, plan and rotations."""
    key = (f"v{CACHE_VERSION}_n{a.n}_d{a.dim}_k{a.clusters}_b{a.bits}_s{a.sigma}_na{a.noise_alpha}"
           f"_q{a.query_clusters}_seed0")
    d = os.path.join(a.cache, key, builder)
    os.makedirs(d, exist_ok=True)
    return d, os.path.join(d, "index.saq"), os.path.join(d, "meta.json")


def build_workload(a, torch):
    from saq_gb300 import workloads
    return workloads.zipf_aniso(a.n, a.dim, a.clusters, nq=max(a.batch, a.gt_queries, a.plain_queries), seed=0,
                                sigma=a.sigma, noise_alpha=a.noise_alpha, query_clusters=a.query_clusters)


ROT_SEED = 1


def tune_nprobe(search, gt, topk, clusters, target):
    """Smallest nprobe on the grid whose recall@topk reaches the target."""
    from saq_gb300 import workloads
    curve = {}
    for npb in NPROBE_GRID:
        if npb > clusters:
            break
        r = workloads.recall_at(search(npb), gt, topk)
        curve[npb] = r
        if r >= target:
            return npb, r, curve
    return max(curve), curve[max(curve)], curve


def get_index_and_meta(a, torch, wl, log):
    """Index built on the GPU (or loaded from this box's cache), ground truth and the tuned nprobe."""
    from saq_gb300 import ivf, workloads
    cdir, ipath, mpath = cache_paths(a, "gpu")
    meta = json.load(open(mpath)) if os.path.exists(mpath) and os.path.exists(ipath) else None
    t0 = time.time()
    if meta:
        index = ivf.IVF.load(ipath)
        log(f"index loaded from cache in {time.time() - t0:.1f}s")
    else:
        plan = ivf.plan(wl.variance, a.bits, True)
        rots = workloads.rotations(plan, ROT_SEED)
        cfg = ivf.QuantizeConfig(avg_bits=a.bits, enable_segmentation=True)
        index = ivf.IVF(a.n, a.dim, a.clusters, cfg)
        index.set_variance(wl.variance)
        index.construct(wl.x, wl.centroids.cpu().numpy(), wl.cids.cpu().numpy().astype(np.uint32), rotations=rots)
        torch.cuda.synchronize()
        build_s = time.time() - t0
        log(f"index built on the GPU in {build_s:.1f}s plan={index.info()['plan']}")
        gt = workloads.ground_truth(wl.x, wl.q[: a.gt_queries], a.topk)
        np.save(os.path.join(cdir, "gt.npy"), gt)
        qg = wl.q[: a.gt_queries].contiguous()
        nprobe, rec, curve = tune_nprobe(lambda npb: index.search(qg, a.topk, npb).cpu().numpy().view(np.uint32),
                                         gt, a.topk, a.clusters, a.target_recall)
        index.save(ipath)
        meta = dict(nprobe=nprobe, recall=rec, curve=curve, build_s=build_s, plan=index.info()["plan"])
        json.dump(meta, open(mpath, "w"))
        log(f"nprobe={nprobe} recall@{a.topk}={rec:.4f} curve={curve}")
    meta["gt"] = np.load(os.path.join(cdir, "gt.npy"))
    return index, ipath, meta


def get_oracle_index(a, torch, wl, log):
    """The reference arm's index: written by the CPU oracle's builder on every
    host thread (same data, plan and rotations as the GPU arm, so the same
    bytes); nprobe tuned with the oracle's own search.  Nothing here touches
    the GPU library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from saq_gb300 import workloads
    cdir, ipath, mpath = cache_paths(a, "oracle")
    meta = json.load(open(mpath)) if os.path.exists(mpath) and os.path.exists(ipath) else None
    if not meta:
        t0 = time.time()
        plan = O.plan(wl.variance, a.bits, True, 0)
        rots = workloads.rotations(plan, ROT_SEED)
        xh = wl.x.cpu().numpy()
        O.build_index(ipath, xh, wl.centroids.cpu().numpy(), wl.cids.cpu().numpy().astype(np.uint32), a.bits, True,
                      0, rots, variance=wl.variance, threads=0)
        del xh
        build_s = time.time() - t0
        log(f"index built by the CPU oracle in {build_s:.1f}s ({os.cpu_count()} threads) plan={plan}")
        gt = workloads.ground_truth(wl.x, wl.q[: a.gt_queries], a.topk)
        np.save(os.path.join(cdir, "gt.npy"), gt)
        oi = O.OracleIndex(ipath)
        qg = wl.q[: a.gt_queries].cpu().numpy()
        nprobe, rec, curve = tune_nprobe(lambda npb: oi.search(qg, a.topk, npb, threads=os.cpu_count() or 1),
                                         gt, a.topk, a.clusters, a.target_recall)
        del oi
        meta = dict(nprobe=nprobe, recall=rec, curve=curve, build_s=build_s, plan=plan)
        json.dump(meta, open(mpath, "w"))
        log(f"nprobe={nprobe} recall@{a.topk}={rec:.4f} curve={curve}")
    meta["gt"] = np.load(os.path.join(cdir, "gt.npy"))
    return ipath, meta


def cpu_search_rate(ipath, q, topk, nprobe, seconds, threads, oi=None):
    """Oracle (CPU port of the reference search) QPS on a bounded sample: single-query
    tasks on `threads` host threads (src/test_qps.cpp's thread pool)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    oi = oi or O.OracleIndex(ipath)
    probe = q[:threads]
    t0 = time.time()
    oi.search(probe, topk, nprobe, threads=threads)
    per_q = (time.time() - t0) / len(probe)
    nsamp = int(min(len(q), max(threads, seconds / max(per_q, 1e-6))))
    sample = q[:nsamp]
    t0 = time.time()
    ids = oi.search(sample, topk, nprobe, threads=threads)
    dt = time.time() - t0
    return nsamp / dt, nsamp, dt, ids, oi


def plain_latencies(torch, lib, index, q, topk, nprobe):
    """Device time (CUDA events, synchronised per call) of one saqg_search call
    per query with nq = 1, the plain drop-in; returns (ms per query, ids)."""
    import ctypes as C
    from saq_gb300 import _native as N, ivf
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    scfg = ivf.SearcherConfig().to_c()
    P = q.shape[0]
    ids = torch.empty((P, topk), dtype=torch.int32, device="cuda")
    dd = torch.empty((P, topk), dtype=torch.float32, device="cuda")

    def one(i):
        N.check(lib.saqg_search(index._h, q[i].data_ptr(), 1, topk, nprobe, C.byref(scfg), ids[i].data_ptr(),
                                dd[i].data_ptr(), N.SAQG_MEM_DEVICE, sptr))
    for i in range(min(8, P)):
        one(i)
    torch.cuda.synchronize()
    lat = []
    for i in range(P):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        one(i)
        e1.record(stream)
        e1.synchronize()
        lat.append(e0.elapsed_time(e1))
    return np.array(lat), ids.cpu().numpy().view(np.uint32)


def plain_threads(torch, lib, index, qh, topk, nprobe, threads, seconds=1.0):
    """The plain drop-in driven the way the reference's drivers drive IVF::search
    (src/test_qps.cpp:77-84): `threads` host threads, each answering one query
    per call on its own stream, with host buffers (the call copies the query in
    and the result out).  Returns (queries/s over the wall clock, queries)."""
    import ctypes as C
    import threading
    from saq_gb300 import _native as N, ivf
    scfg = ivf.SearcherConfig().to_c()
    streams = [torch.cuda.Stream() for _ in range(threads)]
    qpin = torch.from_numpy(np.ascontiguousarray(qh)).pin_memory()
    n_all = qpin.shape[0]
    outs = [(torch.empty((1, topk), dtype=torch.int32).pin_memory(),
             torch.empty((1, topk), dtype=torch.float32).pin_memory()) for _ in range(threads)]

    def run(count):
        done = [0] * threads

        def worker(t):
            sp = C.c_void_p(streams[t].cuda_stream)
            ih, dh = outs[t]
            for j in range(t, count, threads):
                N.check(lib.saqg_search(index._h, qpin[j % n_all].data_ptr(), 1, topk, nprobe, C.byref(scfg),
                                        ih.data_ptr(), dh.data_ptr(), N.SAQG_MEM_HOST, sp))
                done[t] += 1
        th = [threading.Thread(target=worker, args=(t,)) for t in range(threads)]
        t0 = time.perf_counter()
        for x in th:
            x.start()
        for x in th:
            x.join()
        return time.perf_counter() - t0, sum(done)
    dt, n = run(threads * 4)  # warm-up: every thread's context and stream
    count = max(threads * 8, int(n / max(dt, 1e-6) * seconds))
    dt, n = run(count)
    return n / dt, n


def cpu_encode_rate(xh, cent, cids, var, bits, seg, rots, want, tmpdir):
    """The CPU oracle's builder (IVF::construct restated) on every host thread,
    on the first clusters holding at least `want` vectors: vectors/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    sizes = np.bincount(cids, minlength=cent.shape[0])
    kk = int(np.searchsorted(np.cumsum(sizes), min(want, len(cids)))) + 1
    kk = min(kk, cent.shape[0])
    sel = cids < kk
    xs = np.ascontiguousarray(xh[sel])
    path = os.path.join(tmpdir, "cpu_encode.index")
    t0 = time.time()
    O.build_index(path, xs, cent[:kk], cids[sel], bits, seg, 0, rots, variance=var, threads=0)
    dt = time.time() - t0
    os.remove(path)
    return {"value": len(xs) / dt, "unit": "vectors/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{len(xs)} vectors ({kk} clusters) built into an index file in {dt:.1f}s"}


def single_query_config(a, torch, log, wl, name, variants, nprobes, nq_time, tmpdir):
    """One single-query configuration: per (B, segmentation) a GPU-built index,
    per nprobe the plain drop-in's QPS / p50 / p99 / recall@10 against FP64, and
    the CPU oracle's search (all host threads, single-query tasks) and encode
    rates on the same data."""
    from saq_gb300 import ivf, workloads
    threads = os.cpu_count() or 1
    gt = workloads.ground_truth(wl.x, wl.q[:nq_time], 10)
    qd = wl.q[:nq_time].contiguous()
    qh = qd.cpu().numpy()
    xh = None
    cent = wl.centroids.cpu().numpy()
    cids = wl.cids.cpu().numpy().astype(np.uint32)
    out = {"workload": wl.name, "n": int(wl.x.shape[0]), "dim": int(wl.x.shape[1]),
           "clusters": int(cent.shape[0]), "k": 10, "queries_timed": nq_time,
           "timing": "qps / p50 / p99: plain single-query saqg_search per call on one stream (CUDA events, "
                     "synchronised per call), QPS = queries / sum of latencies; threads_qps: one query per call "
                     "from as many host threads as the CPU baseline uses, each on its own stream, host buffers "
                     "(src/test_qps.cpp's driver), over the wall clock", "variants": []}
    for bits, seg in variants:
        plan = ivf.plan(wl.variance, bits, seg)
        rots = workloads.rotations(plan, ROT_SEED)
        t0 = time.time()
        index = ivf.IVF(wl.x.shape[0], wl.x.shape[1], cent.shape[0],
                        ivf.QuantizeConfig(avg_bits=bits, enable_segmentation=seg))
        index.set_variance(wl.variance)
        index.construct(wl.x, cent, cids, rotations=rots)
        torch.cuda.synchronize()
        enc_s = time.time() - t0
        ipath = os.path.join(tmpdir, f"{name}_{bits}_{int(seg)}.index")
        index.save(ipath)
        row = {"bits": bits, "segmentation": seg, "plan": plan,
               "encode_gpu": {"value": wl.x.shape[0] / enc_s, "unit": "vectors/s",
                              "note": "saqg_index_construct from device-resident data, rotation included"},
               "nprobe": []}
        if xh is None:
            xh = wl.x.cpu().numpy()
        row["encode_cpu_baseline"] = cpu_encode_rate(xh, cent, cids, wl.variance, bits, seg, rots,
                                                     min(100_000, wl.x.shape[0]), tmpdir)
        oi = None
        for npb in nprobes:
            lat, ids = plain_latencies(torch, index.lib, index, qd, 10, npb)
            r, ns, dt, cids_cpu, oi = cpu_search_rate(ipath, qh, 10, npb, a.cpu_seconds / 10, threads, oi)
            tq, tn = plain_threads(torch, index.lib, index, qh, 10, npb, threads)
            pt = {"nprobe": npb, "qps": len(lat) / (lat.sum() / 1e3), "p50_ms": float(np.median(lat)),
                  "p99_ms": float(np.percentile(lat, 99)), "recall@10": round(workloads.recall_at(ids, gt, 10), 4),
                  "threads_qps": tq, "threads": threads, "threads_over_cpu": None,
                  "cpu_baseline": {"value": r, "unit": "queries/s", "cores": threads, "kind": "port",
                                   "sample": f"{ns} single-query tasks in {dt:.2f}s"},
                  "ids_equal_cpu": bool(np.array_equal(cids_cpu[:ns], ids[:ns]))}
            pt["threads_over_cpu"] = tq / r
            row["nprobe"].append(pt)
            log(f"{name} B={bits} seg={seg} nprobe={npb}: {pt['qps']:.0f} q/s p50 {pt['p50_ms']:.3f} ms "
                f"p99 {pt['p99_ms']:.3f} ms recall {pt['recall@10']:.4f}; {threads} threads {tq:.0f} q/s; "
                f"cpu {r:.0f} q/s")
        r1, ns1, dt1, _, _ = cpu_search_rate(ipath, qh, 10, nprobes[0], 1.0, 1, oi)
        del oi
        row["cpu_single_thread"] = {"value": r1, "nprobe": nprobes[0], "sample": f"{ns1} queries in {dt1:.2f}s"}
        row["encode_over_cpu"] = row["encode_gpu"]["value"] / row["encode_cpu_baseline"]["value"]
        log(f"{name} B={bits} seg={seg}: encode GPU {row['encode_gpu']['value']:.0f} v/s, "
            f"CPU {row['encode_cpu_baseline']['value']:.0f} v/s")
        out["variants"].append(row)
        os.remove(ipath)
        del index
        torch.cuda.empty_cache()
    return out


def c1_leg(a, torch, log, tmpdir):
    from saq_gb300 import workloads
    t0 = time.time()
    wl = workloads.gaussian_mixture_ivf(100_000, 960, 1024, 0.5, nq=a.c1_queries, k=1024, iters=20, seed=0)
    log(f"c1 workload (k-means 1024 x 20 iterations on the GPU) in {time.time() - t0:.1f}s")
    out = single_query_config(a, torch, log, wl, "c1", [(4.0, True)], [32], a.c1_queries, tmpdir)
    out["data"] = ("Gaussian mixture: 1,024 centres ~ N(0,1)^960, point = centre + N(0, 0.5^2), seed 0; PCA; "
                   "k-means 1,024 clusters x 20 iterations; queries from the same mixture")
    del wl
    torch.cuda.empty_cache()
    return out


def c2_leg(a, torch, log, tmpdir):
    from saq_gb300 import workloads
    t0 = time.time()
    wl = workloads.aniso_ivf(a.c2_n, 1024, 0.8, nq=a.c2_queries, k=4096, iters=8, seed=0)
    log(f"c2 workload (k-means 4096 x 8 iterations on the GPU) in {time.time() - t0:.1f}s")
    out = single_query_config(a, torch, log, wl, "c2", [(1.5, True), (1.5, False), (4.0, True), (4.0, False)],
                              [16, 32, 64, 128], a.c2_queries, tmpdir)
    out["data"] = ("unit-norm rows, random orthogonal basis, per-axis variance ~ i^-0.8, seed 0; PCA; "
                   "k-means 4,096 clusters x 8 iterations")
    del wl
    torch.cuda.empty_cache()
    return out


def exact_bytes(plan, sizes, probes, rerank_bytes, dim):
    """Compulsory bytes of one exact batched search: per scanned block of each
    distinct probed cluster 32 x (dim/8 over the coded segments + 4 bytes of |o|
    per segment), 4 x dim per distinct probed centroid, and the re-rank's bytes."""
    nblk = (sizes + 31) // 32
    per_lane = sum(4 + (d // 8 if b else 0) for d, b in plan)
    distinct = np.unique(probes)
    return int((nblk[distinct] * 32 * per_lane).sum() + len(distinct) * 4 * dim + rerank_bytes)


def contraction_bytes(plan, sizes, probes, pairs, candidates):
    """Algorithmic bytes of one contraction launch (the codes' own width): every
    distinct probed cluster's codes once at their packed width (sum over segments
    of dim x bits / 8) with |o| and the rescale factor per coded segment, the
    queries' rows (BF16) of every (query, cluster) pair, and the approximate
    distances written."""
    dtot = sum(d for d, _ in plan)
    packed_pv = sum(d * b / 8 + (8 if b else 4) for d, b in plan)
    n_distinct = int(sizes[np.unique(probes)].sum())
    return int(n_distinct * packed_pv + 2 * pairs * dtot + 4 * candidates)


def kernels_leg(a, torch, log):
    """The batched calls alone, for kernel profiles: the index of the workload
    (raw vectors freed once it is built), two exact calls (saqg_search) and two
    tensor-core calls (saqg_search_tc) on one batch, in that order, with the
    built-in launch shapes.  Prints their CUDA-event times."""
    import ctypes as C
    from saq_gb300 import _native as N, ivf, workloads
    wl = build_workload(a, torch)
    plan = ivf.plan(wl.variance, a.bits, True)
    index = ivf.IVF(a.n, a.dim, a.clusters, ivf.QuantizeConfig(avg_bits=a.bits, enable_segmentation=True))
    index.set_variance(wl.variance)
    index.construct(wl.x, wl.centroids.cpu().numpy(), wl.cids.cpu().numpy().astype(np.uint32),
                    rotations=workloads.rotations(plan, ROT_SEED))
    q = wl.q[:a.batch].contiguous()
    sizes = np.bincount(wl.cids.cpu().numpy(), minlength=a.clusters)
    del wl
    torch.cuda.empty_cache()
    B, k, npb = q.shape[0], a.topk, 16
    ids = torch.empty((B, k), dtype=torch.int32, device="cuda")
    dd = torch.empty((B, k), dtype=torch.float32, device="cuda")
    scfg = ivf.SearcherConfig().to_c()
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    out = {"workload": f"{a.n} x {a.dim}, {a.clusters} clusters, B={a.bits:g} segmented, batch {B}, nprobe {npb}",
           "plan": plan, "exact_ms": [], "tc_ms": []}
    for form in ("exact", "tc"):
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if form == "exact":
                N.check(index.lib.saqg_search(index._h, q.data_ptr(), B, k, npb, C.byref(scfg), ids.data_ptr(),
                                              dd.data_ptr(), N.SAQG_MEM_DEVICE, sptr))
            else:
                N.check(index.lib.saqg_search_tc(index._h, q.data_ptr(), B, k, npb, a.tc_shortlist, C.byref(scfg),
                                                 ids.data_ptr(), dd.data_ptr(), None, N.SAQG_MEM_DEVICE, sptr, None))
            e1.record(stream)
            e1.synchronize()
            out[f"{form}_ms"].append(e0.elapsed_time(e1))
    # byte counts of these calls (one more call of each form with statistics,
    # after the ones a capture skips and takes), to scale a capture's DRAM bytes
    # to the full workload
    st, tst = N.SearchStats(), N.TcStats()
    probes = torch.empty((B, npb), dtype=torch.int32, device="cuda")
    N.check(index.lib.saqg_search_ex(index._h, q.data_ptr(), B, k, npb, C.byref(scfg), ids.data_ptr(), dd.data_ptr(),
                                     N.SAQG_MEM_DEVICE, sptr, C.byref(st), probes.data_ptr()))
    N.check(index.lib.saqg_search_tc(index._h, q.data_ptr(), B, k, npb, a.tc_shortlist, C.byref(scfg), ids.data_ptr(),
                                     dd.data_ptr(), None, N.SAQG_MEM_DEVICE, sptr, C.byref(tst)))
    torch.cuda.synchronize()
    pr = probes.cpu().numpy()
    out["exact_compulsory_bytes"] = exact_bytes(plan, sizes, pr, st.rerank_bytes, a.dim)
    out["contraction_bytes"] = contraction_bytes(plan, sizes, pr, tst.pairs, tst.candidates)
    log(f"kernels: exact {out['exact_ms']} ms, tensor-core {out['tc_ms']} ms")
    return out


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference" and rank != 0:
        return
    import torch
    torch.cuda.set_device(local)
    if world > 1 and a.impl != "reference":
        import torch.distributed as dist
        dist.init_process_group("nccl")
    log = (lambda m: print(f"[bench] {m}", file=sys.stderr, flush=True)) if rank == 0 else (lambda m: None)
    t_start = time.time()
    if a.only == "precision":
        flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
        prec = precision_leg(a, torch, flush, log)
        print(json.dumps({"metric": "precision form (tensor-core contraction) vs FP32 CUDA-core search",
                          "precision": prec, "wall_s": time.time() - t_start}), flush=True)
        return
    if a.only in ("c1", "c2"):
        with tempfile.TemporaryDirectory() as td:
            out = (c1_leg if a.only == "c1" else c2_leg)(a, torch, log, td)
        print(json.dumps({"metric": "plain single-query QPS, p50/p99, recall@10 and encode vectors/s",
                          a.only: out, "wall_s": time.time() - t_start}), flush=True)
        return
    if a.only == "kernels":
        print(json.dumps(kernels_leg(a, torch, log)), flush=True)
        return
    wl = build_workload(a, torch)
    log(f"workload {wl.name} generated in {time.time() - t_start:.1f}s")
    if a.impl == "reference":
        ipath, meta = get_oracle_index(a, torch, wl, log)
    else:
        index, ipath, meta = get_index_and_meta(a, torch, wl, log)
    nprobe = meta["nprobe"]
    threads = os.cpu_count() or 1
    config = {"workload": f"{a.n // 1_000_000}M x {a.dim}, B={a.bits:g} SAQ (segmented), {a.clusters} clusters "
                          f"Zipf(1.1), PCA, k={a.topk}, batch {a.batch}",
              "nprobe": nprobe, f"recall@{a.topk}": round(meta["recall"], 4), "plan": meta["plan"],
              "l2": "flushed between timed steps (256 MiB write)", "queries": "same distribution as the base set",
              "data_model": f"unit-norm; centre spectrum i^-0.8, within-cluster spectrum i^-{a.noise_alpha:g}, "
                            f"sigma {a.sigma:g}; query clusters {a.query_clusters}",
              "form": "batched exact search (saqg_search): every id and distance equal to the reference's "
                      "IVF::search on the same index, bit for bit"}

    if a.impl == "reference":
        qh = wl.q.cpu().numpy()
        oi = None
        for _ in range(a.warmup):
            _, _, _, _, oi = cpu_search_rate(ipath, qh, a.topk, nprobe, 2.0, threads, oi)
        step_q = None
        times = []
        for _ in range(a.steps):
            r, ns, dt, _, oi = cpu_search_rate(ipath, qh, a.topk, nprobe, 3.0, threads, oi)
            times.append(dt)
            step_q = ns
        v = float(step_q * len(times) / sum(times))
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "queries/s", "n_gpus": world,
                "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32",
                "data": "synthetic (seeded, generated on the GPU)", "config": config,
                "cpu_baseline": {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
                                 "sample": f"{step_q} single-query tasks per step on the same 10M index "
                                           f"(written by the CPU oracle's builder in "
                                           f"{meta.get('build_s', 0.0):.0f}s)"},
                "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    from saq_gb300 import _native as N, ivf, workloads
    import ctypes as C
    lib = index.lib
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)
    scfg = ivf.SearcherConfig().to_c()
    B = a.batch
    qdev = wl.q[:B].contiguous()
    ids = torch.empty((B, a.topk), dtype=torch.int32, device="cuda")
    dd = torch.empty((B, a.topk), dtype=torch.float32, device="cuda")
    probes = torch.empty((B, nprobe), dtype=torch.int32, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    stats = N.SearchStats()

    def batched(with_stats):
        N.check(lib.saqg_search_ex(index._h, qdev.data_ptr(), B, a.topk, nprobe, C.byref(scfg), ids.data_ptr(),
                                   dd.data_ptr(), N.SAQG_MEM_DEVICE, sptr,
                                   C.byref(stats) if with_stats else None,
                                   probes.data_ptr() if with_stats else None))

    ids_t = torch.empty((B, a.topk), dtype=torch.int32, device="cuda")
    d_t = torch.empty((B, a.topk), dtype=torch.float32, device="cuda")
    tst = N.TcStats()

    def tcb(with_stats=False):
        N.check(lib.saqg_search_tc(index._h, qdev.data_ptr(), B, a.topk, nprobe, a.tc_shortlist, C.byref(scfg),
                                   ids_t.data_ptr(), d_t.data_ptr(), None, N.SAQG_MEM_DEVICE, sptr,
                                   C.byref(tst) if with_stats else None))
    # autotuner: time every candidate launch shape of this batch once; later
    # calls of the shape (the timed ones) use the fastest
    tune = {}
    for form, name in ((N.SAQG_FORM_EXACT, "exact"), (N.SAQG_FORM_TC, "tensor_core")):
        rep = N.TuneReport()
        N.check(lib.saqg_autotune(index._h, qdev.data_ptr(), B, a.topk, nprobe, a.tc_shortlist, form, C.byref(scfg),
                                  sptr, C.byref(rep)))
        tune[name] = rep.as_dict()
        log(f"autotune {name}: default {rep.default_ms:.3f} ms, tuned {rep.tuned_ms:.3f} ms ({rep.candidates} shapes)")
    for _ in range(a.warmup):
        batched(True)
    for _ in range(a.warmup):
        tcb()
    torch.cuda.synchronize()
    step_ms, scan_ms, fast_b, rr_b, spec, rr, probe_ms, qprep_ms, split_ms = [], [], [], [], [], [], [], [], []
    vec_counts = []
    with ClockSampler(local) as clk:
        time.sleep(0.3)  # first sample before the timed region
        # ---- headline: the exact batched form (saqg_search), device-resident ----
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        launches0 = lib.saqg_kernel_launches()
        for _ in range(a.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batched(False)
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        launches = lib.saqg_kernel_launches() - launches0
        if world > 1:
            torch.distributed.barrier()
        # ---- the batched tensor-core form (saqg_search_tc) on the same batch ----
        tc_step_ms = []
        for _ in range(a.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tcb()
            e1.record(stream)
            e1.synchronize()
            tc_step_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()

    # stage times and counters of the exact form: the same call with statistics
    # (events between the stages, exact counters), outside the timed region
    for _ in range(min(5, a.steps)):
        flush.zero_()
        batched(True)
        torch.cuda.synchronize()
        scan_ms.append(stats.ms_scan)
        probe_ms.append(stats.ms_probe)
        qprep_ms.append(stats.ms_qprep)
        split_ms.append(stats.ms_split)
        fast_b.append(stats.fast_bytes)
        rr_b.append(stats.rerank_bytes)
        spec.append(stats.speculative)
        rr.append(stats.reranked)
        vec_counts.append(stats.vectors)

    from saq_gb300.replicas import max_over_ranks

    def world_max(x):
        return max_over_ranks(x, "cuda")
    tot_ms = world_max(float(sum(step_ms)))
    value = world * B * a.steps / (tot_ms / 1e3)
    tc_tot_ms = world_max(float(sum(tc_step_ms)))
    tc_value = world * B * a.steps / (tc_tot_ms / 1e3)
    got = ids.cpu().numpy().view(np.uint32)
    gt = meta["gt"]
    ng = min(len(gt), B)
    batch_recall = workloads.recall_at(got[:ng], gt[:ng], a.topk)

    # compulsory bytes of the exact form: each distinct probed cluster once + every re-rank
    info = index.info()
    sizes = np.bincount(wl.cids.cpu().numpy(), minlength=a.clusters)
    probes_np = probes.cpu().numpy()
    compulsory = exact_bytes(info["plan"], sizes, probes_np, rr_b[-1], a.dim)
    effective = fast_b[-1] + rr_b[-1]
    mean_scan = float(np.mean(scan_ms))
    coded_dims = sum(d for d, b in info["plan"] if b)
    lookups = float(np.mean(vec_counts)) * coded_dims / 4
    props = torch.cuda.get_device_properties(local)
    lookup_peak = props.multi_processor_count * 32 * 2070e6  # 32 lanes x SMs x max SM clock
    hbm, peak_kind = peaks()
    achieved = compulsory / (mean_scan / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "k_scan_traffic.json")
    if os.path.exists(tf):
        tj = json.load(open(tf))
        if tj.get("workload") == config["workload"] and tj.get("nprobe") == nprobe:
            traffic = tj.get("dram_bytes_per_launch")

    # tensor-core form: stage times and the contraction's roofline (5 calls with stats)
    tc_stats = []
    for _ in range(5):
        flush.zero_()
        tcb(True)
        tc_stats.append(tst.as_dict())
    torch.cuda.synchronize()
    it_ = ids_t.cpu().numpy().view(np.uint32)
    ts = tc_stats[-1]
    contract_ms = float(np.mean([x["ms_contract"] for x in tc_stats]))
    tc_bytes = contraction_bytes(info["plan"], sizes, probes_np, ts["pairs"], ts["candidates"])
    tc_achieved = tc_bytes / (contract_ms / 1e3) / 1e9
    tc_traffic = None
    tf2 = os.path.join(ROOT, "profiles", "k_tc_contract_traffic.json")
    if os.path.exists(tf2):
        tj = json.load(open(tf2))
        if tj.get("workload") == config["workload"] and tj.get("nprobe") == nprobe:
            tc_traffic = tj.get("dram_bytes_per_launch")
    tc_recall = workloads.recall_at(it_[:ng], gt[:ng], a.topk)

    # ---- e2e: host buffers through the C ABI (exact form; the tensor-core form beside it) ----
    qh = torch.empty((B, a.dim), dtype=torch.float32).pin_memory()
    qh.copy_(qdev.cpu())
    ih = torch.empty((B, a.topk), dtype=torch.int32).pin_memory()
    dh = torch.empty((B, a.topk), dtype=torch.float32).pin_memory()
    for _ in range(max(1, a.warmup)):
        N.check(lib.saqg_search(index._h, qh.data_ptr(), B, a.topk, nprobe, C.byref(scfg), ih.data_ptr(),
                                dh.data_ptr(), N.SAQG_MEM_HOST, sptr))
    e2e_ms = []
    for _ in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(lib.saqg_search(index._h, qh.data_ptr(), B, a.topk, nprobe, C.byref(scfg), ih.data_ptr(),
                                dh.data_ptr(), N.SAQG_MEM_HOST, sptr))
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_v = world * B * a.steps / (world_max(sum(e2e_ms)) / 1e3)
    e2e_same = bool(np.array_equal(ih.numpy().view(np.uint32), got))
    for _ in range(max(1, a.warmup)):
        N.check(lib.saqg_search_tc(index._h, qh.data_ptr(), B, a.topk, nprobe, a.tc_shortlist, C.byref(scfg),
                                   ih.data_ptr(), dh.data_ptr(), None, N.SAQG_MEM_HOST, sptr, None))
    e2e_ms = []
    for _ in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(lib.saqg_search_tc(index._h, qh.data_ptr(), B, a.topk, nprobe, a.tc_shortlist, C.byref(scfg),
                                   ih.data_ptr(), dh.data_ptr(), None, N.SAQG_MEM_HOST, sptr, None))
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_tc = world * B * a.steps / (world_max(sum(e2e_ms)) / 1e3)

    # ---- plain single-query drop-in ----
    P = a.plain_queries
    qp = wl.q[:P].contiguous()
    lat, _ = plain_latencies(torch, lib, index, qp, a.topk, nprobe)
    plain_qps = P / (lat.sum() / 1e3)
    plain_thr_qps, plain_thr_n = plain_threads(torch, lib, index, wl.q[:B].cpu().numpy(), a.topk, nprobe, threads)

    # ---- plain single query through a captured graph (query copied into the bound buffer) ----
    gq = torch.empty((1, a.dim), dtype=torch.float32, device="cuda")
    gq.copy_(qp[0:1])
    gids = torch.empty((1, a.topk), dtype=torch.int32, device="cuda")
    gd = torch.empty((1, a.topk), dtype=torch.float32, device="cuda")
    graph = C.c_void_p()
    N.check(lib.saqg_search_graph_create(index._h, gq.data_ptr(), 1, a.topk, nprobe, C.byref(scfg), gids.data_ptr(),
                                         gd.data_ptr(), sptr, C.byref(graph)))
    glat = []
    for i in range(P):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gq.copy_(qp[i:i + 1])
        N.check(lib.saqg_search_graph_launch(graph, sptr))
        e1.record(stream)
        e1.synchronize()
        glat.append(e0.elapsed_time(e1))
    N.check(lib.saqg_search_graph_free(graph))
    glat = np.array(glat)

    # ---- uneven batch: per-query nprobe ~ U[16, 256], k in {10, 100} (saqg_search_batch) ----
    rng = np.random.default_rng(7)
    np_mix = rng.integers(16, 257, size=B).astype(np.int32)
    k_mix = rng.choice([10, 100], size=B).astype(np.int32)
    ids_m = torch.empty((B, 100), dtype=torch.int32, device="cuda")
    d_m = torch.empty((B, 100), dtype=torch.float32, device="cuda")

    def mixed():
        N.check(lib.saqg_search_batch(index._h, qdev.data_ptr(), B, np_mix.ctypes.data, k_mix.ctypes.data, 256, 100,
                                      C.byref(scfg), ids_m.data_ptr(), d_m.data_ptr(), N.SAQG_MEM_DEVICE, sptr, None))
    mixed()
    mixed_ms = []
    for _ in range(max(3, min(10, a.steps // 10))):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mixed()
        e1.record(stream)
        e1.synchronize()
        mixed_ms.append(e0.elapsed_time(e1))
    mixed_line = {"qps": B / (float(np.mean(mixed_ms)) / 1e3), "batch": B, "ms_per_batch": float(np.mean(mixed_ms)),
                  "nprobe": "U[16,256] per query (mean %.0f)" % float(np_mix.mean()), "k": "10 or 100 per query",
                  "form": "exact (saqg_search_batch)"}
    # the same uneven batch through the tensor-core form (saqg_search_tc_batch), shortlist 4 x 100
    ids_tm = torch.empty((B, 100), dtype=torch.int32, device="cuda")
    d_tm = torch.empty((B, 100), dtype=torch.float32, device="cuda")

    def mixed_tc():
        N.check(lib.saqg_search_tc_batch(index._h, qdev.data_ptr(), B, np_mix.ctypes.data, k_mix.ctypes.data, 256, 100,
                                         400, C.byref(scfg), ids_tm.data_ptr(), d_tm.data_ptr(), None,
                                         N.SAQG_MEM_DEVICE, sptr, None))
    mixed_tc_ms, _ = time_calls(torch, mixed_tc, flush, max(3, min(10, a.steps // 10)))
    em, tm = ids_m.cpu().numpy().view(np.uint32), ids_tm.cpu().numpy().view(np.uint32)
    hit = sum(len(set(em[i, :k_mix[i]].tolist()) & set(tm[i, :k_mix[i]].tolist())) for i in range(B))
    # recall@10 against FP64 ground truth of both forms, over the queries with k = 10 that have ground truth
    sel = [i for i in range(min(B, len(meta["gt"]))) if k_mix[i] == 10]
    gt10 = meta["gt"][sel]
    mixed_line["recall@10_fp64_k10_queries"] = round(workloads.recall_at(em[sel, :10], gt10, 10), 4)
    mixed_line["tensor_core_form"] = {"qps": B / (mixed_tc_ms / 1e3), "ms_per_batch": mixed_tc_ms, "shortlist": 400,
                                      "recall_vs_exact": hit / float(k_mix.sum()),
                                      "recall@10_fp64_k10_queries": round(workloads.recall_at(tm[sel, :10], gt10, 10), 4),
                                      "k10_queries": len(sel)}

    # ---- serving: Poisson arrivals through the continuous-batching server (both forms) ----
    serving, serving_tc = [], []
    if a.serve_seconds > 0:
        qpool = wl.q.cpu().numpy()
        gt_all = meta["gt"]
        for form, out in (("exact", serving), ("tc", serving_tc)):
            srv = ivf.Server(index, max_batch=B, max_inflight=2, max_topk=100, max_nprobe=256, max_wait_us=200,
                             form=form)
            for rate in a.serve_rates:
                n = max(1000, int(rate * a.serve_seconds))
                arr = np.cumsum(rng.exponential(1.0 / rate, size=n))
                qi = np.arange(n) % qpool.shape[0]
                qs = qpool[qi]
                nps = rng.integers(16, 257, size=n).astype(np.int32)
                ks = rng.choice([10, 100], size=n).astype(np.int32)
                before = srv.stats()
                t0 = time.perf_counter()
                sids, _, lat_s = srv.run_trace(qs, arr, nps, ks)
                wall = time.perf_counter() - t0
                after = srv.stats()
                nb = after["batches"] - before["batches"]
                sel = [i for i in range(n) if ks[i] == 10 and qi[i] < len(gt_all)]
                rec = workloads.recall_at(sids[sel, :10], gt_all[qi[sel]], 10) if sel else None
                out.append({"offered_qps": rate, "achieved_qps": n / wall, "queries": n,
                            "p50_ms": float(np.percentile(lat_s, 50)), "p99_ms": float(np.percentile(lat_s, 99)),
                            "mean_batch": n / max(1, nb), "recall@10_fp64_k10_queries": rec})
                log(f"serving ({form}) {rate}/s: p50 {out[-1]['p50_ms']:.2f} ms p99 {out[-1]['p99_ms']:.2f} ms "
                    f"achieved {out[-1]['achieved_qps']:.0f}/s")
            srv.close()

    # ---- CPU baseline (oracle port) on a bounded sample ----
    cpu = None
    if rank == 0:
        qnp = wl.q.cpu().numpy()
        r, ns, dt, cids_cpu, oi = cpu_search_rate(ipath, qnp, a.topk, nprobe, a.cpu_seconds, threads)
        same = bool(np.array_equal(cids_cpu[:min(ns, B)], got[:min(ns, B)]))
        r1, ns1, dt1, _, _ = cpu_search_rate(ipath, qnp, a.topk, nprobe, min(2.0, a.cpu_seconds), 1, oi)
        del oi
        cpu = {"value": r, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": f"{ns} queries of the batch on the same index ({dt:.1f}s, {threads} threads)",
               "ids_equal_gpu": same,
               "single_thread": {"value": r1, "sample": f"{ns1} queries ({dt1:.1f}s, 1 thread)"}}

    del index, wl
    torch.cuda.empty_cache()
    configs = {}
    if rank == 0 and a.configs:
        with tempfile.TemporaryDirectory() as td:
            configs["c1"] = c1_leg(a, torch, log, td)
            configs["c2"] = c2_leg(a, torch, log, td)

    precision = None
    if rank == 0 and a.precision_bits:
        precision = precision_leg(a, torch, flush, log)

    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": tot_ms / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32+f32", "data": "synthetic (seeded, generated on the GPU)",
        "config": config,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": "scan phase (k_scan beside the split pass)",
                     "peak_kind": peak_kind,
                     "bytes_per_launch": compulsory, "effective_bytes_per_launch": effective,
                     "effective_gbs": effective / (mean_scan / 1e3) / 1e9, "scan_ms": mean_scan,
                     "reranked_per_query": float(np.mean(rr)) / B,
                     "speculative_per_query": float(np.mean(spec)) / B,
                     "probe_ms": float(np.mean(probe_ms)), "qprep_ms": float(np.mean(qprep_ms)),
                     "split_pass_ms": float(np.mean(split_ms)),
                     # what bounds the scan: one shared-memory LUT lookup per 4 coded dims per
                     # (query, vector); peak one 32-lane lookup per SM per cycle
                     "lut_lookups_per_s": lookups / (mean_scan / 1e3),
                     "lut_lookup_peak_per_s": lookup_peak,
                     "lut_lookup_frac": lookups / (mean_scan / 1e3) / lookup_peak},
        "batched": {"form": "exact (saqg_search)", "qps": value, "batch": B,
                    "p50_ms": float(np.median(step_ms)), "p99_ms": float(np.percentile(step_ms, 99)),
                    f"recall@{a.topk}": round(batch_recall, 4),
                    "autotune": {"note": "saqg_autotune on this batch before the timed steps (best of 3 per "
                                         "shape, answers checked equal); the timed calls use the chosen shapes",
                                 **tune}},
        "batched_tc": {
            "form": "tensor-core (saqg_search_tc): dense BF16 code contraction, shortlist "
                    f"{a.tc_shortlist}, re-ranked with the exact search's distance; a stated-recall variant",
            "qps": tc_value, "e2e_qps": e2e_tc, "p50_ms": float(np.median(tc_step_ms)),
            "p99_ms": float(np.percentile(tc_step_ms, 99)), f"recall@{a.topk}": round(tc_recall, 4),
            f"recall@{a.topk}_vs_exact_search": round(overlap(it_, got, a.topk), 4),
            "stages_ms": {k: float(np.mean([x[k] for x in tc_stats]))
                          for k in ("ms_probe", "ms_pairs", "ms_contract", "ms_select", "ms_rerank")},
            "roofline": {"bound": "hbm", "achieved": tc_achieved, "peak": hbm, "unit": "GB/s",
                         "frac": tc_achieved / hbm, "traffic": tc_traffic, "peak_kind": peak_kind,
                         "kernel": "k_tc_contract (tcgen05.mma BF16, TMA-fed, persistent)",
                         "bytes_per_launch": tc_bytes,
                         "bytes_note": "packed codes of each distinct probed cluster once + query rows + outputs",
                         "bf16_operand_bytes": ts["code_bytes"], "contract_ms": contract_ms,
                         "tiles": ts["tiles"], "tensor_tflops": ts["flops"] / (contract_ms / 1e3) / 1e12,
                         "tensor_peak_tflops": bf16_peak()[0]}},
        "plain": {"qps": plain_qps, "queries": P, "p50_ms": float(np.median(lat)),
                  "p99_ms": float(np.percentile(lat, 99)),
                  "threads": {"qps": plain_thr_qps, "threads": threads, "queries": plain_thr_n,
                              "note": "one query per saqg_search call from host threads on their own streams, "
                                      "host buffers, wall clock (the reference drivers' thread pool)"},
                  "graph": {"qps": P / (glat.sum() / 1e3), "p50_ms": float(np.median(glat)),
                            "p99_ms": float(np.percentile(glat, 99)),
                            "note": "saqg_search_graph_launch of a captured single-query search"}},
        "batched_over_plain": value / world / plain_qps,
        "batched_tc_over_plain": tc_value / world / plain_qps,
        "p99_ms": float(np.percentile(step_ms, 99)),
        "uneven_batch": mixed_line,
        "c1": configs.get("c1"),
        "c2": configs.get("c2"),
        "precision": precision,
        "serving": {"server": "continuous batching, 2 batches in flight, max batch %d" % B,
                    "nprobe": "U[16,256] per query", "k": "10 or 100 per query", "arrivals": "Poisson",
                    "rates": serving,
                    "tensor_core_form": {"shortlist": 800, "rates": serving_tc,
                                         "note": "the same trace through the tensor-core form (saqg_search_tc_batch "
                                                 "per batch); recall against FP64 on the k = 10 queries with "
                                                 "ground truth"}},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_v, "unit": "queries/s", "h2d_bytes_per_step": B * a.dim * 4,
                "d2h_bytes_per_step": B * a.topk * 8, "ids_equal_device_run": e2e_same},
        "clocks": clocks,
        "gpu_launches": int(launches),
        "wall_s": time.time() - t_start,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
