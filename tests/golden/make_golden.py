"""Generate the golden fixtures in tests/golden/ by running the REFERENCE itself.

Runs only where the reference checkout and the shimmed reference driver exist
(`make -C oracle ref`, x86 + AVX-512).  Every fixture is a small .npz holding
the seeded inputs, the reference-built `.index` file (as bytes) and the
reference's outputs:
  * search  : IVF::search result ids                       (ivf.hpp:275-311)
  * estimate: IVF::estimate ids / accurate / fast / vars   (ivf.hpp:313-362)
  * dump    : probe ids + centroid distances, rotated query segments, prune
              bounds, LUT scalars, u16 LUTs and FastScan integer sums
  * encode  : CAQEncoder codes + factors, packed block and ex-codes
  * plan    : SaqDataMaker plans for several spectra

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from saq_gb300 import data  # noqa: E402

# name -> (generator, params)
INDEX_CASES = {
    # multi-segment SAQ (plan (64,6)(192,3)), anisotropic PCA data
    "aniso_b4_seg": dict(gen="aniso", n=900, d=256, k=10, nq=10, bits=4, seg=1, eqseg=0, topk=10, nprobe=5, seed=11),
    # one segment (CAQ only), Gaussian mixture like the 100k x 960 workload, scaled down
    "mix_b4_noseg": dict(gen="mix", n=900, d=128, k=8, nq=10, bits=4, seg=0, eqseg=0, topk=10, nprobe=4, seed=12),
    # reference unit-test style integers: every cluster holds a multiple of 32
    # vectors (last-block skip in scanCluster) and centroids repeat (ties)
    "grid_b4_ties": dict(gen="grid", n=768, d=64, k=24, nq=8, bits=4, seg=0, eqseg=0, topk=10, nprobe=6, seed=13),
    # 1-bit segments (two equal segments of B=1): the reference crashes here
    # (caq_encoder.hpp:239-246); the harness hands the code to the packer itself
    "aniso_b1_eqseg2_1bit": dict(gen="aniso", n=700, d=128, k=8, nq=8, bits=1, seg=1, eqseg=2, topk=10, nprobe=4, seed=14),
    # B=1.5 with segmentation: a 0-bit segment
    "aniso_b15_seg_0bit": dict(gen="aniso", n=700, d=128, k=8, nq=8, bits=1.5, seg=1, eqseg=0, topk=10, nprobe=4, seed=15),
    # wide ex-codes: 8 bits (ex 7) single segment; 10 and 13 bits (ex 9, ex 12) in two equal segments
    "mix_b8_noseg": dict(gen="mix", n=600, d=128, k=8, nq=8, bits=8, seg=0, eqseg=0, topk=10, nprobe=3, seed=16),
    "mix_b10_eqseg2": dict(gen="mix", n=600, d=128, k=8, nq=8, bits=10, seg=1, eqseg=2, topk=10, nprobe=3, seed=17),
    "mix_b13_eqseg2": dict(gen="mix", n=500, d=128, k=8, nq=6, bits=13, seg=1, eqseg=2, topk=10, nprobe=3, seed=18),
    # top-100 with nprobe covering every cluster
    "aniso_b4_seg_top100": dict(gen="aniso", n=800, d=256, k=6, nq=6, bits=4, seg=1, eqseg=0, topk=100, nprobe=6, seed=19),
}

# IVF::construct without rotation: residuals are exact, so the whole index is
# comparable (inputs are stored too)
CONSTRUCT_CASES = {
    "construct_norot_b4_seg": dict(gen="aniso", n=400, d=256, k=5, bits=4, seg=1, eqseg=0, seed=31),
    "construct_norot_b15_seg": dict(gen="aniso", n=300, d=128, k=4, bits=1.5, seg=1, eqseg=0, seed=32),
    "construct_norot_b9_noseg": dict(gen="mix", n=300, d=128, k=4, bits=9, seg=0, eqseg=0, seed=33),
}

ENCODE_BITS = [1, 2, 3, 4, 5, 6, 7, 8, 9, 13]
PLAN_CASES = [(256, 4), (1024, 4), (1024, 1.5), (960, 4), (1536, 6), (1536, 8), (512, 2), (1024, 0.5)]


def make_data(p):
    if p["gen"] == "aniso":
        x, q = data.anisotropic(p["n"], p["d"], 0.8, seed=p["seed"], n_query=p["nq"])
        mean, comp, _ = data.pca_fit(x)
        x, q = data.pca_apply(x, mean, comp), data.pca_apply(q, mean, comp)
        cent, cids = data.kmeans(x, p["k"], iters=20, seed=p["seed"])
    elif p["gen"] == "mix":
        x, q = data.gaussian_mixture(p["n"], p["d"], 3 * p["k"], 0.5, seed=p["seed"], n_query=p["nq"])
        mean, comp, _ = data.pca_fit(x)
        x, q = data.pca_apply(x, mean, comp), data.pca_apply(q, mean, comp)
        cent, cids = data.kmeans(x, p["k"], iters=20, seed=p["seed"])
    else:
        x, q, cent, cids = data.int_grid(p["n"], p["nq"], p["d"], p["k"], seed=p["seed"])
    return x, q, cent, cids


def index_case(name, p, tmp):
    x, q, cent, cids = make_data(p)
    N, D = x.shape
    K = cent.shape[0]
    f = lambda s: os.path.join(tmp, s)  # noqa: E731
    x.tofile(f("x.f32"))
    q.tofile(f("q.f32"))
    cent.astype(np.float32).tofile(f("c.f32"))
    cids.astype(np.uint32).tofile(f("cid.u32"))
    info = json.loads(O.run_ref("build", f("x.f32"), N, D, f("c.f32"), K, f("cid.u32"), f("a.index"), p["bits"],
                                p["seg"], p["eqseg"], 1, 6, 1e-8, 4))
    NQ = q.shape[0]
    O.run_ref("search", f("a.index"), f("q.f32"), NQ, p["topk"], p["nprobe"], 4, f("ids.u32"), f("ms.f32"), 1)
    O.run_ref("estimate", f("a.index"), f("q.f32"), min(NQ, 3), p["nprobe"], 4, f("est"))
    O.run_ref("dump", f("a.index"), f("q.f32"), min(NQ, 2), p["nprobe"], f("dump"))
    rd = lambda s, t: np.fromfile(f(s), dtype=t)  # noqa: E731
    out = dict(
        q=q,
        index_bytes=np.frombuffer(open(f("a.index"), "rb").read(), dtype=np.uint8),
        plan=np.array(info["plan"], dtype=np.int64),
        params=np.frombuffer(json.dumps(p).encode(), dtype=np.uint8),
        search_ids=rd("ids.u32", np.uint32).reshape(NQ, p["topk"]),
        est_count=rd("est.count.u64", np.uint64), est_ids=rd("est.ids.u32", np.uint32),
        est_acc=rd("est.acc.f32", np.float32), est_fast=rd("est.fast.f32", np.float32),
        est_vars=rd("est.vars.f32", np.float32),
        dump_probe_ids=rd("dump.probe_ids.u32", np.uint32), dump_probe_d=rd("dump.probe_d.f32", np.float32),
        dump_rotq=rd("dump.rotq.f32", np.float32), dump_prune=rd("dump.prune.f32", np.float32),
        dump_scal=rd("dump.scal.f32", np.float32), dump_lut=rd("dump.lut.u16", np.uint16),
        dump_sums=rd("dump.sums.i32", np.int32),
    )
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, info["plan"], "index bytes", out["index_bytes"].size)


def construct_case(name, p, tmp):
    pp = dict(p, nq=1)
    x, _, cent, cids = make_data(pp)
    N, D = x.shape
    K = cent.shape[0]
    f = lambda s: os.path.join(tmp, s)  # noqa: E731
    x.tofile(f("x.f32"))
    cent.astype(np.float32).tofile(f("c.f32"))
    cids.astype(np.uint32).tofile(f("cid.u32"))
    info = json.loads(O.run_ref("build", f("x.f32"), N, D, f("c.f32"), K, f("cid.u32"), f("a.index"), p["bits"],
                                p["seg"], p["eqseg"], 0, 6, 1e-8, 2))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), x=x, centroids=cent.astype(np.float32),
                        cids=cids.astype(np.uint32),
                        index_bytes=np.frombuffer(open(f("a.index"), "rb").read(), dtype=np.uint8),
                        plan=np.array(info["plan"], dtype=np.int64),
                        params=np.frombuffer(json.dumps(p).encode(), dtype=np.uint8))
    print(name, info["plan"])


def encode_case(tmp):
    rng = np.random.default_rng(21)
    D, n = 128, 40
    out = {}
    for bits in ENCODE_BITS:
        r = (rng.standard_normal((n, D)) * rng.uniform(0.1, 2, size=(n, 1))).astype(np.float32)
        cen = rng.standard_normal(D).astype(np.float32)
        f = lambda s: os.path.join(tmp, s)  # noqa: E731
        r.tofile(f("r.f32"))
        cen.tofile(f("cen.f32"))
        O.run_ref("encode", f("r.f32"), n, D, bits, f("cen.f32"), 6, f("enc"))
        out[f"b{bits}_resid"] = r
        out[f"b{bits}_centroid"] = cen
        out[f"b{bits}_codes"] = np.fromfile(f("enc.codes.i32"), np.int32).reshape(n, D)
        out[f"b{bits}_facs"] = np.fromfile(f("enc.facs.f64"), np.float64).reshape(n, 4).astype(np.float32)
        out[f"b{bits}_blocks"] = np.fromfile(f("enc.blocks.u8"), np.uint8)
        out[f"b{bits}_long"] = np.fromfile(f("enc.long.u8"), np.uint8).reshape(n, -1)
        out[f"b{bits}_exfac"] = np.fromfile(f("enc.exfac.f32"), np.float32).reshape(n, 2)
    np.savez_compressed(os.path.join(HERE, "encode.npz"), **out)
    print("encode", ENCODE_BITS)


def plan_case(tmp):
    rng = np.random.default_rng(22)
    out = {}
    for i, (D, ab) in enumerate(PLAN_CASES):
        var = (np.arange(1, D + 1) ** -0.8).astype(np.float32) * rng.uniform(0.9, 1.1, size=D).astype(np.float32)
        f = lambda s: os.path.join(tmp, s)  # noqa: E731
        var.tofile(f("var.f32"))
        O.run_ref("plan", f("var.f32"), D, ab, 1, 0, f("plan.txt"))
        plan = [tuple(map(int, l.split())) for l in open(f("plan.txt"))]
        out[f"c{i}_var"] = var
        out[f"c{i}_avg_bits"] = np.float32(ab)
        out[f"c{i}_plan"] = np.array(plan, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "plan.npz"), **out)
    print("plan", len(PLAN_CASES))


def main():
    if not O.ref_available():
        sys.exit("reference driver missing: run `make -C oracle ref` on an x86 AVX-512 host with the reference")
    with tempfile.TemporaryDirectory() as tmp:
        for name, p in INDEX_CASES.items():
            index_case(name, p, tmp)
        for name, p in CONSTRUCT_CASES.items():
            construct_case(name, p, tmp)
        encode_case(tmp)
        plan_case(tmp)


if __name__ == "__main__":
    main()
