"""Reader/writer for the reference's binary `.index` file (IVF::save, ivf.hpp:197-228).

Layout, all little-endian, `size_t` = 8 bytes:
  [N][D][K]                                   ivf.hpp:207-209
  centroids K x D float32                     initializer.hpp:78-84
  SaqData                                     saq_data.hpp:29-39
    QuantizeConfig (raw struct, 32 bytes)
    num_dim, variance (size_t n + n float32)
    #segments, then per segment               quantizer_data.hpp:26-35
      num_dim_pad, num_bits, QuantSingleConfig (raw, 20 bytes),
      rotator flag (1 byte), P (D_s x D_s float32, row-major) if flag
  cluster sizes K x size_t                    ivf.hpp:216-221
  per cluster                                 cluster_data.hpp:327-336
    short_factors  (multi-segment only) num_blocks x S x 64 float32
    short_code     num_blocks x block_bytes
    long_code      num_vec x long_bytes_per_vec
    long_factors   num_vec x S x (rescale, error) float32
    ids            num_vec x uint32
    centroid       per segment D_s float32 (rotated)

Block layout (cluster_data.hpp:206-294):
  * one segment: block = [32 x |o|][32 x ip_cent_oa][D_s*4 bytes packed codes];
    long codes are compact (num_vec x D_s*(B-1)/8).
  * several segments: short_factors holds per block [seg0 64 floats][seg1 ...],
    short_code holds per block [seg0 D_0*4 bytes][seg1 ...]; long codes are
    per vector [seg0 padded to 16 B][seg1 padded to 16 B]...
    (the default `use_compact_layout = false`).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

QUANTIZE_CONFIG_BYTES = 32
QUANT_SINGLE_CONFIG_BYTES = 20
FASTSCAN = 32


def _rd_up(x, m):
    return (x + m - 1) // m * m


@dataclass
class Segment:
    dim: int
    bits: int
    P: np.ndarray | None  # D_s x D_s float32 or None (no rotation)
    single_cfg: bytes = b""


@dataclass
class Cluster:
    num_vec: int
    short_factors: np.ndarray  # float32 (multi-seg) or empty
    short_code: np.ndarray     # uint8 blocks
    long_code: np.ndarray      # uint8
    long_factors: np.ndarray   # float32 (num_vec, S, 2)
    ids: np.ndarray            # uint32
    centroids: list            # per segment float32 (D_s,)


@dataclass
class IndexFile:
    N: int
    D: int
    K: int
    centroids: np.ndarray
    quantize_cfg: bytes
    num_dim: int
    variance: np.ndarray
    segments: list
    clusters: list = field(default_factory=list)

    @property
    def avg_bits(self) -> float:
        return struct.unpack_from("<f", self.quantize_cfg, 0)[0]

    @property
    def use_compact_layout(self) -> bool:
        return len(self.segments) == 1 or bool(self.quantize_cfg[9])


def segment_sizes(segments, use_compact):
    """Per-segment byte counts used by the block and long-code layouts."""
    S = len(segments)
    short_code = [s.dim * FASTSCAN // 8 if s.bits else 0 for s in segments]
    long_pv = [s.dim * (s.bits - 1) // 8 if s.bits else 0 for s in segments]
    if S == 1:
        block_bytes = 64 * 4 + short_code[0]
        long_stride = long_pv[0]
    else:
        block_bytes = sum(short_code)
        long_stride = sum(_rd_up(b, 16) for b in long_pv) if not use_compact else sum(long_pv)
    return short_code, long_pv, block_bytes, long_stride


def load(path: str) -> IndexFile:
    buf = open(path, "rb").read()
    off = 0

    def take(nbytes):
        nonlocal off
        b = buf[off:off + nbytes]
        if len(b) != nbytes:
            raise ValueError(f"truncated index file {path}")
        off += nbytes
        return b

    def size_t():
        return struct.unpack("<Q", take(8))[0]

    N, D, K = size_t(), size_t(), size_t()
    cent = np.frombuffer(take(4 * K * D), dtype=np.float32).reshape(K, D).copy()
    qcfg = take(QUANTIZE_CONFIG_BYTES)
    num_dim = size_t()
    nv = size_t()
    var = np.frombuffer(take(4 * nv), dtype=np.float32).copy()
    nseg = size_t()
    segs = []
    for _ in range(nseg):
        dpad, bits = size_t(), size_t()
        scfg = take(QUANT_SINGLE_CONFIG_BYTES)
        flag = take(1)[0]
        P = None
        if flag:
            P = np.frombuffer(take(4 * dpad * dpad), dtype=np.float32).reshape(dpad, dpad).copy()
        segs.append(Segment(dpad, bits, P, scfg))
    idx = IndexFile(N, D, K, cent, qcfg, num_dim, var, segs)
    sizes = [size_t() for _ in range(K)]
    S = len(segs)
    compact = idx.use_compact_layout
    short_code, long_pv, block_bytes, long_stride = segment_sizes(segs, compact)
    for c in range(K):
        n = sizes[c]
        nb = (n + FASTSCAN - 1) // FASTSCAN
        sf = np.frombuffer(take(4 * 64 * S * nb), dtype=np.float32).copy() if S > 1 else np.zeros(0, np.float32)
        sc = np.frombuffer(take(block_bytes * nb), dtype=np.uint8).copy()
        lc = np.frombuffer(take(long_stride * n), dtype=np.uint8).copy()
        lf = np.frombuffer(take(8 * S * n), dtype=np.float32).reshape(n, S, 2).copy()
        ids = np.frombuffer(take(4 * n), dtype=np.uint32).copy()
        cl = [np.frombuffer(take(4 * s.dim), dtype=np.float32).copy() for s in segs]
        idx.clusters.append(Cluster(n, sf, sc, lc, lf, ids, cl))
    if off != len(buf):
        raise ValueError(f"{len(buf) - off} trailing bytes in {path}")
    return idx


def save(idx: IndexFile, path: str) -> None:
    out = bytearray()
    out += struct.pack("<QQQ", idx.N, idx.D, idx.K)
    out += np.ascontiguousarray(idx.centroids, np.float32).tobytes()
    out += idx.quantize_cfg
    out += struct.pack("<Q", idx.num_dim)
    out += struct.pack("<Q", idx.variance.size) + np.ascontiguousarray(idx.variance, np.float32).tobytes()
    out += struct.pack("<Q", len(idx.segments))
    for s in idx.segments:
        out += struct.pack("<QQ", s.dim, s.bits) + s.single_cfg
        out += bytes([1 if s.P is not None else 0])
        if s.P is not None:
            out += np.ascontiguousarray(s.P, np.float32).tobytes()
    out += struct.pack(f"<{idx.K}Q", *[c.num_vec for c in idx.clusters])
    for c in idx.clusters:
        out += c.short_factors.tobytes() + c.short_code.tobytes() + c.long_code.tobytes()
        out += c.long_factors.tobytes() + c.ids.tobytes()
        for ce in c.centroids:
            out += ce.tobytes()
    open(path, "wb").write(bytes(out))


def plan_of(idx: IndexFile):
    return [(s.dim, s.bits) for s in idx.segments]
