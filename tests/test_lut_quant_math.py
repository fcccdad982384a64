"""The u16 LUT quantiser's fast path, checked on the CPU in IEEE float32.

Lut::prepare (saqlib/quantization/fastscan/lut.hpp:60-87) stores trunc(RN(x / delta)) for
each float entry x - vl >= 0 of a segment's LUT, with delta = RN((vr - vl) /
(65536 - 0.01)) taken in double.  The GPU quantiser (search.cu lut_quant_fast /
quant_codebook) multiplies instead: y = RN(x * RN(1 / delta)), and keeps trunc(y)
when no integer lies within 2^-21 * y of y, checking it as floor(RN(y - e)) ==
floor(RN(y + e)) with e = RN(y * 2^-21), the floors taken as RD(v + 2^23) - 2^23;
every other entry is divided.  These tests check, with numpy's correctly rounded
float32 operations, that whenever that check passes the two integers agree, on
random entries and on entries placed next to every integer boundary, and that
the 2^23 addition gives the floor for the values the check meets.
"""
import numpy as np

F = np.float32
E21 = F(2.0 ** -21)


def _delta(vl, vr):
    return F(np.float64(F(vr - vl)) / (65536.0 - 0.01))


def _fast(x, r):
    """(ok, trunc) of the fast path for float32 arrays x >= 0 and scalar r."""
    y = (x * r).astype(F)
    e = (y * E21).astype(F)
    lo = (y - e).astype(F)
    hi = (y + e).astype(F)
    ok = (np.floor(lo) == np.floor(hi)) & (y < F(4194304.0))
    return ok, np.floor(lo).astype(np.int64) & 0xFFFF


def _exact(x, d):
    return np.trunc((x / d).astype(F)).astype(np.int64) & 0xFFFF


def _check(vl, vr, x):
    d = _delta(vl, vr)
    r = F(F(1.0) / d)
    ok, fast = _fast(x, r)
    exact = _exact(x, d)
    assert np.array_equal(fast[ok], exact[ok])
    return float(ok.mean())


def test_fast_path_agrees_with_division_on_random_entries():
    rng = np.random.default_rng(5)
    rates = []
    for scale in (1e-30, 1e-6, 1e-2, 1.0, 37.0, 1e4, 1e30):
        for _ in range(8):
            vl = F(rng.standard_normal() * scale)
            vr = F(vl + F(abs(rng.standard_normal()) * scale + scale * 1e-3))
            if not vr > vl:
                continue
            x = (rng.random(200_000) * np.float64(F(vr - vl))).astype(F)
            rates.append(_check(vl, vr, x))
    # the fast path settles nearly every entry; the rest are divided
    assert min(rates) > 0.9


def test_fast_path_agrees_with_division_next_to_integer_boundaries():
    rng = np.random.default_rng(6)
    for _ in range(40):
        vl = F(rng.standard_normal())
        vr = F(vl + F(rng.random() * 10 + 1e-3))
        d = _delta(vl, vr)
        k = rng.integers(1, 65536, 5_000).astype(np.float64)
        base = (k * np.float64(d)).astype(F)
        # the float32 neighbours around k * delta, where trunc(x / delta) changes
        xs = [base]
        up, down = base.copy(), base.copy()
        for _ in range(6):
            up = np.nextafter(up, F(np.inf)).astype(F)
            down = np.nextafter(down, F(0)).astype(F)
            xs += [up, down]
        x = np.concatenate(xs)
        x = x[(x >= 0) & (x <= F(vr - vl))]
        _check(vl, vr, x)


def test_round_down_addition_of_2_pow_23_gives_the_floor():
    # RD(v + 2^23) for 0 <= v < 2^22: the exact sum lies in [2^23, 2^24), where
    # float32 spacing is 1, so rounding down keeps 2^23 + floor(v)
    rng = np.random.default_rng(7)
    v = np.concatenate([rng.random(300_000) * 70_000, np.arange(0, 70_000, 0.125),
                        [0.0, 65535.999, 65536.0, 4194303.5]]).astype(F)
    exact = np.float64(v) + 8388608.0
    rd = np.floor(exact)  # spacing 1 in [2^23, 2^24): round down = floor
    bits = rd.astype(F).view(np.uint32) & 0xFFFF
    assert np.array_equal(bits, np.floor(v).astype(np.int64).astype(np.uint32) & 0xFFFF)
