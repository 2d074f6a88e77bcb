"""CPU restatement of the rasterizer's integer-built float products
(exact_fmul in farm_gb300/csrc/raster.cu): the double assembled from the
24 x 24-bit significand product and the two exponents equals
(double)a * (double)b for every finite float pair, subnormals and zeros
included. The GPU's bit-exact cell areas rest on this identity."""
import numpy as np


def exact_fmul(a: np.float32, b: np.float32) -> float:
    ua = int(np.float32(a).view(np.uint32))
    ub = int(np.float32(b).view(np.uint32))
    ea, eb = (ua >> 23) & 0xFF, (ub >> 23) & 0xFF
    assert ea != 0xFF and eb != 0xFF
    ma, mb = ua & 0x7FFFFF, ub & 0x7FFFFF
    if ea:
        ma |= 0x800000
    else:
        ea = 1
    if eb:
        mb |= 0x800000
    else:
        eb = 1
    sign = ((ua ^ ub) & 0x80000000) << 32
    m = ma * mb
    if m == 0:
        return float(np.uint64(sign).view(np.float64))
    top = m.bit_length() - 1
    assert top <= 47
    frac = (m << (52 - top)) & 0xFFFFFFFFFFFFF
    ex = top + ea + eb - 300 + 1023
    assert 0 < ex < 2047
    return float(np.uint64(sign | (ex << 52) | frac).view(np.float64))


def check(a, b):
    got = exact_fmul(a, b)
    want = float(np.float64(a) * np.float64(b))
    assert got == want and np.signbit(got) == np.signbit(want), (a, b, got, want)


def test_random_coordinates():
    rng = np.random.default_rng(1)
    xs = (rng.uniform(-500, 500, 20000)).astype(np.float32)
    ys = (rng.uniform(-500, 500, 20000)).astype(np.float32)
    for a, b in zip(xs, ys):
        check(a, b)


def test_random_bit_patterns_including_subnormals():
    rng = np.random.default_rng(2)
    bits = rng.integers(0, 2**32, 40000, dtype=np.uint64).astype(np.uint32)
    vals = bits.view(np.float32)
    vals = vals[np.isfinite(vals)]
    sub = (rng.integers(0, 2**23, 2000, dtype=np.uint64).astype(np.uint32) |
           (rng.integers(0, 2, 2000).astype(np.uint32) << 31)).view(np.float32)
    pool = np.concatenate([vals, sub, np.array([0.0, -0.0, 1.0, -1.0, 2.0**-149, -(2.0**-149),
                                                 np.finfo(np.float32).max, np.finfo(np.float32).tiny],
                                                np.float32)])
    for k in range(0, len(pool) - 1, 2):
        check(pool[k], pool[k + 1])
    for v in pool[:3000]:
        check(v, np.float32(0.0))
        check(np.float32(-0.0), v)
