"""The FP32-first shortcuts of the GPU kernels, emulated in numpy with the
same operation order, against the arithmetic they stand in for (no GPU).

* within: pt_seg_dist32's error bound covers its distance from the
  reference's FP64 point-to-segment distance (geometry_computation.h:49-89);
* area: apart32 only rejects segment pairs that do not cross (exact rational
  test);
* raster: the cell clip's certified float rounding of the line abscissa gives
  (float)(((Y - B.y) / slope) + B.x) whenever it does not fall back.
"""
from fractions import Fraction

import numpy as np

f32 = np.float32
U32 = 2.0 ** -24


def dist64(p, p1, p2):
    # geometry_computation.h:49-89 (planar): float differences, then double
    A = float(f32(p[0]) - f32(p1[0]))
    B = float(f32(p[1]) - f32(p1[1]))
    C = float(f32(p2[0]) - f32(p1[0]))
    D = float(f32(p2[1]) - f32(p1[1]))
    dot = A * C + B * D
    len_sq = C * C + D * D
    param = dot / len_sq if len_sq != 0 else -1.0
    if param < 0:
        xx, yy = float(p1[0]), float(p1[1])
    elif param > 1:
        xx, yy = float(p2[0]), float(p2[1])
    else:
        xx, yy = float(p1[0]) + param * C, float(p1[1]) + param * D
    dx, dy = float(p[0]) - xx, float(p[1]) - yy
    return np.sqrt(dx * dx + dy * dy)


def dist32(p, p1, p2):
    # pt_seg_dist32 (planar), float32 throughout, the kernel's order
    A, B = f32(p[0]) - f32(p1[0]), f32(p[1]) - f32(p1[1])
    C, D = f32(p2[0]) - f32(p1[0]), f32(p2[1]) - f32(p1[1])
    dot = A * C + B * D
    ln = C * C + D * D
    t = dot / ln if ln != 0 else f32(0)
    t = min(max(t, f32(0)), f32(1))
    dx, dy = A - t * C, B - t * D
    d = np.sqrt(dx * dx + dy * dy, dtype=np.float32)
    M, L = abs(A) + abs(B), abs(C) + abs(D)
    absx = abs(f32(p[0])) + abs(f32(p[1])) + abs(f32(p1[0])) + abs(f32(p1[1]))
    err = f32(4e-6) * (M + L) + f32(1.2e-6) * d + f32(3e-15) * (absx + M + L)
    return float(d), float(err)


def test_within_fp32_distance_bound():
    rng = np.random.default_rng(1)
    worst = 0.0
    with np.errstate(all="ignore"):
        for scale, n in ((1.0, 3000), (1e5, 3000), (50.0, 3000)):
            base = rng.uniform(0, scale, (n, 2))
            p1 = (base + rng.normal(0, 1e-3 * scale, (n, 2))).astype(np.float32)
            p2 = (p1 + rng.normal(0, 1e-3 * scale, (n, 2)) * rng.choice([1.0, 1e-6, 0.0], (n, 1))).astype(np.float32)
            # points near the segment, on its line, and at its ends
            t = rng.uniform(-0.2, 1.2, (n, 1))
            off = rng.normal(0, 1e-3 * scale, (n, 2)) * rng.choice([1.0, 1e-7, 0.0], (n, 1))
            p = (p1 + t * (p2.astype(np.float64) - p1) + off).astype(np.float32)
            for k in range(n):
                d64 = dist64(p[k], p1[k], p2[k])
                d32, err = dist32(p[k], p1[k], p2[k])
                assert abs(d32 - d64) <= err, (scale, k, d32, d64, err)
                worst = max(worst, abs(d32 - d64) / err if err else 0.0)
    assert worst < 1.0


def apart32(P, Q, A, B):
    ex, ey = Q[0] - P[0], Q[1] - P[1]
    ax, ay, bx, by = A[0] - P[0], A[1] - P[1], B[0] - P[0], B[1] - P[1]
    oa, ob = ex * ay - ey * ax, ex * by - ey * bx
    ma, mb = f32(1e-6) * (abs(ex * ay) + abs(ey * ax)), f32(1e-6) * (abs(ex * by) + abs(ey * bx))
    if (oa > ma and ob > mb) or (oa < -ma and ob < -mb):
        return True
    gx, gy = B[0] - A[0], B[1] - A[1]
    px, py, qx, qy = P[0] - A[0], P[1] - A[1], Q[0] - A[0], Q[1] - A[1]
    op, oq = gx * py - gy * px, gx * qy - gy * qx
    mp, mq = f32(1e-6) * (abs(gx * py) + abs(gy * px)), f32(1e-6) * (abs(gx * qy) + abs(gy * qx))
    return (op > mp and oq > mq) or (op < -mp and oq < -mq)


def orient(a, b, c):
    F = lambda v: Fraction(float(v))  # float32 values are exact in double
    return (F(b[0]) - F(a[0])) * (F(c[1]) - F(a[1])) - (F(b[1]) - F(a[1])) * (F(c[0]) - F(a[0]))


def test_area_fp32_rejection_never_drops_a_crossing():
    rng = np.random.default_rng(2)
    rejected = 0
    with np.errstate(all="ignore"):
        for k in range(6000):
            s = 10.0 ** rng.uniform(-3, 2)
            c = rng.uniform(0, 400, 2)
            P, Q, A = (c + rng.normal(0, s, (3, 2))).astype(np.float32)
            if rng.random() < 0.5:  # B nearly on the line P-Q: near-degenerate cases
                tt = rng.uniform(-1, 2)
                B = (P.astype(np.float64) + tt * (Q.astype(np.float64) - P) + rng.normal(0, s * 1e-7, 2))
                B = B.astype(np.float32)
            else:
                B = (c + rng.normal(0, s, 2)).astype(np.float32)
            P, Q, A, B = (tuple(map(f32, v)) for v in (P, Q, A, B))
            if apart32(P, Q, A, B):
                rejected += 1
                # exactly: A and B strictly on one side of P-Q, or P and Q strictly on one side of A-B
                o1, o2 = orient(P, Q, A), orient(P, Q, B)
                o3, o4 = orient(A, B, P), orient(A, B, Q)
                assert (o1 > 0 and o2 > 0) or (o1 < 0 and o2 < 0) or (o3 > 0 and o4 > 0) or (o3 < 0 and o4 < 0), k
    assert rejected > 1000


def absc_f(Y, Bx, By, slope):
    # ClipYEdge::absc_f: reciprocal product, certified against float midpoints
    isl = 1.0 / slope  # correctly rounded reciprocal (__drcp_rn)
    t = Y - By
    q = t * isl
    sx = q + Bx
    bs = np.float64(sx).view(np.int64)
    bq = np.float64(q).view(np.int64)
    es, eq = int((bs >> 52) & 0x7FF), int((bq >> 52) & 0x7FF)
    k = eq - es + 1
    low = int(bs & 0x1FFFFFFF)
    dist = abs(low - (1 << 28))
    thr = (4 if k < 0 else ((1 << 30) if k > 24 else (4 << k))) + 2
    if 1023 - 125 <= es <= 1023 + 126 and dist > thr:
        return f32(sx), True
    return f32(((Y - By) / slope) + Bx), False


def test_clip_certified_float_rounding():
    rng = np.random.default_rng(3)
    fast = 0
    for k in range(20000):
        A = rng.uniform(-500, 500, 2).astype(np.float32)
        B = (A + rng.normal(0, 10.0 ** rng.uniform(-4, 1), 2)).astype(np.float32)
        if A[0] == B[0] or A[1] == B[1]:
            continue
        slope = (float(B[1]) - float(A[1])) / float(f32(B[0] - A[0]))
        Y = float(A[1]) + rng.uniform(0, 1) * (float(B[1]) - float(A[1]))
        got, certified = absc_f(Y, float(B[0]), float(B[1]), slope)
        exact = f32(((Y - float(B[1])) / slope) + float(B[0]))
        assert got == exact, (k, got, exact)
        fast += certified
    assert fast > 19000


def double_to_int(v):
    # util.h:98-106
    vi = int(v)
    if abs(1.0 * (vi + 1) - v) < 0.00000001:
        vi += 1
    return vi


def test_walk_certified_quotients():
    # walk_edge's double_to_int(t / d) and grid-corner test on t * fl(1/d)
    # decide as the exact quotient would, including values placed at the
    # decision thresholds
    rng = np.random.default_rng(4)
    dim = 4000
    qlim = dim + 2.0
    band = 1e-15 * (qlim + 2.0)
    n_fallback = 0
    for k in range(40000):
        step = 10.0 ** rng.uniform(-5, 0)
        inv = 1.0 / step
        r = rng.random()
        if r < 0.3:  # just below an integer, at the snap threshold
            q = rng.integers(1, dim) - 1e-8 + rng.normal(0, 1e-13)
        elif r < 0.5:  # at a grid corner's 1e-9 threshold
            q = rng.integers(0, dim) + rng.choice([-1, 1]) * (1e-9 + rng.normal(0, 1e-13))
        else:
            q = rng.uniform(0, dim)
        t = q * step
        # double_to_int
        v = t * inv
        if not (-0.5 <= v <= qlim) or abs(abs(v - np.rint(v)) - 1e-8) <= band:
            v = t / step
            n_fallback += 1
        assert double_to_int(v) == double_to_int(t / step), (k, t, step)
        # corner test and truncation (x-branch)
        qa = t * inv
        d = abs(qa - np.rint(qa))
        if not (abs(qa) <= qlim) or abs(d - 1e-9) <= band:
            qa = t / step
            d = abs(qa - np.round(qa))
        qe = t / step
        de = abs(qe - np.round(qe))
        assert (d < 1e-9) == (de < 1e-9), (k, t, step)
        if de >= 1e-9:
            assert int(qa) == int(qe), (k, t, step)
    assert n_fallback > 0
