"""The FP64 area oracle against exact rational answers.

No reference code computes an intersection area, so the oracle's area
(fo_intersection_area, a boundary integral in FP64) is pinned here by an
independent method in exact arithmetic. For any apex c, the fan triangles
T_i = (c, b_i, b_i+1) of a simple polygon B satisfy w_B = sum_i w_{T_i} for the
winding number at almost every point, so

    area(A n B) = sum_i orient(T_i) * area(A n |T_i|)

and each term is the shoelace area of A clipped by the convex triangle
(Sutherland-Hodgman), which keeps A's winding number inside the clip region.
Every coordinate is a float32 taken exactly as a Fraction, so the right-hand
side is the exact area of the two float polygons. The oracle must agree to
1e-9 relative, the engine's own tolerance against it.
"""
from fractions import Fraction

import numpy as np
import pytest

from farm_gb300 import polygons as P
from oracle import oracle as O


def exact_ring(r):
    pts = [(Fraction(float(x)), Fraction(float(y))) for x, y in np.asarray(r, np.float32)]
    if pts[0] == pts[-1]:
        pts = pts[:-1]
    return pts


def shoelace(pts):
    s = Fraction(0)
    n = len(pts)
    for i in range(n):
        x0, y0 = pts[i]
        x1, y1 = pts[(i + 1) % n]
        s += x0 * y1 - x1 * y0
    return s / 2


def clip_halfplane(pts, p, q):
    """Keep the part of closed polygon pts left of the directed line p -> q."""
    if not pts:
        return pts
    ex, ey = q[0] - p[0], q[1] - p[1]

    def side(v):
        return ex * (v[1] - p[1]) - ey * (v[0] - p[0])

    out = []
    n = len(pts)
    for i in range(n):
        a, b = pts[i], pts[(i + 1) % n]
        sa, sb = side(a), side(b)
        if sa >= 0:
            out.append(a)
        if (sa > 0 and sb < 0) or (sa < 0 and sb > 0):
            t = sa / (sa - sb)
            out.append((a[0] + t * (b[0] - a[0]), a[1] + t * (b[1] - a[1])))
    return out


def exact_intersection_area(ra, rb):
    A, B = exact_ring(ra), exact_ring(rb)
    c = B[0]  # any apex works; the first vertex drops two degenerate triangles
    total = Fraction(0)
    for i in range(1, len(B) - 1):
        t = [c, B[i], B[i + 1]]
        o = shoelace(t)
        if o == 0:
            continue
        if o < 0:
            t = [t[0], t[2], t[1]]
        clipped = A
        for k in range(3):
            clipped = clip_halfplane(clipped, t[k], t[(k + 1) % 3])
        if len(clipped) >= 3:
            total += (1 if o > 0 else -1) * shoelace(clipped)
    # A's own orientation flips the sign of every clipped area
    return abs(total)


def close(r):
    r = np.asarray(r, np.float32)
    return np.concatenate([r, r[:1]])


def test_exact_method_known_answers():
    sq = close([[0, 0], [4, 0], [4, 4], [0, 4]])
    assert exact_intersection_area(sq, close([[2, 1], [6, 1], [6, 3], [2, 3]])) == 4
    assert exact_intersection_area(sq, close([[5, 5], [6, 5], [6, 6]])) == 0
    assert exact_intersection_area(close([[1, 1], [2, 1], [2, 2], [1, 2]]), sq) == 1
    # a clockwise triangle crossing the bottom edge: the part above y = 0
    tri = close([[1, -1], [2, 3.5], [3, -1]])
    base0 = Fraction(2) * Fraction(35, 10) / Fraction(45, 10)
    assert exact_intersection_area(sq, tri) == base0 * Fraction(35, 10) / 2


def test_oracle_area_known_answers(host_built):
    sq = close([[0, 0], [4, 0], [4, 4], [0, 4]])
    cases = [
        (close([[2, 1], [6, 1], [6, 3], [2, 3]]), 4.0),
        (close([[5, 5], [6, 5], [6, 6]]), 0.0),
        (close([[1.5, 1.25], [2.5, 1.25], [2.5, 2.75], [1.5, 2.75]]), 1.5),
        (close([[1, -1], [2, 3.5], [3, -1]]), 0.5 * (2.0 * 3.5 / 4.5) * 3.5),
        # a square rotated by 45 degrees about the same centre: an octagon
        (close([[2, 2 - 2 * 2 ** 0.5], [2 + 2 * 2 ** 0.5, 2], [2, 2 + 2 * 2 ** 0.5], [2 - 2 * 2 ** 0.5, 2]]), None),
    ]
    for r, want in cases:
        got = O.intersection_area(sq, r)
        if want is None:
            want = float(exact_intersection_area(sq, r))
        assert abs(got - want) <= 1e-12 * max(want, 1.0), (got, want)


@pytest.mark.parametrize("seed,n_hi,count", [(81, 24, 14), (82, 80, 10), (83, 200, 6)])
def test_oracle_area_matches_exact_rational(host_built, seed, n_hi, count):
    # overlapping star polygons (not convex, not star-shaped about each other)
    prm = P.StarParams(dom_lo=0.0, dom_hi=3.0, r_lo=0.8, r_hi=1.5, n_lo=8, n_hi=n_hi)
    S, T = P.generate(prm, seed, count), P.generate(prm, seed + 1, count)
    nonzero = 0
    for k in range(count):
        a, b = S.ring(k), T.ring(k)
        got = O.intersection_area(a, b)
        want = exact_intersection_area(a, b)
        assert abs(Fraction(got) - want) <= Fraction(1, 10 ** 9) * want + Fraction(1, 10 ** 12), (k, got, float(want))
        # the oracle is symmetric in its two polygons
        assert abs(O.intersection_area(b, a) - got) <= 1e-12 * max(got, 1e-300)
        nonzero += want > 0
    assert nonzero >= count // 2


def test_indexed_area_oracle_equals_its_plain_definition(host_built):
    """The area oracle finds crossing edges and inside tests through spatial
    indexes; the loops over every edge pair that define it give the same
    double, bit for bit, on star polygons of mixed sizes and shapes."""
    from farm_gb300 import polygons as P
    rng = np.random.default_rng(17)
    for k in range(24):
        na, nb = int(rng.integers(4, 2500)), int(rng.integers(4, 2500))
        ra, rb = float(rng.uniform(0.2, 2.0)), float(rng.uniform(0.2, 2.0))
        pa = P.StarParams(dom_lo=5.0, dom_hi=5.0 + 1e-9, r_lo=ra, r_hi=ra, n_lo=na, n_hi=na,
                          sigma=float(rng.uniform(0.05, 0.7)))
        pb = P.StarParams(dom_lo=5.0 + float(rng.uniform(-1, 1)), dom_hi=6.0, r_lo=rb, r_hi=rb, n_lo=nb, n_hi=nb,
                          sigma=float(rng.uniform(0.05, 0.7)))
        A = P.generate(pa, 100 + k, 1).ring(0)
        B = P.generate(pb, 200 + k, 1).ring(0)
        fast, plain = O.intersection_area(A, B), O.intersection_area(A, B, plain=True)
        assert fast == plain, (k, fast, plain)
