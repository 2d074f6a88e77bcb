"""GPU intersection area (stage d) against the FP64 CPU oracle, 1e-9 relative."""
import numpy as np
import pytest

from farm_gb300 import polygons as P
from farm_gb300.engine import Store
from oracle import oracle as O

pytestmark = pytest.mark.gpu
# 1e-9 relative, plus an absolute floor at FP64's conditioning limit for
# slivers: the boundary integral sums O(polygon area) terms, so no FP64 method
# resolves an intersection below ~1e-14 of the polygons' own area.
RTOL = 1e-9
FLOOR = 1e-14


def mkset(rings):
    off = np.zeros(len(rings) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rings])
    return P.PolygonSet(off, np.ascontiguousarray(np.concatenate(rings), dtype=np.float32))


def ring_area(r):
    r = r.astype(np.float64)
    return 0.5 * abs(np.sum(r[:-1, 0] * r[1:, 1] - r[1:, 0] * r[:-1, 1]))


def run_area(S, T, pairs, vpr=10):
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=vpr)
    out = st.intersection_area(np.ascontiguousarray(pairs, dtype=np.uint32))
    st.close()
    return out


def check(S, T, pairs, out):
    for k, (s, t) in enumerate(pairs):
        exp = O.intersection_area(S.ring(s), T.ring(t))
        tol = RTOL * exp + FLOOR * max(ring_area(S.ring(s)), ring_area(T.ring(t)))
        assert abs(out[k] - exp) <= tol, (k, s, t, out[k], exp)


def test_gpu_area_known_answers(gpu_lib):
    sq = np.array([[0, 0], [4, 0], [4, 4], [0, 4], [0, 0]], np.float32)
    tri = np.array([[1, -1], [3, -1], [2, 3.5], [1, -1]], np.float32)  # crosses the bottom edge
    small = np.array([[1.5, 1.25], [2.5, 1.25], [2.5, 2.75], [1.5, 2.75], [1.5, 1.25]], np.float32)  # inside
    far = sq + np.float32(10.0)
    cw = sq[::-1].copy()  # clockwise copy, shifted
    cw = cw + np.float32(0.5)
    S = mkset([sq, sq, sq, sq])
    T = mkset([tri, small, far, cw])
    pairs = np.array([[0, 0], [1, 1], [2, 2], [3, 3]], np.uint32)
    out = run_area(S, T, pairs)
    # triangle (1,-1),(3,-1),(2,3.5) above y=0: similar triangle of height 3.5
    h = 3.5
    above = 0.5 * (2.0 * 3.5 / 4.5) * 3.5  # base at y=0 scaled by (4.5-1)/4.5... computed below
    base0 = 2.0 * (3.5 - 0.0) / 4.5  # width at y = 0
    above = 0.5 * base0 * 3.5
    assert abs(out[0] - above) <= 1e-9 * above
    assert abs(out[1] - 1.0 * 1.5) <= 1e-12
    assert out[2] == 0.0
    assert abs(out[3] - 3.5 * 3.5) <= 1e-9 * 12.25


@pytest.mark.parametrize("vpr,seed", [(10, 61), (4, 62), (64, 63)])
def test_gpu_area_matches_oracle(gpu_lib, vpr, seed):
    prm = P.StarParams(dom_hi=15.0, n_lo=8, n_hi=800)
    S, T = P.generate(prm, seed, 80), P.generate(prm, seed + 1, 200)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    out = run_area(S, T, pairs, vpr)
    check(S, T, pairs, out)
    assert (out > 0).sum() > len(out) // 4
