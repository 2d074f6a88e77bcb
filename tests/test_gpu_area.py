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


def _mixed_sets(seed):
    # configuration 4 in miniature: tiny and huge polygons mixed in one batch
    rng = np.random.default_rng(seed)
    small = P.StarParams(dom_hi=12.0, r_lo=0.2, r_hi=1.0, n_lo=8, n_hi=40)
    big = P.StarParams(dom_hi=12.0, r_lo=1.0, r_hi=2.0, n_lo=500, n_hi=3000)
    A, B = P.generate(small, seed, 120), P.generate(big, seed + 1, 12)
    C, D = P.generate(small, seed + 2, 120), P.generate(big, seed + 3, 12)
    S = P.PolygonSet(np.concatenate([A.off[:-1], A.off[-1] + B.off]).astype(np.uint64), np.concatenate([A.xy, B.xy]))
    T = P.PolygonSet(np.concatenate([C.off[:-1], C.off[-1] + D.off]).astype(np.uint64), np.concatenate([C.xy, D.xy]))
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    return S, T, pairs[rng.permutation(len(pairs))]


def _checkable(S, T, pairs, k=40):
    # pairs the O(n m) oracle finishes quickly: tiny x tiny and tiny x huge
    return [i for i, (s, t) in enumerate(pairs) if len(S.ring(s)) * len(T.ring(t)) < 2_000_000][:k]


def test_gpu_area_plan_replays_graph(gpu_lib):
    # one captured graph, replayed on two different batches: the same doubles
    # as the direct call, and a batch beyond capacity is refused
    S, T, pairs = _mixed_sets(61)
    assert len(pairs) > 200
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=10)
    half = len(pairs) // 2
    b1, b2 = np.ascontiguousarray(pairs[:half]), np.ascontiguousarray(pairs[half:])
    ref1, ref2 = st.intersection_area(b1), st.intersection_area(b2)
    plan = st.area_plan(max_pairs=len(pairs), max_items=1 << 20)
    got1, got2 = plan.run(b1), plan.run(b2)
    assert np.array_equal(got1, ref1) and np.array_equal(got2, ref2)
    assert plan.last_stats["kernel_launches"] == 1
    from farm_gb300._native import FarmError
    with pytest.raises(FarmError):
        plan.run(np.ascontiguousarray(np.concatenate([pairs, pairs])))
    small = st.area_plan(max_pairs=len(pairs), max_items=4)
    with pytest.raises(FarmError) as ei:
        small.run(b1)
    assert ei.value.code == -4  # FARM_EOVERFLOW
    plan.close()
    small.close()
    sel = _checkable(S, T, b1)
    check(S, T, b1[sel], ref1[sel])
    st.close()


def test_gpu_area_autotune(gpu_lib):
    # the tuned chunk table changes how edges are split into work items, not
    # the answer (within the FP64 tolerance)
    S, T, pairs = _mixed_sets(62)
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=10)
    base = st.intersection_area(pairs)
    tab, wide = st.area_autotune(pairs, with_wide=True)
    assert tab.shape == (32,) and (tab > 0).any()
    assert set(np.unique(tab[tab > 0])) <= {8, 16, 32, 64, 128, 256}
    assert set(np.unique(wide[tab > 0])) <= {24, 48, 200, 800}
    tuned = st.intersection_area(pairs)
    st.close()
    scale = np.maximum(base, 1e-300)
    assert np.all(np.abs(tuned - base) <= 1e-9 * scale + 1e-12)
    sel = _checkable(S, T, pairs)
    check(S, T, pairs[sel], tuned[sel])


def _star(nv, cx, cy, r, seed, sigma=0.3):
    prm = P.StarParams(dom_lo=0.0, dom_hi=1e-9, r_lo=r, r_hi=r, n_lo=nv, n_hi=nv, sigma=sigma)
    ring = P.generate(prm, seed, 1).ring(0).astype(np.float64)
    ring[:, 0] += cx
    ring[:, 1] += cy
    return ring.astype(np.float32)


_LARGE = {}


@pytest.mark.parametrize("vpr", [10, 64])
def test_gpu_area_large_polygons(gpu_lib, vpr):
    """Configuration 4's heavy side: polygons of 50k-200k vertices against
    sparser polygons whose long spiky edges cross them thousands of times
    (the case the warp-shared window search exists for), against the FP64
    oracle (a thread per pair) at 1e-9 relative. The radii keep consecutive
    vertices a hundred float spacings apart or more, so that rounding the
    coordinates to float32 leaves every ring simple (general position, which
    the boundary integral assumes)."""
    import concurrent.futures as cf
    dense = [_star(200_000, 10.0, 10.0, 8.0, 1, sigma=0.15), _star(100_000, 10.5, 9.7, 5.0, 2, sigma=0.15),
             _star(50_000, 9.5, 10.3, 4.0, 3, sigma=0.2)]
    sparse = [_star(4_000, 10.2, 10.1, 9.0, 11, sigma=0.5), _star(9_000, 9.8, 10.2, 7.0, 12, sigma=0.5),
              _star(1_500, 10.3, 9.9, 6.0, 13, sigma=0.6), _star(20_000, 10.0, 10.4, 8.0, 14, sigma=0.4)]
    S, T = mkset(dense), mkset(sparse)
    pairs = np.array([[0, 0], [0, 2], [1, 1], [1, 0], [2, 3], [2, 2]], np.uint32)
    out = run_area(S, T, pairs, vpr)
    if "exp" not in _LARGE:  # the oracle does not depend on -v: computed once
        with cf.ThreadPoolExecutor(max_workers=len(pairs)) as ex:
            _LARGE["exp"] = list(ex.map(lambda st: O.intersection_area(S.ring(int(st[0])), T.ring(int(st[1]))),
                                        pairs))
    exp = _LARGE["exp"]
    for k, (s, t) in enumerate(pairs):
        tol = RTOL * exp[k] + FLOOR * max(ring_area(S.ring(s)), ring_area(T.ring(t)))
        assert abs(out[k] - exp[k]) <= tol, (k, s, t, out[k], exp[k])
        assert exp[k] > 0
