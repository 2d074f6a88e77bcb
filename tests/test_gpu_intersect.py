"""GPU intersect (stages b + c) gives the reference's pair set, bit for bit."""
import numpy as np
import pytest

from fixtures import manifest, pair_case
from farm_gb300 import polygons as P
from farm_gb300.engine import Store
from oracle import oracle as O

pytestmark = pytest.mark.gpu
M = manifest()


def run(S, T, pairs, vpr, cc=16):
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=vpr, category_count=cc)
    out, found = st.intersect(np.ascontiguousarray(pairs, dtype=np.uint32))
    stats = st.last_stats
    st.close()
    return out, found, stats


@pytest.mark.parametrize("case", [c for c in M["pairs"] if c["mode"] == "intersect"],
                         ids=[c["name"] for c in M["pairs"] if c["mode"] == "intersect"])
def test_gpu_intersect_matches_reference_fixture(gpu_lib, case):
    S, T, ref = pair_case(case)
    pairs = ref[:, :2].astype(np.uint32)
    out, found, _ = run(S, T, pairs, case["vpr"])
    assert np.array_equal(out.astype(np.int64), ref[:, 2])
    assert found == int(ref[:, 2].sum())


@pytest.mark.parametrize("vpr,cc,seed", [(10, 16, 11), (4, 16, 12), (64, 4, 13), (1, 256, 14)])
def test_gpu_intersect_matches_oracle(gpu_lib, vpr, cc, seed):
    prm = P.StarParams(dom_hi=25.0, n_hi=1500)
    S, T = P.generate(prm, seed, 150), P.generate(prm, seed + 100, 500)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    out, found, stats = run(S, T, pairs, vpr, cc)
    RS, RT = O.rasterize_set(S, vpr), O.rasterize_set(T, vpr)
    exp = np.array([O.intersect(RS[s], RT[t]) for s, t in pairs], np.uint8)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} differ"
    assert stats["pairs"] == len(pairs)


def test_gpu_intersect_edge_cases(gpu_lib):
    sq = np.array([[0, 0], [2, 0], [2, 2], [0, 2], [0, 0]], np.float32)
    rings_s = [sq, sq + 5, sq * 0.25 + 0.8]
    rings_t = [sq, sq + np.float32(1), sq + np.float32(2), sq * 0.1 + 0.9, sq + 5.5]
    mk = lambda rs: P.PolygonSet(np.concatenate([[0], np.cumsum([len(r) for r in rs])]).astype(np.uint64),
                                 np.ascontiguousarray(np.concatenate(rs), dtype=np.float32))
    S, T = mk(rings_s), mk(rings_t)
    pairs = np.array([[s, t] for s in range(S.n) for t in range(T.n)], np.uint32)
    for vpr in (1, 2, 10):
        out, found, _ = run(S, T, pairs, vpr)
        RS, RT = O.rasterize_set(S, vpr), O.rasterize_set(T, vpr)
        exp = np.array([O.intersect(RS[s], RT[t]) for s, t in pairs], np.uint8)
        assert np.array_equal(out, exp), vpr
    # empty pair list
    out, found, _ = run(S, T, np.zeros((0, 2), np.uint32), 10)
    assert found == 0 and len(out) == 0


def test_gpu_intersect_marks_pairs_of_unrasterizable_polygons(gpu_lib):
    from farm_gb300._native import FarmError
    # the diamond's edges pass exactly through grid corners at -v 1: the
    # reference's edge walk never terminates on it; the engine flags it
    diamond = np.array([[0, 0], [3, 3], [0, 6], [-3, 3], [0, 0]], np.float32)
    sq = np.array([[-1, 1], [1, 1], [1, 5], [-1, 5], [-1, 1]], np.float32)
    mk = lambda rs: P.PolygonSet(np.concatenate([[0], np.cumsum([len(r) for r in rs])]).astype(np.uint64),
                                 np.ascontiguousarray(np.concatenate(rs), dtype=np.float32))
    S, T = mk([diamond, sq]), mk([sq, diamond])
    st = Store()
    st.load_sets(S, T)
    with pytest.raises(FarmError):
        st.rasterize(vpr=1)
    assert st.raster_errors(0).tolist() == [-10, 0] and st.raster_errors(1).tolist() == [0, -10]
    pairs = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.uint32)
    out, found = st.intersect(pairs)
    RS, RT = O.Raster(sq, 1), O.Raster(sq, 1)
    assert out.tolist() == [2, int(O.intersect(RS, RT)), 2, 2]
    assert found == int(out[1] == 1)
    st.close()


def test_gpu_intersect_lattice_collinear(gpu_lib):
    # axis-aligned rectangles and right triangles on an integer lattice: edges
    # that overlap collinearly, touch end to end or meet at corners, which the
    # refinement settles with the collinear interval rule
    rng = np.random.default_rng(5)

    def shapes(n):
        rings = []
        for _ in range(n):
            x0, y0 = rng.integers(0, 12, 2)
            w, h = rng.integers(1, 5, 2)
            if rng.random() < 0.5:
                r = [[x0, y0], [x0 + w, y0], [x0 + w, y0 + h], [x0, y0 + h], [x0, y0]]
            else:
                r = [[x0, y0], [x0 + w, y0], [x0, y0 + h], [x0, y0]]
            rings.append(np.array(r, np.float32))
        off = np.zeros(n + 1, np.uint64)
        off[1:] = np.cumsum([len(r) for r in rings])
        return P.PolygonSet(off, np.ascontiguousarray(np.concatenate(rings)))

    def ras(ps, vpr):
        out = []
        for k in range(ps.n):
            try:
                out.append(O.Raster(ps.ring(k), vpr))
            except RuntimeError:  # the reference aborts on this polygon
                out.append(None)
        return out

    S, T = shapes(60), shapes(80)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    for vpr in (1, 2, 3):
        RS, RT = ras(S, vpr), ras(T, vpr)
        ok = [i for i, (s, t) in enumerate(pairs) if RS[s] is not None and RT[t] is not None]
        st = Store()
        st.load_sets(S, T)
        st.rasterize(vpr=vpr, strict=False)
        out, _ = st.intersect(np.ascontiguousarray(pairs, dtype=np.uint32))
        st.close()
        exp = np.array([O.intersect(RS[pairs[i][0]], RT[pairs[i][1]]) for i in ok], np.uint8)
        assert np.array_equal(out[ok], exp), (vpr, int((out[ok] != exp).sum()))
        assert len(ok) > len(pairs) // 2


@pytest.mark.parametrize("vpr,seed", [(10, 41), (4, 42), (32, 43)])
def test_gpu_intersect_approx_heuristic_matches_oracle(gpu_lib, vpr, seed):
    # FARM_MODE_APPROX is the reference's -a fill-ratio heuristic: no
    # refinement, decided by IN overlaps and (apx_s + apx_t) / max area > 1
    from farm_gb300.engine import MODE_APPROX
    prm = P.StarParams(dom_hi=25.0, n_hi=1500)
    S, T = P.generate(prm, seed, 150), P.generate(prm, seed + 100, 500)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=vpr)
    out, found = st.intersect(np.ascontiguousarray(pairs, dtype=np.uint32), mode=MODE_APPROX)
    st.close()
    RS, RT = O.rasterize_set(S, vpr), O.rasterize_set(T, vpr)
    exp = np.array([O.intersect_heuristic(RS[s], RT[t]) for s, t in pairs], np.uint8)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} differ"
    assert found == int(exp.sum())
