"""The CPU oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by compiling the reference's unmodified CPU code
(tests/golden/make_golden.py); a match here pins the oracle that every GPU
parity test then compares the engine with.
"""
import hashlib

import numpy as np
import pytest

from fixtures import manifest, pair_case, point_case, raster_case, raster_mismatches
from farm_gb300.polygons import degree_table, mbr_join
from oracle import oracle as O

M = manifest()


@pytest.mark.parametrize("case", M["raster"], ids=[c["name"] for c in M["raster"]])
def test_oracle_raster_matches_reference(host_built, case):
    ps, ref = raster_case(case)
    assert ps.n == len(ref)
    for k in range(ps.n):
        r = O.Raster(ps.ring(k), case["vpr"], bool(case["hierarchy"])).arrays()
        bad = raster_mismatches(r, ref[k])
        assert not bad, f"polygon {k}: {bad}"
        assert r["layers"] == ref[k]["layers"]


@pytest.mark.parametrize("case", M["pairs"], ids=[c["name"] for c in M["pairs"]])
def test_oracle_pairs_match_reference(host_built, case):
    S, T, ref = pair_case(case)
    within = case["mode"] == "within"
    if within:
        pairs = mbr_join(S.mbrs(), T.mbrs(), expand=10.0, geography=True, skip_same=True)
    else:
        pairs = mbr_join(S.mbrs(), T.mbrs())
    # the candidate join equals the reference's R-tree join
    assert np.array_equal(pairs.astype(np.int64), ref[:, :2])
    RS = O.rasterize_set(S, case["vpr"], within)
    RT = RS if case["self_join"] else O.rasterize_set(T, case["vpr"], within)
    got = np.array([O.within(RS[s], RT[t]) if within else O.intersect(RS[s], RT[t]) for s, t in pairs], np.int64)
    assert np.array_equal(got, ref[:, 2]), f"{int((got != ref[:, 2]).sum())} mismatching pairs"
    assert 0 < got.sum() < len(got)  # both outcomes occur


def test_degree_table_matches_reference(host_built):
    t = degree_table()
    txt = ",".join("%.6f" % v for v in t)
    assert hashlib.sha256(txt.encode()).hexdigest() == M["degree_table"]["sha256_of_6_decimal_text"]
    # the oracle's own copy agrees
    for lat in (0.0, 12.34, 45.0, 89.95, 90.0):
        i = min(int(abs(lat if lat != 90 else 89.9) * 10), 899)
        assert O.lib().fo_degree_per_km_longitude(lat) == t[i]


def test_segment_predicates_known_answers(host_built):
    import ctypes as C
    L = O.lib()

    def si(a, b, c, d):
        arr = [np.array(v, np.float32) for v in (a, b, c, d)]
        fp = C.POINTER(C.c_float)
        return L.fo_segment_intersect(*[x.ctypes.data_as(fp) for x in arr])

    assert si((0, 0), (2, 2), (0, 2), (2, 0)) == 1          # proper crossing
    assert si((0, 0), (1, 1), (2, 2), (3, 3)) == 0          # collinear, disjoint
    assert si((0, 0), (2, 2), (1, 1), (3, 3)) == 1          # collinear overlap
    assert si((0, 0), (1, 0), (1, 0), (2, 5)) == 1          # shared endpoint
    assert si((0, 0), (1, 0), (0, 1), (1, 1)) == 0          # parallel
    fp = C.POINTER(C.c_float)
    p, a, b = (np.array(v, np.float32) for v in ((0, 1), (-1, 0), (1, 0)))
    d = L.fo_point_to_segment_distance(p.ctypes.data_as(fp), a.ctypes.data_as(fp), b.ctypes.data_as(fp), 0)
    assert d == 1.0



def test_oracle_within_heuristic_small_pixels(host_built):
    # The within -a rule has no CPU counterpart in the reference to pin it
    # to. It judges a pixel pair by the midpoint of its box distance range, so
    # it is only informative where pixels are small against the distance:
    # polygons of 0.5-7 km radius and 10 km here, where it agrees with the
    # exact answer on most pairs (with 40 km pixels it says false throughout).
    from farm_gb300 import polygons as P
    prm = P.StarParams(dom_hi=2.0, r_lo=0.005, r_hi=0.06, n_hi=1500)
    S = P.generate(prm, 45, 220)
    pairs = P.mbr_join(S.mbrs(), S.mbrs(), expand=10.0, geography=True, skip_same=True)
    RS = O.rasterize_set(S, 10, True)
    exact = np.array([O.within(RS[s], RS[t]) for s, t in pairs], np.int64)
    apx = np.array([O.within_heuristic(RS[s], RS[t]) for s, t in pairs], np.int64)
    assert (apx == exact).mean() > 0.9
    assert 0 < apx.sum() < len(apx)
    # far apart: the descent prunes every pixel pair; the same polygon: the
    # descent decides it
    sq = np.array([[0, 0], [0.01, 0], [0.01, 0.01], [0, 0.01], [0, 0]], np.float32)
    a, b = O.Raster(sq, 10, True), O.Raster(sq + np.float32(1.0), 10, True)
    assert not O.within_heuristic(a, b) and not O.within(a, b)
    assert O.within_heuristic(a, a) and O.within(a, a)


@pytest.mark.parametrize("case", M.get("contain", []), ids=[c["name"] for c in M.get("contain", [])])
def test_oracle_contain_matches_reference(host_built, case):
    """Ideal::contain(Ideal *) of every MBR candidate pair (large sources, small
    targets): the oracle against the reference's decisions."""
    S, T, ref = pair_case(case)
    pairs = mbr_join(S.mbrs(), T.mbrs())
    assert np.array_equal(pairs.astype(np.int64), ref[:, :2])
    RS, RT = O.rasterize_set(S, case["vpr"]), O.rasterize_set(T, case["vpr"])
    got = O.contain_many(RS, RT, pairs)
    assert np.array_equal(got.astype(np.int64), ref[:, 2]), f"{int((got != ref[:, 2]).sum())} mismatching pairs"
    assert 0 < got.sum() < len(got)


@pytest.mark.parametrize("case", M.get("contain_point", []), ids=[c["name"] for c in M.get("contain_point", [])])
def test_oracle_contain_point_matches_reference(host_built, case):
    """Ideal::contain(Point &) of every (polygon, point) pair whose MBR holds
    the point, points on vertices and edge midpoints included."""
    S, pts, ref = point_case(case)
    RS = O.rasterize_set(S, case["vpr"])
    got = O.contain_points_many(RS, pts, ref[:, :2])
    assert np.array_equal(got.astype(np.int64), ref[:, 2]), f"{int((got != ref[:, 2]).sum())} mismatching pairs"
    assert 0 < got.sum() < len(got)
