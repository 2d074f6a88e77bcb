"""GPU within-distance (hierarchical filter + ordered refinement) gives the
reference's pair set, bit for bit."""
import numpy as np
import pytest

from fixtures import manifest, pair_case
from farm_gb300 import polygons as P
from farm_gb300.engine import Store
from oracle import oracle as O

pytestmark = pytest.mark.gpu
M = manifest()


def run_within(S, T, pairs, vpr, self_join, distance=10.0, geography=True, grid_extent=0.0):
    st = Store()
    st.load_sets(S, None if self_join else T)
    st.rasterize(vpr=vpr, hierarchy=True, grid_extent=grid_extent)
    out, found = st.within(np.ascontiguousarray(pairs, dtype=np.uint32), distance=distance, geography=geography,
                           self_join=self_join)
    stats = st.last_stats
    st.close()
    return out, found, stats


@pytest.mark.parametrize("case", [c for c in M["pairs"] if c["mode"] == "within"],
                         ids=[c["name"] for c in M["pairs"] if c["mode"] == "within"])
def test_gpu_within_matches_reference_fixture(gpu_lib, case):
    S, T, ref = pair_case(case)
    pairs = ref[:, :2].astype(np.uint32)
    out, found, _ = run_within(S, T, pairs, case["vpr"], case["self_join"])
    assert np.array_equal(out.astype(np.int64), ref[:, 2]), f"{int((out != ref[:, 2]).sum())} differ"
    assert found == int(ref[:, 2].sum())


@pytest.mark.parametrize("vpr,seed,self_join", [(10, 41, True), (4, 42, False), (64, 43, True), (2, 44, False)])
def test_gpu_within_matches_oracle(gpu_lib, vpr, seed, self_join):
    prm = P.StarParams(dom_hi=25.0, n_hi=1500)
    S = P.generate(prm, seed, 220)
    T = S if self_join else P.generate(prm, seed + 7, 260)
    pairs = P.mbr_join(S.mbrs(), T.mbrs(), expand=10.0, geography=True, skip_same=self_join)
    out, found, _ = run_within(S, T, pairs, vpr, self_join)
    RS = O.rasterize_set(S, vpr, True)
    RT = RS if self_join else O.rasterize_set(T, vpr, True)
    exp = np.array([O.within(RS[s], RT[t]) for s, t in pairs], np.uint8)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} differ"
    assert 0 < found < len(pairs)


def test_gpu_within_planar_metres(gpu_lib):
    # projected metre coordinates (configuration 3's units) need the planar
    # mode and a grid extent wider than the reference's 360 degrees
    prm = P.StarParams(dom_lo=0.0, dom_hi=2.0e5, r_lo=50.0, r_hi=5000.0, n_lo=32, n_hi=2000)
    S = P.generate(prm, 51, 300)
    d = 1000.0
    pairs = P.mbr_join(S.mbrs(), S.mbrs(), expand=d, geography=False, skip_same=True)
    out, found, _ = run_within(S, S, pairs, 10, True, distance=d, geography=False, grid_extent=1e7)
    RS = O.rasterize_set(S, 10, True, grid_extent=1e7)
    exp = np.array([O.within(RS[s], RS[t], distance=d, geography=False) for s, t in pairs], np.uint8)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} differ"
    assert 0 < found < len(pairs)


def test_gpu_within_planar_large_coordinates(gpu_lib):
    # metre coordinates up to ~1e5 (the reference's Box starts at +-100000,
    # Box.h:6-12, so beyond that its MBRs clamp): the FP32 first pass works
    # relative to each segment, so only sequence pairs whose lower bound can
    # lower the running minimum are re-evaluated in FP64; the pair set must
    # still be the reference's
    prm = P.StarParams(dom_lo=5.0e4, dom_hi=9.5e4, r_lo=50.0, r_hi=3000.0, n_lo=32, n_hi=1500)
    S = P.generate(prm, 52, 300)
    d = 500.0
    pairs = P.mbr_join(S.mbrs(), S.mbrs(), expand=d, geography=False, skip_same=True)
    out, found, stats = run_within(S, S, pairs, 10, True, distance=d, geography=False, grid_extent=1e7)
    RS = O.rasterize_set(S, 10, True, grid_extent=1e7)
    exp = np.array([O.within(RS[s], RS[t], distance=d, geography=False) for s, t in pairs], np.uint8)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} differ"
    assert 0 < found < len(pairs)
    assert stats["fp64_rechecks"] > 0


@pytest.mark.parametrize("vpr,seed,self_join", [(10, 45, True), (4, 46, False)])
def test_gpu_within_approx_matches_oracle(gpu_lib, vpr, seed, self_join):
    # the reference's within -a rule (no refinement) against the oracle's
    # restatement of it on the same descent, pair for pair; pixels small
    # against the 10 km distance, where the rule is informative
    prm = P.StarParams(dom_hi=2.0, r_lo=0.005, r_hi=0.06, n_hi=1500)
    S = P.generate(prm, seed, 220)
    T = S if self_join else P.generate(prm, seed + 7, 260)
    pairs = np.ascontiguousarray(P.mbr_join(S.mbrs(), T.mbrs(), expand=10.0, geography=True, skip_same=self_join),
                                 dtype=np.uint32)
    st = Store()
    st.load_sets(S, None if self_join else T)
    st.rasterize(vpr=vpr, hierarchy=True)
    out, found = st.within(pairs, distance=10.0, self_join=self_join, mode=1)
    stats = st.last_stats
    exact, _ = st.within(pairs, distance=10.0, self_join=self_join)
    st.close()
    assert stats["segment_tests"] == 0
    RS = O.rasterize_set(S, vpr, True)
    RT = RS if self_join else O.rasterize_set(T, vpr, True)
    exp = np.array([O.within_heuristic(RS[s], RT[t]) for s, t in pairs], np.uint8)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} differ"
    assert found == int(exp.sum()) and 0 < found < len(pairs)
    # a heuristic: most pairs agree with the exact answer
    assert (out == exact).mean() > 0.9
