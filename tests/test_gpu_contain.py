"""GPU containment queries against the reference's own decisions (fixtures
made by its compiled CPU code) and against the oracle on larger inputs.

farm_contain is Ideal::contain(Ideal *) per (source, target) pair and
farm_contain_points Ideal::contain(Point &) per (polygon, point) pair; both
are boolean and must match bit for bit.
"""
import numpy as np
import pytest

from fixtures import manifest, pair_case, point_case
from farm_gb300 import polygons as P
from farm_gb300.engine import Store
from oracle import oracle as O

pytestmark = pytest.mark.gpu

M = manifest()


@pytest.mark.parametrize("case", M["contain"], ids=[c["name"] for c in M["contain"]])
def test_gpu_contain_matches_reference_fixture(gpu_lib, case):
    S, T, ref = pair_case(case)
    pairs = np.ascontiguousarray(ref[:, :2].astype(np.uint32))
    with Store() as st:
        st.load_sets(S, T)
        st.rasterize(vpr=case["vpr"])
        out, found = st.contain(pairs)
    assert np.array_equal(out.astype(np.int64), ref[:, 2]), f"{int((out != ref[:, 2]).sum())} pairs differ"
    assert found == int(ref[:, 2].sum())


@pytest.mark.parametrize("case", M["contain_point"], ids=[c["name"] for c in M["contain_point"]])
def test_gpu_contain_points_matches_reference_fixture(gpu_lib, case):
    S, pts, ref = point_case(case)
    pairs = np.ascontiguousarray(ref[:, :2].astype(np.uint32))
    with Store() as st:
        st.load(0, S.off, S.xy)
        st.rasterize(vpr=case["vpr"])
        out, found = st.contain_points(pts, pairs)
    assert np.array_equal(out.astype(np.int64), ref[:, 2]), f"{int((out != ref[:, 2]).sum())} pairs differ"
    assert found == int(ref[:, 2].sum())


@pytest.mark.parametrize("vpr,hier", [(64, False), (128, False), (10, True)])
def test_gpu_contain_large_sources_match_oracle(gpu_lib, vpr, hier):
    """Sources of 5k-60k vertices holding targets of 8-5,000 vertices, all MBR
    candidates, device pairs and outputs (torch), against the oracle."""
    import torch
    src = P.StarParams(dom_hi=16.0, r_lo=2.0, r_hi=4.0, n_lo=5000, n_hi=60000)
    tgt = P.StarParams(dom_hi=16.0, r_lo=0.02, r_hi=0.8, n_lo=8, n_hi=5000)
    S, T = P.generate(src, 41 + vpr, 10), P.generate(tgt, 42 + vpr, 600)
    pairs = np.ascontiguousarray(P.mbr_join(S.mbrs(), T.mbrs()), dtype=np.uint32)
    with Store() as st:
        st.load_sets(S, T)
        st.rasterize(vpr=vpr, hierarchy=hier, strict=False)
        dp = torch.from_numpy(pairs.view(np.int32)).cuda()
        out_d, found = st.contain(dp)
        out = out_d.cpu().numpy()
    RS = O.rasterize_many([S.ring(k) for k in range(S.n)], vpr, hierarchy=hier)
    RT = O.rasterize_many([T.ring(k) for k in range(T.n)], vpr, hierarchy=hier)
    exp = O.contain_many(RS, RT, pairs)
    assert np.array_equal(out, exp), f"-v {vpr}: {int((out != exp).sum())} of {len(exp)} pairs differ"
    assert found == int((exp == 1).sum())
    assert 0 < int((exp == 1).sum()) < len(exp)


def test_gpu_contain_points_on_boundaries_match_oracle(gpu_lib):
    """Points on vertices, edge midpoints and pixel grid lines of 20k-vertex
    polygons at -v 64, host memory."""
    prm = P.StarParams(dom_hi=10.0, r_lo=1.0, r_hi=3.0, n_lo=20000, n_hi=40000)
    S = P.generate(prm, 51, 4)
    rng = np.random.default_rng(3)
    pts = [rng.uniform(-1, 11, (20000, 2)).astype(np.float32)]
    for k in range(S.n):
        r = S.ring(k).astype(np.float64)
        pts.append(r[::13].astype(np.float32))
        pts.append(((r[:-1:17] + r[1::17][: len(r[:-1:17])]) / 2).astype(np.float32))
    pts = np.ascontiguousarray(np.concatenate(pts), dtype=np.float32)
    mb = S.mbrs()
    pairs = np.array([(p, q) for q in range(len(pts)) for p in range(S.n)
                      if mb[p, 0] <= pts[q, 0] <= mb[p, 2] and mb[p, 1] <= pts[q, 1] <= mb[p, 3]], np.uint32)
    with Store() as st:
        st.load(0, S.off, S.xy)
        st.rasterize(vpr=64, strict=False)
        out, found = st.contain_points(pts, pairs)
        # the pixel grid: points on the polygon's vertical grid lines
        v = st.fetch_raster(0, 0)
    RS = O.rasterize_many([S.ring(k) for k in range(S.n)], 64)
    exp = O.contain_points_many(RS, pts, pairs)
    assert np.array_equal(out, exp), f"{int((out != exp).sum())} of {len(exp)} pairs differ"
    assert 0 < found < len(pairs)
    # grid-line points of polygon 0: x on a vertical line, y anywhere in the MBR
    mbr, step = v["mbr"], v["step"]
    xs = (mbr[0] + np.arange(1, v["dimx"]) * step[0]).astype(np.float32)
    ys = rng.uniform(mbr[1], mbr[3], len(xs)).astype(np.float32)
    gp = np.ascontiguousarray(np.stack([xs, ys], 1))
    gpairs = np.ascontiguousarray(np.stack([np.zeros(len(gp), np.uint32), np.arange(len(gp), dtype=np.uint32)], 1))
    with Store() as st:
        st.load(0, S.off, S.xy)
        st.rasterize(vpr=64, strict=False)
        gout, _ = st.contain_points(gp, gpairs)
    gexp = O.contain_points_many(RS, gp, gpairs)
    assert np.array_equal(gout, gexp)


def test_gpu_contain_rejects_out_of_range(gpu_lib):
    from farm_gb300._native import FarmError
    prm = P.StarParams(dom_hi=10.0, n_hi=200)
    S, T = P.generate(prm, 61, 10), P.generate(prm, 62, 20)
    pts = np.zeros((5, 2), np.float32)
    with Store() as st:
        st.load_sets(S, T)
        st.rasterize(vpr=10)
        with pytest.raises(FarmError, match="out of range"):
            st.contain(np.array([[0, T.n]], np.uint32))
        with pytest.raises(FarmError, match="out of range"):
            st.contain_points(pts, np.array([[0, 5]], np.uint32))
        with pytest.raises(FarmError, match="out of range"):
            st.contain_points(pts, np.array([[T.n, 0]], np.uint32), side=1)
        out, _ = st.contain_points(pts, np.array([[T.n - 1, 4]], np.uint32), side=1)
        assert out.tolist() in ([0], [1])


def test_gpu_contain_points_refuses_misaligned_device_points(gpu_lib):
    import torch
    from farm_gb300._native import FarmError
    prm = P.StarParams(dom_hi=10.0, n_hi=200)
    S = P.generate(prm, 63, 10)
    dev = torch.device("cuda:0")
    buf = torch.zeros(11, dtype=torch.float32, device=dev)
    pts = buf[1:].view(5, 2)  # 4 bytes into the allocation
    pairs = torch.tensor([[0, 0], [1, 4]], dtype=torch.int32, device=dev)
    with Store() as st:
        st.load(0, S.off, S.xy)
        st.rasterize(vpr=10)
        with pytest.raises(FarmError, match="8-byte"):
            st.contain_points(pts, pairs)
        out, _ = st.contain_points(buf[:10].view(5, 2), pairs)  # aligned: answers
        assert out.shape[0] == 2
