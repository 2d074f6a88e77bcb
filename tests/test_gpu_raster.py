"""GPU rasterization (stage a) is byte-identical to the reference's raster."""
import numpy as np
import pytest

from fixtures import manifest, raster_case, raster_mismatches
from farm_gb300 import polygons as P
from farm_gb300.engine import Store
from oracle import oracle as O

pytestmark = pytest.mark.gpu
M = manifest()


def gpu_rasters(ps, vpr, hier, side=0, cc=16):
    st = Store()
    st.load(0, ps.off, ps.xy)
    st.rasterize(vpr=vpr, category_count=cc, hierarchy=hier)
    return st, [st.fetch_raster(0, k) for k in range(ps.n)]


def layer_tuples(layers):
    return [(tuple(m), dx, dy, sx, sy) for (m, dx, dy, sx, sy, *_rest) in layers]


@pytest.mark.parametrize("case", M["raster"], ids=[c["name"] for c in M["raster"]])
def test_gpu_raster_matches_reference_fixture(gpu_lib, case):
    ps, ref = raster_case(case)
    st, got = gpu_rasters(ps, case["vpr"], bool(case["hierarchy"]))
    for k in range(ps.n):
        assert got[k]["err"] == 0
        bad = raster_mismatches(got[k], ref[k])
        assert not bad, f"polygon {k}: {bad}"
        assert layer_tuples(got[k]["layers"]) == layer_tuples(ref[k]["layers"])
    st.close()


@pytest.mark.parametrize("vpr,hier,seed", [(10, 0, 1), (2, 1, 2), (32, 0, 3), (10, 1, 4)])
def test_gpu_raster_matches_oracle_random(gpu_lib, vpr, hier, seed):
    ps = P.generate(P.StarParams(dom_hi=30.0, n_hi=2048), seed, 400)
    st, got = gpu_rasters(ps, vpr, bool(hier))
    for k in range(ps.n):
        r = O.Raster(ps.ring(k), vpr, bool(hier)).arrays()
        bad = raster_mismatches(got[k], r)
        assert not bad, f"polygon {k}: {bad}"
    st.close()


@pytest.mark.parametrize("cc", [4, 256])
def test_gpu_raster_category_counts(gpu_lib, cc):
    ps = P.generate(P.StarParams(dom_hi=30.0), 9, 150)
    st, got = gpu_rasters(ps, 10, False, cc=cc)
    for k in range(ps.n):
        r = O.Raster(ps.ring(k), 10, False, category_count=cc).arrays()
        assert not raster_mismatches(got[k], r), k
    st.close()


def test_gpu_raster_edge_cases(gpu_lib):
    # single-pixel polygons, axis-aligned edges, a polygon on the grid corners
    rings = [
        np.array([[0, 0], [1, 0], [1, 1], [0, 1], [0, 0]], np.float32),
        np.array([[0, 0], [4, 0], [4, 4], [2, 6], [0, 4], [0, 0]], np.float32),
        np.array([[10, 10], [10.5, 10], [10.5, 10.25], [10, 10]], np.float32),
        np.array([[0, 0], [3, 3], [0, 6], [-3, 3], [0, 0]], np.float32),
        np.array([[1, 1], [9, 1], [9, 2], [2, 2], [2, 8], [9, 8], [9, 9], [1, 9], [1, 1]], np.float32),
    ]
    off = np.zeros(len(rings) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rings])
    ps = P.PolygonSet(off, np.ascontiguousarray(np.concatenate(rings)))
    from farm_gb300._native import FarmError
    for vpr in (1, 2, 10):
        exp = {}
        for k in range(ps.n):
            try:
                exp[k] = O.Raster(ps.ring(k), vpr, False).arrays()
            except RuntimeError:
                exp[k] = None  # the reference aborts or loops forever on this polygon
        st = Store()
        st.load(0, ps.off, ps.xy)
        if any(v is None for v in exp.values()):
            with pytest.raises(FarmError) as ei:
                st.rasterize(vpr=vpr)
            assert ei.value.code == -10
        else:
            st.rasterize(vpr=vpr)
        for k in range(ps.n):
            g = st.fetch_raster(0, k)
            if exp[k] is None:
                assert g["err"] == -10, (vpr, k)
            else:
                assert g["err"] == 0 and not raster_mismatches(g, exp[k]), (vpr, k)
        st.close()


def test_gpu_raster_many_chunks(gpu_lib, monkeypatch):
    # tiny scratch budgets force one or two polygons per chunk
    monkeypatch.setenv("FARM_CHUNK_EDGES", "700")
    monkeypatch.setenv("FARM_CHUNK_CROSS", "300")
    monkeypatch.setenv("FARM_CHUNK_PIX", "64")
    ps = P.generate(P.StarParams(dom_hi=30.0, n_hi=1200), 21, 120)
    for hier in (False, True):
        st, got = gpu_rasters(ps, 4, hier)
        for k in range(ps.n):
            r = O.Raster(ps.ring(k), 4, hier).arrays()
            assert not raster_mismatches(got[k], r), (hier, k)
        st.close()


def _ulp_chains(ps, steps=(1, 2, 3)):
    """Each vertex followed by copies nudged by 1..3 float ulps: distinct points
    within 1e-9 of each other (near the origin), including non-transitive
    chains (v ~ v+1ulp ~ v+2ulp, but v !~ v+3ulp)."""
    rings = []
    for k in range(ps.n):
        r = ps.ring(k)[:-1]
        out = []
        for i, v in enumerate(r):
            out.append(v)
            if i % 3 == 0:
                for s in steps:
                    w = v.copy()
                    for _ in range(s):
                        w = np.nextafter(w, np.float32(np.inf)).astype(np.float32)
                    out.append(w)
        out.append(r[0])
        rings.append(np.array(out, np.float32))
    off = np.zeros(len(rings) + 1, np.uint64)
    off[1:] = np.cumsum([len(r) for r in rings])
    return P.PolygonSet(off, np.ascontiguousarray(np.concatenate(rings)))


@pytest.mark.parametrize("vpr,seed", [(1, 31), (4, 32), (16, 33)])
def test_gpu_raster_small_point_tolerance(gpu_lib, vpr, seed):
    # every coordinate below 2^-5: the fill clip's point dedup runs on the
    # 1e-9 tolerance rule, not on bit equality
    prm = P.StarParams(dom_lo=-0.02, dom_hi=0.02, r_lo=0.001, r_hi=0.01, n_lo=8, n_hi=120)
    ps = _ulp_chains(P.generate(prm, seed, 60))
    st = Store()
    st.load(0, ps.off, ps.xy)
    st.rasterize(vpr=vpr, strict=False)
    checked = 0
    for k in range(ps.n):
        g = st.fetch_raster(0, k)
        try:
            r = O.Raster(ps.ring(k), vpr, False).arrays()
        except RuntimeError:
            assert g["err"] == -10, k
            continue
        assert g["err"] == 0 and not raster_mismatches(g, r), k
        checked += 1
    st.close()
    assert checked >= ps.n // 2


@pytest.mark.parametrize("scale,vpr", [(1.0, 10), (1.0, 64), (2500.0, 16), (0.01, 4)])
def test_gpu_raster_certified_clip_equals_fp64_clip(gpu_lib, monkeypatch, scale, vpr):
    """The fill clip's points come from certified double-float arithmetic, with
    the reference's FP64 expression only where a float rounding midpoint lies
    within the error bound. FARM_RASTER_EXACT=1 takes the FP64 expression for
    every point: both give the same rasters, bit for bit, at coordinate scales
    from 0.01 to 1e5 (and the oracle agrees with the certified path)."""
    prm = P.StarParams(dom_lo=0.0, dom_hi=30.0 * scale, r_lo=0.05 * scale, r_hi=2.0 * scale, n_hi=4000)
    ps = P.generate(prm, 70 + vpr, 120)
    st_c, got_c = gpu_rasters(ps, vpr, False)
    st_c.close()
    monkeypatch.setenv("FARM_RASTER_EXACT", "1")
    st_e, got_e = gpu_rasters(ps, vpr, False)
    st_e.close()
    for k in range(ps.n):
        assert not raster_mismatches(got_c[k], got_e[k]), k
    for k in range(0, ps.n, 7):
        r = O.Raster(ps.ring(k), vpr, False).arrays()
        assert not raster_mismatches(got_c[k], r), k
