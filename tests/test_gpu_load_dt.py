"""farm_store_load_dt: .dt files streamed into the store through pinned staging
buffers must give the store exactly what farm_store_load gives for the same
rings (the reference's loader rules: holes dropped, rings under 3 in-memory
vertices skipped)."""
import struct
import time

import numpy as np
import pytest

from farm_gb300 import polygons as P
from farm_gb300.engine import Store

pytestmark = pytest.mark.gpu


def write_dt_with_holes(path, rings, holes_of, tiny):
    """A .dt file in the storage.cpp layout with holes on some records and
    degenerate (one stored vertex) records at the indices in `tiny`."""
    meta, data, cur = [], bytearray(), 0
    for k, r in enumerate(rings):
        r = np.ascontiguousarray(r, np.float32)
        if k in tiny:
            r = r[:1]
        hs = holes_of.get(k, [])
        rec = struct.pack("<QQ", len(hs), len(r)) + r.tobytes()
        for h in hs:
            h = np.ascontiguousarray(h, np.float32)
            rec += struct.pack("<Q", len(h)) + h.tobytes()
        lo, hi = r.min(0).astype(np.float64), r.max(0).astype(np.float64)
        meta.append(struct.pack("<IIQ4d", len(rec), len(r) + 1, cur, lo[0], lo[1], hi[0], hi[1]))
        data += rec
        cur += len(rec)
    with open(path, "wb") as f:
        f.write(bytes(data))
        f.write(b"".join(meta))
        f.write(struct.pack("<Q", len(rings)))


def test_load_dt_matches_array_load(gpu_lib, tmp_path):
    prm = P.StarParams(dom_hi=30.0, n_lo=16, n_hi=20000)
    S, T = P.generate(prm, 71, 300), P.generate(prm, 72, 900)
    sdt, tdt = tmp_path / "S.dt", tmp_path / "T.dt"
    S.write_dt(str(sdt))
    T.write_dt(str(tdt))
    pairs = np.ascontiguousarray(P.mbr_join(S.mbrs(), T.mbrs()), dtype=np.uint32)
    with Store() as a, Store() as b:
        assert a.load_dt(0, sdt, threads=4) == S.n
        assert a.load_dt(1, tdt) == T.n
        b.load_sets(S, T)
        a.rasterize(vpr=64, strict=False)
        b.rasterize(vpr=64, strict=False)
        for k in (0, 7, S.n - 1):
            ra, rb = a.fetch_raster(0, k), b.fetch_raster(0, k)
            for key in ("status", "offset", "seq", "vnodes", "areas"):
                assert np.array_equal(ra[key], rb[key]), (k, key)
        oa, fa = a.intersect(pairs)
        ob, fb = b.intersect(pairs)
    assert np.array_equal(oa, ob) and fa == fb


def test_load_dt_drops_holes_and_degenerate_rings(gpu_lib, tmp_path):
    prm = P.StarParams(dom_hi=10.0, n_hi=300)
    S = P.generate(prm, 73, 40)
    rings = [S.ring(k) for k in range(S.n)]
    holes = {3: [rings[5][:6]], 9: [rings[1][:4], rings[2][:5]]}
    path = tmp_path / "h.dt"
    write_dt_with_holes(path, rings, holes, tiny={4, 20})
    ps = P.read_dt(str(path))  # the host reader applies the same rules
    assert ps.n == S.n - 2
    with Store() as a, Store() as b:
        assert a.load_dt(0, path) == ps.n
        b.load(0, ps.off, ps.xy)
        a.rasterize(vpr=10)
        b.rasterize(vpr=10)
        for k in range(ps.n):
            ra, rb = a.fetch_raster(0, k), b.fetch_raster(0, k)
            assert ra["nv"] == rb["nv"] and np.array_equal(ra["status"], rb["status"]), k


def test_load_dt_rejects_malformed_files(gpu_lib, tmp_path):
    from farm_gb300._native import FarmError
    bad = tmp_path / "bad.dt"
    bad.write_bytes(struct.pack("<Q", 5))
    with Store() as st:
        with pytest.raises(FarmError):
            st.load_dt(0, bad)
        with pytest.raises(FarmError):
            st.load_dt(0, tmp_path / "missing.dt")
    # a record whose vertex count runs past the data
    prm = P.StarParams(dom_hi=10.0, n_hi=100)
    S = P.generate(prm, 74, 5)
    path = tmp_path / "cut.dt"
    S.write_dt(str(path))
    raw = bytearray(path.read_bytes())
    raw[8:16] = struct.pack("<Q", 1 << 40)
    path.write_bytes(bytes(raw))
    with Store() as st:
        with pytest.raises(FarmError, match="malformed"):
            st.load_dt(0, path)


def test_load_dt_streams_a_large_file(gpu_lib, tmp_path):
    """About 0.8 GB of rings: streamed in several staging chunks; prints the
    load rate against the array path (page-cache reads)."""
    prm = P.StarParams(dom_hi=200.0, n_lo=1000, n_hi=100000)
    S = P.generate(prm, 75, 3000)
    path = tmp_path / "big.dt"
    S.write_dt(str(path))
    with Store() as a, Store() as b:
        a.load_dt(0, path)  # warm: staging buffers and page cache
        t0 = time.perf_counter()
        n = a.load_dt(0, path)
        t_dt = time.perf_counter() - t0
        t0 = time.perf_counter()
        ps = P.read_dt(str(path))
        b.load(0, ps.off, ps.xy)
        t_arr = time.perf_counter() - t0
        assert n == S.n
        a.rasterize(vpr=64, strict=False)
        b.rasterize(vpr=64, strict=False)
        for k in (0, S.n // 2, S.n - 1):
            assert np.array_equal(a.fetch_raster(0, k)["status"], b.fetch_raster(0, k)["status"])
    gb = path.stat().st_size / 1e9
    print(f"\n.dt {gb:.2f} GB: streamed {gb / t_dt:.1f} GB/s; read + array load {gb / t_arr:.1f} GB/s")
