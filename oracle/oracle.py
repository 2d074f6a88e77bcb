"""ctypes front end of the CPU oracle (oracle/farm_oracle.c).

TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module, and only to verify the engine's results or
as the timed CPU baseline; the engine never routes through it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None


class FoLayer(C.Structure):
    _fields_ = [("mbr", C.c_double * 4), ("dimx", C.c_int32), ("dimy", C.c_int32), ("step_x", C.c_double),
                ("step_y", C.c_double), ("offset", C.c_uint32)]


class FoRaster(C.Structure):
    _fields_ = [("mbr", C.c_double * 4), ("dimx", C.c_int32), ("dimy", C.c_int32), ("step_x", C.c_double),
                ("step_y", C.c_double), ("nv", C.c_uint32), ("status_size", C.c_uint32),
                ("status", C.POINTER(C.c_uint8)), ("P", C.c_uint32), ("offset", C.POINTER(C.c_uint32)),
                ("n_seq", C.c_uint32), ("seq", C.POINTER(C.c_uint32)), ("n_hlines", C.c_uint32),
                ("n_hnodes", C.c_uint32), ("hoff", C.POINTER(C.c_uint32)), ("hnodes", C.POINTER(C.c_double)),
                ("n_vlines", C.c_uint32), ("n_vnodes", C.c_uint32), ("voff", C.POINTER(C.c_uint32)),
                ("vnodes", C.POINTER(C.c_double)), ("areas", C.POINTER(C.c_double)), ("num_layers", C.c_uint32),
                ("layers", C.POINTER(FoLayer))]


class FoOpts(C.Structure):
    _fields_ = [("vpr", C.c_int), ("hierarchy", C.c_int), ("category_count", C.c_int), ("merge_carry", C.c_int),
                ("grid_extent", C.c_double)]


class FoCounters(C.Structure):
    _fields_ = [("window_pixels", C.c_uint64), ("pixel_pairs", C.c_uint64), ("segment_tests", C.c_uint64),
                ("seq_pairs", C.c_uint64)]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            from farm_gb300 import build
            build.build_oracle()
        L = C.CDLL(str(path))
        fp = C.POINTER(C.c_float)
        L.fo_rasterize.argtypes = [fp, C.c_uint32, C.POINTER(FoOpts), C.POINTER(FoRaster)]
        L.fo_raster_free.argtypes = [C.POINTER(FoRaster)]
        L.fo_raster_free.restype = None
        L.fo_intersect.argtypes = [C.POINTER(FoRaster), fp, C.POINTER(FoRaster), fp, C.POINTER(FoCounters)]
        L.fo_intersect_heuristic.argtypes = [C.POINTER(FoRaster), C.POINTER(FoRaster)]
        L.fo_within.argtypes = [C.POINTER(FoRaster), fp, C.POINTER(FoRaster), fp, C.c_double, C.c_int,
                                C.POINTER(FoCounters)]
        L.fo_within_heuristic.argtypes = [C.POINTER(FoRaster), C.POINTER(FoRaster), C.c_double, C.c_int]
        L.fo_segment_intersect.argtypes = [fp, fp, fp, fp]
        L.fo_point_to_segment_distance.argtypes = [fp, fp, fp, C.c_int]
        L.fo_point_to_segment_distance.restype = C.c_double
        L.fo_segment_contain.argtypes = [C.POINTER(FoRaster), fp, C.c_float, C.c_float]
        L.fo_contain_point.argtypes = [C.POINTER(FoRaster), fp, C.c_float, C.c_float]
        L.fo_contain.argtypes = [C.POINTER(FoRaster), fp, C.POINTER(FoRaster), fp, C.POINTER(FoCounters)]
        L.fo_intersection_area.argtypes = [fp, C.c_uint32, fp, C.c_uint32]
        L.fo_intersection_area.restype = C.c_double
        L.fo_intersection_area_plain.argtypes = [fp, C.c_uint32, fp, C.c_uint32]
        L.fo_intersection_area_plain.restype = C.c_double
        L.fo_degree_per_km_longitude.argtypes = [C.c_double]
        L.fo_degree_per_km_longitude.restype = C.c_double
        _lib = L
    return _lib


def mem_ring(stored: np.ndarray) -> np.ndarray:
    """The ring the reference decodes from a stored record: stored vertices, one
    more copy of the first (vertex_sequence.cpp:206-219), and the pad vertex the
    single-pixel sequence reads (a copy of the first)."""
    s = np.ascontiguousarray(stored, dtype=np.float32)
    return np.ascontiguousarray(np.concatenate([s, s[:1], s[:1]]), dtype=np.float32)


class Raster:
    """One rasterized polygon (owns the C allocation)."""

    def __init__(self, stored: np.ndarray, vpr: int, hierarchy: bool = False, category_count: int = 16,
                 merge_carry: int = 1, grid_extent: float = 0.0):
        self.ring = mem_ring(stored)
        self.nv = len(stored) + 1
        self.r = FoRaster()
        o = FoOpts(vpr, int(hierarchy), category_count, merge_carry, float(grid_extent))
        rc = lib().fo_rasterize(self.ring.ctypes.data_as(C.POINTER(C.c_float)), self.nv, C.byref(o), C.byref(self.r))
        self.rc = rc
        if rc != 0:
            raise RuntimeError(f"oracle rasterize failed: {rc}")

    def __del__(self):
        try:
            lib().fo_raster_free(C.byref(self.r))
        except Exception:
            pass

    def arrays(self) -> dict:
        r = self.r

        def arr(p, n, dt):
            if n == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)

        out = {
            "mbr": np.array(r.mbr[:], dtype=np.float64), "dimx": r.dimx, "dimy": r.dimy,
            "step": np.array([r.step_x, r.step_y]), "status": arr(r.status, r.status_size, np.uint8),
            "offset": arr(r.offset, r.P + 1, np.uint32), "seq": arr(r.seq, 2 * r.n_seq, np.uint32).reshape(-1, 2),
            "hoff": arr(r.hoff, r.n_hlines, np.uint32), "hnodes": arr(r.hnodes, r.n_hnodes, np.float64),
            "voff": arr(r.voff, r.n_vlines, np.uint32), "vnodes": arr(r.vnodes, r.n_vnodes, np.float64),
            "areas": arr(r.areas, r.P, np.float64), "num_layers": r.num_layers,
        }
        layers = []
        for i in range(r.num_layers):
            L = r.layers[i]
            layers.append((tuple(L.mbr[:]), L.dimx, L.dimy, L.step_x, L.step_y, L.offset))
        out["layers"] = layers
        return out


def rasterize_set(ps, vpr: int, hierarchy: bool = False, category_count: int = 16, merge_carry: int = 1,
                  grid_extent: float = 0.0):
    return [Raster(ps.ring(k), vpr, hierarchy, category_count, merge_carry, grid_extent) for k in range(ps.n)]


def _try_raster(args):
    ring, vpr, hierarchy, category_count = args
    try:
        return Raster(ring, vpr, hierarchy, category_count)
    except RuntimeError:  # the reference asserts or never terminates on this polygon
        return None


def rasterize_many(rings, vpr: int, hierarchy: bool = False, category_count: int = 16, threads: int = 0) -> list:
    """Raster objects of many rings (None where the reference fails on one),
    built on a thread pool: ctypes releases the GIL while the C code runs, so
    the threads use every core. Largest rings are started first."""
    import concurrent.futures as cf
    import os
    lib()
    rings = list(rings)
    order = sorted(range(len(rings)), key=lambda k: -len(rings[k]))
    out = [None] * len(rings)
    with cf.ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        futs = {ex.submit(_try_raster, (rings[k], vpr, hierarchy, category_count)): k for k in order}
        for f in cf.as_completed(futs):
            out[futs[f]] = f.result()
    return out


def intersect_many(rs: list, rt: list, pairs, threads: int = 0, counters: bool = False):
    """Oracle intersect of (s, t) pairs over prebuilt rasters, on a thread
    pool: 0/1 per pair, 2 where either raster is None; with counters, also the
    reference-order segment tests per pair (uint64)."""
    import concurrent.futures as cf
    import os
    pairs = np.asarray(pairs)
    n = len(pairs)
    res = np.zeros(n, np.uint8)
    tests = np.zeros(n, np.uint64)
    nt = threads or os.cpu_count() or 1
    bounds = np.linspace(0, n, min(n, 4 * nt) + 1).astype(np.int64) if n else np.zeros(1, np.int64)

    def run(lo_hi):
        lo, hi = lo_hi
        for k in range(lo, hi):
            a, b = rs[int(pairs[k, 0])], rt[int(pairs[k, 1])]
            if a is None or b is None:
                res[k] = 2
                continue
            v, c = intersect(a, b, counters=True)
            res[k] = int(v)
            tests[k] = c.segment_tests
    with cf.ThreadPoolExecutor(max_workers=nt) as ex:
        list(ex.map(run, zip(bounds[:-1], bounds[1:])))
    return (res, tests) if counters else res


def intersect(rs: Raster, rt: Raster, counters: bool = False):
    c = FoCounters()
    fp = C.POINTER(C.c_float)
    v = lib().fo_intersect(C.byref(rs.r), rs.ring.ctypes.data_as(fp), C.byref(rt.r), rt.ring.ctypes.data_as(fp),
                           C.byref(c))
    if v < 0:
        raise RuntimeError(f"oracle intersect failed: {v}")
    return (bool(v), c) if counters else bool(v)


def contain(rs: Raster, rt: Raster, counters: bool = False):
    """Ideal::contain(Ideal *): does polygon rs hold polygon rt."""
    c = FoCounters()
    fp = C.POINTER(C.c_float)
    v = lib().fo_contain(C.byref(rs.r), rs.ring.ctypes.data_as(fp), C.byref(rt.r), rt.ring.ctypes.data_as(fp),
                         C.byref(c))
    return (bool(v), c) if counters else bool(v)


def contain_point(rs: Raster, x: float, y: float) -> bool:
    """Ideal::contain(Point &): does polygon rs hold the float32 point (x, y)."""
    fp = C.POINTER(C.c_float)
    return bool(lib().fo_contain_point(C.byref(rs.r), rs.ring.ctypes.data_as(fp), float(np.float32(x)),
                                       float(np.float32(y))))


def contain_many(rs: list, rt: list, pairs, threads: int = 0) -> np.ndarray:
    """Oracle polygon containment of (s, t) pairs on a thread pool: 0/1, 2 where
    either raster is None."""
    return _pairwise(lambda a, b: contain(a, b), rs, rt, pairs, threads)


def contain_points_many(rs: list, pts, pairs, threads: int = 0) -> np.ndarray:
    """Oracle point containment of (polygon, point) pairs: 0/1, 2 where the
    polygon's raster is None."""
    pts = np.asarray(pts, dtype=np.float32)
    return _pairwise(lambda a, k: contain_point(a, pts[k, 0], pts[k, 1]), rs, range(len(pts)), pairs, threads)


def _pairwise(fn, ra, rb, pairs, threads):
    import concurrent.futures as cf
    import os
    pairs = np.asarray(pairs)
    n = len(pairs)
    res = np.zeros(n, np.uint8)
    nt = threads or os.cpu_count() or 1
    bounds = np.linspace(0, n, min(n, 4 * nt) + 1).astype(np.int64) if n else np.zeros(1, np.int64)

    def run(lo_hi):
        for k in range(*lo_hi):
            a, b = ra[int(pairs[k, 0])], rb[int(pairs[k, 1])]
            res[k] = 2 if a is None or b is None else int(fn(a, b))
    with cf.ThreadPoolExecutor(max_workers=nt) as ex:
        list(ex.map(run, zip(bounds[:-1], bounds[1:])))
    return res


def read_points(path: str) -> np.ndarray:
    """A points file of the contain-point fixtures: uint64 n, then n float32 (x, y)."""
    buf = open(path, "rb").read()
    n = int(np.frombuffer(buf, dtype=np.uint64, count=1)[0])
    return np.frombuffer(buf, dtype=np.float32, count=2 * n, offset=8).reshape(n, 2).copy()


def intersect_heuristic(rs: Raster, rt: Raster) -> bool:
    """The reference's -a approximate intersect (fill-probability heuristic)."""
    return bool(lib().fo_intersect_heuristic(C.byref(rs.r), C.byref(rt.r)))


def within(rs: Raster, rt: Raster, distance: float = 10.0, geography: bool = True, counters: bool = False):
    c = FoCounters()
    fp = C.POINTER(C.c_float)
    v = lib().fo_within(C.byref(rs.r), rs.ring.ctypes.data_as(fp), C.byref(rt.r), rt.ring.ctypes.data_as(fp),
                        float(distance), int(geography), C.byref(c))
    if v < 0:
        raise RuntimeError(f"oracle within failed: {v}")
    return (bool(v), c) if counters else bool(v)


def within_heuristic(rs: Raster, rt: Raster, distance: float = 10.0, geography: bool = True) -> bool:
    """The reference's within -a rule on the hierarchical descent (no refinement)."""
    v = lib().fo_within_heuristic(C.byref(rs.r), C.byref(rt.r), float(distance), int(geography))
    if v < 0:
        raise RuntimeError(f"oracle within heuristic failed: {v}")
    return bool(v)


def intersection_area(a: np.ndarray, b: np.ndarray, plain: bool = False) -> float:
    """FP64 area of ring a intersected with ring b (plain: the definition by
    loops over every edge pair, for checking the indexed version)."""
    fp = C.POINTER(C.c_float)
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    f = lib().fo_intersection_area_plain if plain else lib().fo_intersection_area
    return f(a.ctypes.data_as(fp), len(a), b.ctypes.data_as(fp), len(b))


def read_ref_rasters(path: str) -> list[dict]:
    """Parse a raster dump written by oracle/ref/harness.cpp."""
    buf = open(path, "rb").read()
    pos = 0

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(buf, dtype=dt, count=n, offset=pos)
        pos += a.nbytes
        return a.copy()

    magic, n = take(np.uint32, 2)
    assert magic == 0x46415231
    out = []
    for _ in range(int(n)):
        mbr = take(np.float64, 4)
        dimx, dimy = take(np.int32, 2)
        step = take(np.float64, 2)
        nv = int(take(np.uint32, 1)[0])
        ss = int(take(np.uint32, 1)[0])
        status = take(np.uint8, ss)
        P = int(take(np.uint32, 1)[0])
        offset = take(np.uint32, P + 1)
        les = int(take(np.uint32, 1)[0])
        seq = take(np.uint32, 2 * les).reshape(-1, 2)
        nl = int(take(np.uint32, 1)[0])
        hoff = take(np.uint32, nl)
        nc = int(take(np.uint32, 1)[0])
        hnodes = take(np.float64, nc)
        nl = int(take(np.uint32, 1)[0])
        voff = take(np.uint32, nl)
        nc = int(take(np.uint32, 1)[0])
        vnodes = take(np.float64, nc)
        areas = take(np.float64, P)
        L = int(take(np.uint32, 1)[0])
        layers = []
        for _ in range(L):
            lm = take(np.float64, 4)
            ldx, ldy = take(np.int32, 2)
            lst = take(np.float64, 2)
            lo = int(take(np.uint32, 1)[0])
            layers.append((tuple(lm), int(ldx), int(ldy), float(lst[0]), float(lst[1]), lo))
        out.append({"mbr": mbr, "dimx": int(dimx), "dimy": int(dimy), "step": step, "nv": nv, "status": status,
                    "offset": offset, "seq": seq, "hoff": hoff, "hnodes": hnodes, "voff": voff, "vnodes": vnodes,
                    "areas": areas, "num_layers": L, "layers": layers})
    return out


def read_ref_pairs(path: str) -> np.ndarray:
    """Parse a pair-decision file written by oracle/ref/harness.cpp: [k, 3] (s, t, result)."""
    buf = open(path, "rb").read()
    n = int(np.frombuffer(buf, dtype=np.uint64, count=1)[0])
    rec = np.dtype([("s", "<u4"), ("t", "<u4"), ("r", "u1")])
    a = np.frombuffer(buf, dtype=rec, count=n, offset=8)
    return np.stack([a["s"].astype(np.int64), a["t"].astype(np.int64), a["r"].astype(np.int64)], axis=1)
