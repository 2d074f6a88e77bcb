"""Polygon sets in the engine's host layout, .dt I/O, generation and the MBR join.

A :class:`PolygonSet` holds rings exactly as a .dt file stores them: polygon k
owns ``xy[off[k]:off[k+1]]`` (float32 pairs, closing copy of the first vertex
included). Reference: storage.cpp:158-193, :320-449.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._native import GenParams, check_host, f32p, f64p, host, ptr, u32p, u64p


@dataclass
class PolygonSet:
    off: np.ndarray  # uint64 [n+1]
    xy: np.ndarray  # float32 [total, 2]

    @property
    def n(self) -> int:
        return len(self.off) - 1

    @property
    def total(self) -> int:
        return int(self.off[-1])

    def ring(self, k: int) -> np.ndarray:
        return self.xy[self.off[k]:self.off[k + 1]]

    def subset(self, idx) -> "PolygonSet":
        idx = np.asarray(idx, dtype=np.int64)
        counts = (self.off[idx + 1] - self.off[idx]).astype(np.uint64)
        off = np.zeros(len(idx) + 1, dtype=np.uint64)
        np.cumsum(counts, out=off[1:])
        xy = np.concatenate([self.xy[self.off[k]:self.off[k + 1]] for k in idx]) if len(idx) else \
            np.zeros((0, 2), np.float32)
        return PolygonSet(off, np.ascontiguousarray(xy, dtype=np.float32))

    def mbrs(self, threads: int = 0) -> np.ndarray:
        out = np.empty((self.n, 4), dtype=np.float64)
        check_host(host().farm_mbr(self.n, ptr(self.off, u64p), ptr(self.xy, f32p), ptr(out, f64p), threads))
        return out

    def write_dt(self, path: str) -> None:
        check_host(host().farm_dt_write(str(path).encode(), self.n, ptr(self.off, u64p), ptr(self.xy, f32p)))


def read_dt(path: str) -> PolygonSet:
    n = C.c_uint64(0)
    tot = C.c_uint64(0)
    lib = host()
    check_host(lib.farm_dt_read(str(path).encode(), C.byref(n), C.byref(tot), None, None))
    off = np.zeros(n.value + 1, dtype=np.uint64)
    xy = np.zeros((tot.value, 2), dtype=np.float32)
    check_host(lib.farm_dt_read(str(path).encode(), C.byref(n), C.byref(tot), ptr(off, u64p), ptr(xy, f32p)))
    return PolygonSet(off, xy)


@dataclass
class StarParams:
    """Seeded star-polygon distribution (the benchmark configurations' generator)."""
    dom_lo: float = 0.0
    dom_hi: float = 100.0
    r_lo: float = 0.05
    r_hi: float = 2.0
    n_lo: int = 16
    n_hi: int = 1024
    sigma: float = 0.3

    def c(self) -> GenParams:
        return GenParams(self.dom_lo, self.dom_hi, self.r_lo, self.r_hi, self.n_lo, self.n_hi, self.sigma)


def generate(params: StarParams, seed: int, count: int, first: int = 0, threads: int = 0) -> PolygonSet:
    gp = params.c()
    counts = np.zeros(count, dtype=np.uint32)
    lib = host()
    check_host(lib.farm_gen_counts(C.byref(gp), seed, first, count, ptr(counts, u32p)))
    off = np.zeros(count + 1, dtype=np.uint64)
    np.cumsum(counts, dtype=np.uint64, out=off[1:])
    xy = np.empty((int(off[-1]), 2), dtype=np.float32)
    check_host(lib.farm_gen_fill(C.byref(gp), seed, first, count, ptr(off, u64p), ptr(xy, f32p), threads))
    return PolygonSet(off, xy)


def centres(params: StarParams, seed: int, count: int, first: int = 0) -> np.ndarray:
    """Centre x, y and mean radius of generator polygons first..first+count-1; float64 [count, 3]."""
    gp = params.c()
    out = np.zeros((count, 3), dtype=np.float64)
    check_host(host().farm_gen_centres(C.byref(gp), seed, first, count, ptr(out, f64p)))
    return out


def radii(params: StarParams, seed: int, count: int, first: int = 0, threads: int = 0) -> np.ndarray:
    """Largest vertex distance from the centre of generator polygons
    first..first+count-1 (float64 [count]), without drawing their vertices."""
    gp = params.c()
    out = np.zeros(count, dtype=np.float64)
    check_host(host().farm_gen_radii(C.byref(gp), seed, first, count, ptr(out, f64p), threads))
    return out


def generate_indices(params: StarParams, seed: int, idx, threads: int = 0, out_off=None, out_xy=None) -> PolygonSet:
    """Generator polygons idx[0], idx[1], ... (any order) as one set. out_off / out_xy
    may supply preallocated (e.g. pinned) arrays of the right sizes."""
    gp = params.c()
    idx = np.ascontiguousarray(idx, dtype=np.uint64)
    lib = host()
    counts = np.zeros(len(idx), dtype=np.uint32)
    check_host(lib.farm_gen_counts_idx(C.byref(gp), seed, ptr(idx, u64p), len(idx), ptr(counts, u32p)))
    off = out_off if out_off is not None else np.zeros(len(idx) + 1, dtype=np.uint64)
    off[0] = 0
    np.cumsum(counts, dtype=np.uint64, out=off[1:])
    xy = out_xy if out_xy is not None else np.empty((int(off[-1]), 2), dtype=np.float32)
    check_host(lib.farm_gen_fill_idx(C.byref(gp), seed, ptr(idx, u64p), len(idx), ptr(off, u64p), ptr(xy, f32p),
                                     threads))
    return PolygonSet(off, xy)


def vertex_counts(params: StarParams, seed: int, idx) -> np.ndarray:
    gp = params.c()
    idx = np.ascontiguousarray(idx, dtype=np.uint64)
    counts = np.zeros(len(idx), dtype=np.uint32)
    check_host(host().farm_gen_counts_idx(C.byref(gp), seed, ptr(idx, u64p), len(idx), ptr(counts, u32p)))
    return counts


def mbr_join(ms: np.ndarray, mt: np.ndarray, expand: float = 0.0, geography: bool = False,
             skip_same: bool = False, threads: int = 0) -> np.ndarray:
    """Candidate pairs (s, t) with overlapping closed MBRs, sorted; uint32 [k, 2]."""
    ms = np.ascontiguousarray(ms, dtype=np.float64)
    mt = np.ascontiguousarray(mt, dtype=np.float64)
    lib = host()
    n = C.c_uint64(0)
    check_host(lib.farm_mbr_join(len(ms), ptr(ms, f64p), len(mt), ptr(mt, f64p), expand, int(geography),
                                 int(skip_same), C.byref(n), None, threads))
    out = np.zeros((n.value, 2), dtype=np.uint32)
    if n.value:
        check_host(lib.farm_mbr_join(len(ms), ptr(ms, f64p), len(mt), ptr(mt, f64p), expand, int(geography),
                                     int(skip_same), C.byref(n), ptr(out, u32p), threads))
    return out


def degree_table() -> np.ndarray:
    out = np.zeros(900, dtype=np.float64)
    host().farm_degree_table(ptr(out, f64p))
    return out
