"""Host-side mirror of the reference's query interface for the polygon-join path.

The reference's GPU entry points take a ``query_context`` (src/include/Ideal.h:205-213);
here a :class:`Store` owns the device-resident polygons and rasters and each
query mirrors one of them:

==========================  ==================================================
reference                   here
==========================  ==================================================
preprocess + rasterization  ``Store.load(...)`` + ``Store.rasterize(vpr, ...)``
``Ideal::intersect``         ``Store.intersect(pairs)``
``Ideal::within``            ``Store.within(pairs, distance)``
``Ideal::intersection``      ``Store.intersection_area(pairs)``
==========================  ==================================================

Every call goes through the C ABI of ``libfarm_gpu.so`` (include/farm_gpu.h);
there is no CPU path behind it. Pair arrays are ``uint32 [n, 2]`` of
(source index, target index). Arrays may be numpy (host) or torch CUDA tensors
(device-resident; no copy).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from ._gpu_sig import RasterOpts, RasterTotals, RasterView, Stats
from ._native import check_gpu, gpu

MODE_EXACT = 0
MODE_APPROX = 1
MODE_LEARNED = 2
MODE_FILTER = 3
MEM_HOST = 0
MEM_DEVICE = 1


def _addr(a):
    """(pointer, mem) of a numpy array or a CUDA tensor."""
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return C.c_void_p(a.ctypes.data), MEM_HOST
    if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return C.c_void_p(a.data_ptr()), MEM_DEVICE
    raise TypeError(f"unsupported array type {type(a)!r}")


def stats_dict(st: Stats) -> dict:
    return {"pairs": st.pairs, "found": st.found, "in_hits": st.in_hits, "border_pairs": st.border_pairs,
            "segment_tests": st.segment_tests, "fp64_rechecks": st.fp64_rechecks, "ms_total": st.ms_total,
            "ms_stage": list(st.ms_stage), "kernel_launches": st.kernel_launches,
            "src_window_pixels": st.src_window_pixels, "tgt_window_pixels": st.tgt_window_pixels,
            "sequence_pairs": st.sequence_pairs}


class Store:
    """Device-resident source/target polygon tables with their rasters."""

    def __init__(self):
        self._lib = gpu()
        self._h = C.c_void_p()
        check_gpu(self._lib.farm_store_create(C.byref(self._h)))
        self.n_source = 0
        self.n_target = 0
        self.last_stats: dict = {}

    def close(self):
        if self._h:
            self._lib.farm_store_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def load(self, side: int, off, xy) -> None:
        """Load rings (host layout, closing vertex included) for side 0 (source) or 1 (target)."""
        po, mo = _addr(off)
        px, mx = _addr(xy)
        if mo != mx:
            raise ValueError("offsets and vertices must live in the same memory")
        n = (off.shape[0] if hasattr(off, "shape") else len(off)) - 1
        check_gpu(self._lib.farm_store_load(self._h, side, n, po, px, mo))
        if side == 0:
            self.n_source, self.n_target = n, 0
        else:
            self.n_target = n

    def load_dt(self, side: int, path: str, threads: int = 0) -> int:
        """Stream a .dt file into one side (farm_store_load_dt); the polygons kept."""
        n = C.c_uint64(0)
        check_gpu(self._lib.farm_store_load_dt(self._h, int(side), str(path).encode(), int(threads), C.byref(n)))
        return n.value

    def load_sets(self, source, target=None) -> None:
        self.load(0, source.off, source.xy)
        if target is not None:
            self.load(1, target.off, target.xy)

    def rasterize(self, vpr: int = 10, category_count: int = 16, hierarchy: bool = False,
                  strict: bool = True, grid_extent: float = 0.0) -> int:
        """Rasterize every loaded polygon. With strict=False, polygons on which
        the reference asserts or never terminates (FARM_EASSERT) are reported
        by count instead of raising; queries then return 2 for their pairs."""
        o = RasterOpts(vpr, category_count, int(hierarchy), 0, float(grid_extent))
        rc = self._lib.farm_rasterize(self._h, C.byref(o))
        if rc == -10 and not strict:
            return int((self.raster_errors(0) != 0).sum() + (self.raster_errors(1) != 0).sum())
        check_gpu(rc)
        return 0

    def mbr_join(self, expand: float = 0.0, geography: bool = False, self_join: bool = False, device=None,
                 cap: int = 0):
        """Candidate pairs of the loaded sides computed on the GPU (uint32
        [k, 2], ascending (source, target)): a CUDA tensor when `device` is
        given, else numpy. `cap` bounds the pairs (0: counted first)."""
        lib = self._lib
        n = C.c_uint64(0)
        if cap <= 0:
            rc = lib.farm_mbr_join_gpu(self._h, float(expand), int(geography), int(self_join), None, 0, MEM_HOST,
                                       C.byref(n))
            if rc not in (0, -4):
                check_gpu(rc)
            cap = int(n.value)
        if device is not None:
            import torch
            out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device=device)
            check_gpu(lib.farm_mbr_join_gpu(self._h, float(expand), int(geography), int(self_join),
                                             C.c_void_p(out.data_ptr()), cap, MEM_DEVICE, C.byref(n)))
            return out[:n.value]
        out = np.zeros((max(cap, 1), 2), dtype=np.uint32)
        check_gpu(lib.farm_mbr_join_gpu(self._h, float(expand), int(geography), int(self_join),
                                         C.c_void_p(out.ctypes.data), cap, MEM_HOST, C.byref(n)))
        return out[:n.value]

    def intersect(self, pairs, mode: int = MODE_EXACT, out=None):
        """Per-pair 0/1 results (same memory kind as ``pairs``) and the found count."""
        n = pairs.shape[0]
        pp, mem = _addr(pairs)
        if out is None:
            out = np.zeros(n, dtype=np.uint8) if mem == MEM_HOST else _torch_empty_u8(n, pairs.device)
        po, mo = _addr(out)
        if mo != mem:
            raise ValueError("pairs and out must live in the same memory")
        found = C.c_uint64(0)
        st = Stats()
        check_gpu(self._lib.farm_intersect(self._h, pp, n, mode, mem, po, C.byref(found), C.byref(st)))
        self.last_stats = stats_dict(st)
        return out, found.value

    def within(self, pairs, distance: float = 10.0, geography: bool = True, self_join: bool = False, out=None,
               mode: int = MODE_EXACT):
        """Ideal::within per pair; mode MODE_APPROX is the reference's within -a rule."""
        n = pairs.shape[0]
        pp, mem = _addr(pairs)
        if out is None:
            out = np.zeros(n, dtype=np.uint8) if mem == MEM_HOST else _torch_empty_u8(n, pairs.device)
        po, mo = _addr(out)
        found = C.c_uint64(0)
        st = Stats()
        check_gpu(self._lib.farm_within_mode(self._h, pp, n, float(distance), int(geography), int(self_join),
                                             int(mode), mem, po, C.byref(found), C.byref(st)))
        self.last_stats = stats_dict(st)
        return out, found.value

    def contain(self, pairs, out=None):
        """Ideal::contain(Ideal *) per (source, target) pair: does the source hold the target."""
        n = pairs.shape[0]
        pp, mem = _addr(pairs)
        if out is None:
            out = np.zeros(n, dtype=np.uint8) if mem == MEM_HOST else _torch_empty_u8(n, pairs.device)
        po, mo = _addr(out)
        if mo != mem:
            raise ValueError("pairs and out must live in the same memory")
        found = C.c_uint64(0)
        st = Stats()
        check_gpu(self._lib.farm_contain(self._h, pp, n, mem, po, C.byref(found), C.byref(st)))
        self.last_stats = stats_dict(st)
        return out, found.value

    def contain_points(self, points, pairs, side: int = 0, out=None):
        """Ideal::contain(Point &) per (polygon, point) pair; points is an
        [m, 2] float32 array in the same memory as pairs."""
        if isinstance(points, np.ndarray) and points.dtype != np.float32:
            raise TypeError("points must be float32")
        n = pairs.shape[0]
        pp, mem = _addr(pairs)
        xp, mx = _addr(points)
        if mx != mem:
            raise ValueError("points and pairs must live in the same memory")
        if out is None:
            out = np.zeros(n, dtype=np.uint8) if mem == MEM_HOST else _torch_empty_u8(n, pairs.device)
        po, _ = _addr(out)
        found = C.c_uint64(0)
        check_gpu(self._lib.farm_contain_points(self._h, int(side), xp, points.shape[0], pp, n, mem, po,
                                                C.byref(found)))
        return out, found.value

    def intersection_area(self, pairs, out=None):
        n = pairs.shape[0]
        pp, mem = _addr(pairs)
        if out is None:
            out = np.zeros(n, dtype=np.float64) if mem == MEM_HOST else _torch_empty_f64(n, pairs.device)
        po, _ = _addr(out)
        st = Stats()
        check_gpu(self._lib.farm_intersection_area(self._h, pp, n, mem, po, C.byref(st)))
        self.last_stats = stats_dict(st)
        return out

    # ---- batched area (captured CUDA graph, autotuned chunks) ------------
    def area_plan(self, max_pairs: int, max_items: int) -> "AreaPlan":
        h = C.c_void_p()
        check_gpu(self._lib.farm_area_plan_create(self._h, max_pairs, max_items, C.byref(h)))
        return AreaPlan(self, h)

    def area_autotune(self, pairs, with_wide: bool = False):
        """Tune the area knobs per size bucket on a sample of pairs; returns the
        chunk table, or (chunk table, window table) with with_wide."""
        pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
        tab = np.zeros(32, np.int32)
        wide = np.zeros(32, np.int32)
        check_gpu(self._lib.farm_area_autotune(self._h, C.c_void_p(pairs.ctypes.data), pairs.shape[0], MEM_HOST,
                                               C.c_void_p(tab.ctypes.data), C.c_void_p(wide.ctypes.data)))
        return (tab, wide) if with_wide else tab

    def area_set_wide(self, table) -> None:
        tab = np.ascontiguousarray(table, dtype=np.int32)
        assert tab.size == 32
        check_gpu(self._lib.farm_area_set_wide(self._h, C.c_void_p(tab.ctypes.data)))

    def area_set_chunks(self, table) -> None:
        tab = np.ascontiguousarray(table, dtype=np.int32)
        assert tab.size == 32
        check_gpu(self._lib.farm_area_set_chunks(self._h, C.c_void_p(tab.ctypes.data)))

    # ---- learned scorer (device tensors: torch CUDA) -------------------
    def mlp_init(self, seed: int = 1) -> None:
        check_gpu(self._lib.farm_mlp_init(self._h, seed))

    def mlp_params(self) -> np.ndarray:
        out = np.zeros(int(self._lib.farm_mlp_param_count()), np.float32)
        check_gpu(self._lib.farm_mlp_get(self._h, C.c_void_p(out.ctypes.data)))
        return out

    def mlp_load(self, params: np.ndarray) -> None:
        params = np.ascontiguousarray(params, dtype=np.float32)
        assert params.size == int(self._lib.farm_mlp_param_count())
        check_gpu(self._lib.farm_mlp_set(self._h, C.c_void_p(params.ctypes.data)))

    def mlp_band(self, lo: float, hi: float, cost_lambda: float = 0.0) -> None:
        check_gpu(self._lib.farm_mlp_set_band(self._h, lo, hi))
        check_gpu(self._lib.farm_mlp_set_band_cost(self._h, cost_lambda))

    def filter_costs(self, d_pairs):
        """The exact filter alone on device pairs: (codes 0/1/3, refinement cost
        proxies) as device tensors."""
        import torch
        n = d_pairs.shape[0]
        code = torch.empty(n, dtype=torch.uint8, device=d_pairs.device)
        cost = torch.empty(n, dtype=torch.float32, device=d_pairs.device)
        check_gpu(self._lib.farm_intersect_filter(self._h, C.c_void_p(d_pairs.data_ptr()), n,
                                                  C.c_void_p(code.data_ptr()), C.c_void_p(cost.data_ptr())))
        return code, cost

    def mlp_features(self, d_pairs, rows: int = 0):
        import torch
        n = d_pairs.shape[0]
        rows = max(rows, (n + 127) // 128 * 128)
        X = torch.empty((rows, 576), dtype=torch.bfloat16, device=d_pairs.device)
        check_gpu(self._lib.farm_mlp_features(self._h, C.c_void_p(d_pairs.data_ptr()), n, C.c_void_p(X.data_ptr()),
                                              rows))
        return X

    def mlp_grad(self, X, y, n: int):
        loss = C.c_float(0)
        g = np.zeros(int(self._lib.farm_mlp_param_count()), np.float32)
        check_gpu(self._lib.farm_mlp_grad(self._h, C.c_void_p(X.data_ptr()), C.c_void_p(y.data_ptr()), n,
                                          X.shape[0], C.byref(loss), C.c_void_p(g.ctypes.data)))
        return loss.value, g

    def mlp_train(self, d_pairs, d_labels, epochs: int = 4, batch: int = 4096, lr: float = 2e-3,
                  seed: int = 1) -> float:
        loss = C.c_float(0)
        check_gpu(self._lib.farm_mlp_train(self._h, C.c_void_p(d_pairs.data_ptr()), C.c_void_p(d_labels.data_ptr()),
                                           d_pairs.shape[0], epochs, batch, lr, seed, C.byref(loss)))
        return loss.value

    def mlp_predict(self, d_pairs):
        import torch
        p = torch.empty(d_pairs.shape[0], dtype=torch.float32, device=d_pairs.device)
        check_gpu(self._lib.farm_mlp_predict(self._h, C.c_void_p(d_pairs.data_ptr()), d_pairs.shape[0],
                                             C.c_void_p(p.data_ptr())))
        return p

    @property
    def launches(self) -> int:
        """Engine kernels launched through this store so far."""
        return int(self._lib.farm_store_launches(self._h))

    def device_bytes(self) -> int:
        """Device bytes held by the store's own allocations."""
        b = C.c_uint64(0)
        check_gpu(self._lib.farm_store_device_bytes(self._h, C.byref(b)))
        return int(b.value)

    def raster_totals(self) -> dict:
        """Sizes of the last rasterization (units processed, arrays written)."""
        t = RasterTotals()
        check_gpu(self._lib.farm_raster_get_totals(self._h, C.byref(t)))
        return {k: (float(getattr(t, k)) if k.startswith("ms_") else int(getattr(t, k))) for k, _ in RasterTotals._fields_}

    def event_record(self, slot: int) -> None:
        check_gpu(self._lib.farm_event_record(self._h, slot))

    def event_elapsed(self, a: int, b: int) -> float:
        ms = C.c_double(0)
        check_gpu(self._lib.farm_event_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def raster_errors(self, side: int) -> np.ndarray:
        """Per-polygon rasterization status (0 or FARM_EASSERT) of one side."""
        n = self.n_source if side == 0 else self.n_target
        out = np.zeros(n, np.int32)
        check_gpu(self._lib.farm_raster_errors(self._h, side, C.c_void_p(out.ctypes.data), n))
        return out

    def sync(self) -> None:
        check_gpu(self._lib.farm_sync(self._h))

    def fetch_raster(self, side: int, index: int) -> dict:
        """One polygon's raster arrays (for parity tests)."""
        v = RasterView()
        lib = self._lib
        check_gpu(lib.farm_raster_fetch(self._h, side, index, C.byref(v), None, None, None, None, None, None, None,
                                        None, None))
        P = v.dimx * v.dimy
        status = np.zeros(v.status_size, np.uint8)
        offset = np.zeros(P + 1, np.uint32)
        seq = np.zeros((v.n_seq, 2), np.uint32)
        hoff = np.zeros(v.dimy + 2, np.uint32)
        hnodes = np.zeros(v.n_hnodes, np.float64)
        voff = np.zeros(v.dimx + 2, np.uint32)
        vnodes = np.zeros(v.n_vnodes, np.float64)
        areas = np.zeros(P, np.float64)
        layers = np.zeros((max(v.num_layers, 1), 7), np.float64)

        def p(a, t):
            return a.ctypes.data_as(C.POINTER(t))

        check_gpu(lib.farm_raster_fetch(self._h, side, index, C.byref(v), p(status, C.c_uint8),
                                        p(offset, C.c_uint32), p(seq, C.c_uint32), p(hoff, C.c_uint32),
                                        p(hnodes, C.c_double), p(voff, C.c_uint32), p(vnodes, C.c_double),
                                        p(areas, C.c_double), p(layers, C.c_double)))
        out_layers = []
        for i in range(v.num_layers):
            L = layers[i]
            packed = int(L[6])
            out_layers.append((tuple(L[:4]), packed >> 32, packed & 0xFFFFFFFF, float(L[4]), float(L[5])))
        return {"mbr": np.array(v.mbr[:]), "dimx": v.dimx, "dimy": v.dimy, "step": np.array([v.step_x, v.step_y]),
                "nv": v.nv, "status": status, "offset": offset, "seq": seq, "hoff": hoff, "hnodes": hnodes,
                "voff": voff, "vnodes": vnodes, "areas": areas, "num_layers": v.num_layers, "layers": out_layers,
                "err": v.err}


def _torch_empty_u8(n, device):
    import torch
    return torch.empty(n, dtype=torch.uint8, device=device)


def _torch_empty_f64(n, device):
    import torch
    return torch.empty(n, dtype=torch.float64, device=device)


def issue_rates() -> dict:
    """Measured non-fused FP64 and FP32 operation rates of the current device (ops/s)."""
    a, b = C.c_double(0), C.c_double(0)
    check_gpu(gpu().farm_probe_issue_rates(C.byref(a), C.byref(b)))
    return {"fp64_ops_per_s": a.value, "fp32_ops_per_s": b.value}


def device_name() -> str:
    buf = C.create_string_buffer(256)
    ordn = C.c_int(0)
    check_gpu(gpu().farm_device_info(C.byref(ordn), buf, 256))
    return buf.value.decode()


class AreaPlan:
    """A captured area pass (farm_area_plan): run() replays it on a batch."""

    def __init__(self, store: Store, handle):
        self._store, self._h = store, handle
        self.last_stats = {}

    def run(self, pairs, out=None):
        n = pairs.shape[0]
        pp, mem = _addr(pairs)
        if out is None:
            out = np.zeros(n, dtype=np.float64) if mem == MEM_HOST else _torch_empty_f64(n, pairs.device)
        po, _ = _addr(out)
        st = Stats()
        check_gpu(self._store._lib.farm_area_plan_run(self._h, pp, n, mem, po, C.byref(st)))
        self.last_stats = stats_dict(st)
        return out

    def close(self):
        if self._h:
            self._store._lib.farm_area_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

