"""ctypes signatures of include/farm_gpu.h."""
import ctypes as C


class RasterOpts(C.Structure):
    _fields_ = [("vpr", C.c_int32), ("category_count", C.c_int32), ("hierarchy", C.c_int32),
                ("reserved", C.c_int32), ("grid_extent", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("pairs", C.c_uint64), ("found", C.c_uint64), ("in_hits", C.c_uint64),
                ("border_pairs", C.c_uint64), ("segment_tests", C.c_uint64), ("fp64_rechecks", C.c_uint64),
                ("ms_total", C.c_double), ("ms_stage", C.c_double * 4), ("kernel_launches", C.c_int32),
                ("reserved", C.c_int32), ("src_window_pixels", C.c_uint64), ("tgt_window_pixels", C.c_uint64),
                ("sequence_pairs", C.c_uint64)]


class RasterTotals(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("polygons", "vertices", "pixels", "status_bytes", "sequences", "hnodes",
                                          "vnodes", "crossings", "clip_x_points", "clip_y_points", "chunks")] + \
               [(k, C.c_double) for k in ("ms_walk", "ms_clip_x", "ms_clip_y", "ms_cells", "ms_total")]


class RasterView(C.Structure):
    _fields_ = [("mbr", C.c_double * 4), ("dimx", C.c_int32), ("dimy", C.c_int32), ("step_x", C.c_double),
                ("step_y", C.c_double), ("nv", C.c_uint32), ("status_size", C.c_uint32), ("n_seq", C.c_uint32),
                ("n_hnodes", C.c_uint32), ("n_vnodes", C.c_uint32), ("num_layers", C.c_uint32),
                ("err", C.c_int32), ("reserved", C.c_uint32)]


SYMBOLS = ["farm_last_error", "farm_device_info", "farm_store_create", "farm_store_destroy", "farm_store_load",
           "farm_rasterize", "farm_intersect", "farm_within", "farm_intersection_area", "farm_raster_fetch",
           "farm_sync"]


def declare(lib):
    vp = C.c_void_p
    u8p = C.POINTER(C.c_uint8)
    u32p = C.POINTER(C.c_uint32)
    u64p = C.POINTER(C.c_uint64)
    f64p = C.POINTER(C.c_double)
    lib.farm_last_error.restype = C.c_char_p
    lib.farm_device_info.argtypes = [C.POINTER(C.c_int), C.c_char_p, C.c_size_t]
    lib.farm_store_create.argtypes = [C.POINTER(vp)]
    lib.farm_store_destroy.argtypes = [vp]
    lib.farm_store_destroy.restype = None
    lib.farm_store_load.argtypes = [vp, C.c_int, C.c_uint64, vp, vp, C.c_int]
    lib.farm_rasterize.argtypes = [vp, C.POINTER(RasterOpts)]
    lib.farm_store_load_dt.argtypes = [vp, C.c_int, C.c_char_p, C.c_int, u64p]
    lib.farm_intersect.argtypes = [vp, vp, C.c_uint64, C.c_int, C.c_int, vp, u64p, C.POINTER(Stats)]
    if hasattr(lib, "farm_within"):
        lib.farm_within.argtypes = [vp, vp, C.c_uint64, C.c_double, C.c_int, C.c_int, C.c_int, vp, u64p,
                                    C.POINTER(Stats)]
    lib.farm_within_mode.argtypes = [vp, vp, C.c_uint64, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, vp, u64p,
                                     C.POINTER(Stats)]
    lib.farm_contain.argtypes = [vp, vp, C.c_uint64, C.c_int, vp, u64p, C.POINTER(Stats)]
    lib.farm_contain_points.argtypes = [vp, C.c_int, vp, C.c_uint64, vp, C.c_uint64, C.c_int, vp, u64p]
    if hasattr(lib, "farm_intersection_area"):
        lib.farm_intersection_area.argtypes = [vp, vp, C.c_uint64, C.c_int, vp, C.POINTER(Stats)]
    lib.farm_raster_fetch.argtypes = [vp, C.c_int, C.c_uint64, C.POINTER(RasterView), u8p, u32p, u32p, u32p, f64p,
                                      u32p, f64p, f64p, f64p]
    lib.farm_sync.argtypes = [vp]
    lib.farm_raster_errors.argtypes = [vp, C.c_int, vp, C.c_uint64]
    lib.farm_raster_get_totals.argtypes = [vp, C.POINTER(RasterTotals)]
    lib.farm_intersect_static.argtypes = [vp, vp, C.c_uint64, vp, u64p]
    lib.farm_tc_gemm_test.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int]
    f32p = C.POINTER(C.c_float)
    lib.farm_mlp_param_count.restype = C.c_uint64
    lib.farm_mlp_param_count.argtypes = []
    lib.farm_mlp_init.argtypes = [vp, C.c_uint64]
    lib.farm_mlp_get.argtypes = [vp, vp]
    lib.farm_mlp_set.argtypes = [vp, vp]
    lib.farm_mlp_set_band.argtypes = [vp, C.c_float, C.c_float]
    lib.farm_area_plan_create.argtypes = [vp, C.c_uint64, C.c_uint64, C.POINTER(vp)]
    lib.farm_area_plan_run.argtypes = [vp, vp, C.c_uint64, C.c_int, vp, vp]
    lib.farm_area_plan_destroy.argtypes = [vp]
    lib.farm_area_plan_destroy.restype = None
    lib.farm_area_set_chunks.argtypes = [vp, vp]
    lib.farm_area_autotune.argtypes = [vp, vp, C.c_uint64, C.c_int, vp, vp]
    lib.farm_area_set_wide.argtypes = [vp, vp]
    lib.farm_mlp_set_band_cost.argtypes = [vp, C.c_float]
    lib.farm_intersect_filter.argtypes = [vp, vp, C.c_uint64, vp, vp]
    lib.farm_mlp_features.argtypes = [vp, vp, C.c_uint64, vp, C.c_uint64]
    lib.farm_mlp_grad.argtypes = [vp, vp, vp, C.c_uint64, C.c_uint64, f32p, vp]
    lib.farm_mlp_train.argtypes = [vp, vp, vp, C.c_uint64, C.c_int, C.c_int, C.c_float, C.c_uint64, f32p]
    lib.farm_mlp_predict.argtypes = [vp, vp, C.c_uint64, vp]
    lib.farm_event_record.argtypes = [vp, C.c_int]
    lib.farm_event_elapsed.argtypes = [vp, C.c_int, C.c_int, f64p]
    lib.farm_store_launches.argtypes = [vp]
    lib.farm_store_launches.restype = C.c_uint64
    lib.farm_store_device_bytes.argtypes = [vp, u64p]
    lib.farm_probe_issue_rates.argtypes = [f64p, f64p]
    lib.farm_mbr_join_gpu.argtypes = [vp, C.c_double, C.c_int, C.c_int, vp, C.c_uint64, C.c_int, u64p]

