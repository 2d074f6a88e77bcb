"""bench.py's JSON-line pieces that need no GPU: the roofline block's keys and
arithmetic, and the strip workload's bookkeeping."""
import json

import bench


def fake_totals():
    return {"polygons": 1000, "vertices": 10_000_000, "pixels": 200_000, "status_bytes": 200_000,
            "sequences": 20_000_000, "hnodes": 10_000_000, "vnodes": 10_000_000, "crossings": 20_000_000,
            "clip_x_points": 30_000_000, "clip_y_points": 50_000_000, "chunks": 2, "ms_walk": 12.0,
            "ms_clip_x": 4.0, "ms_clip_y": 9.0, "ms_cells": 5.0, "ms_total": 40.0}


def test_roofline_block_has_the_contract_keys():
    qs = {"segment_tests": 10**9, "src_window_pixels": 10**6, "tgt_window_pixels": 2 * 10**6}
    stage = {"raster_ms": 80.0, "query_ms": 20.0, "load_ms": 1.0}
    rl = bench.rooflines(fake_totals(), qs, 50_000, stage, steps=2)
    dom = rl["dominant"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic", "kernel"):
        assert k in dom
    # the dominant stage is the one with the most device time per step
    assert dom["kernel"] == "k_walk_tot + k_walk_fill"
    assert abs(dom["frac"] - dom["achieved"] / dom["peak"]) < 1e-12
    # edge walk: 16 flops per edge + 16 per crossing over 12 ms
    assert abs(dom["achieved"] - (16 * 1e7 + 16 * 2e7) / 12e-3 / 1e12) < 1e-9
    json.dumps(rl)  # serialisable as it goes into the JSON line
    assert rl["stages"]["refine"]["unit"] == "TFLOP/s" and rl["stages"]["raster_hbm_view"]["unit"] == "GB/s"


def test_filter_bytes_per_pair_and_pixel():
    qs = {"src_window_pixels": 800, "tgt_window_pixels": 1600}
    # 8 B ids + 2 x 64 B headers + 1/8 B result per pair, w/8 B per visited pixel
    assert bench.filter_bytes(qs, 10, 4) == 10 * (8 + 128 + 0.125) + 0.5 * 2400
