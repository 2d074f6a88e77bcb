"""bench.py's JSON-line pieces that need no GPU: the roofline block's keys and
arithmetic, and the strip workload's bookkeeping."""
import json

import numpy as np

import bench


def fake_totals():
    return {"polygons": 1000, "vertices": 10_000_000, "pixels": 200_000, "status_bytes": 200_000,
            "sequences": 20_000_000, "hnodes": 10_000_000, "vnodes": 10_000_000, "crossings": 20_000_000,
            "clip_x_points": 30_000_000, "clip_y_points": 50_000_000, "chunks": 2, "ms_walk": 12.0,
            "ms_clip_x": 4.0, "ms_clip_y": 9.0, "ms_cells": 5.0, "ms_total": 40.0}


PEAKS = {"hbm": 6.8e12, "hbm_src": "test", "fp64": 0.5e12, "fp32": 39e12, "fp_src": "test"}


def test_roofline_block_has_the_contract_keys():
    qs = {"segment_tests": 10**9, "src_window_pixels": 10**6, "tgt_window_pixels": 2 * 10**6}
    stage = {"raster_ms": 80.0, "query_ms": 10.0, "load_ms": 1.0, "step_ms": 92.0}
    rl = bench.rooflines(fake_totals(), qs, 50_000, stage, steps=2, peaks=PEAKS, ref_tests=None)
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
    # traffic: the ncu bytes per edge of the walk times the step's edges
    assert abs(dom["traffic"] - bench.TRAFFIC_PER_UNIT["edge_walk"] * fake_totals()["vertices"] / 2) < 1e-3
    # the per-edge traffic is above the walk's algorithmic bytes (ring, crossings, nodes), not below
    assert bench.TRAFFIC_PER_UNIT["edge_walk"] > 61.0


def test_filter_bytes_per_pair_and_pixel():
    qs = {"src_window_pixels": 800, "tgt_window_pixels": 1600}
    # 8 B ids + 2 x 64 B headers + 1/8 B result per pair, w/8 B per visited pixel
    assert bench.filter_bytes(qs, 10, 4) == 10 * (8 + 128 + 0.125) + 0.5 * 2400


def test_whole_path_fraction_and_reference_order_tests():
    qs = {"segment_tests": 4 * 10**9, "src_window_pixels": 10**6, "tgt_window_pixels": 2 * 10**6}
    stage = {"raster_ms": 80.0, "query_ms": 20.0, "load_ms": 1.0, "step_ms": 102.0}
    rl = bench.rooflines(fake_totals(), qs, 50_000, stage, steps=2, peaks=PEAKS, ref_tests=10**9)
    wp = rl["stages"]["whole_path"]
    t = fake_totals()
    f64 = (16 * t["vertices"] + 16 * t["crossings"] + 4 * t["clip_y_points"] + 2 * t["clip_x_points"] +
           4 * t["clip_y_points"]) / 2
    raster = max(f64 / PEAKS["fp64"], 0.0)
    query = max(28 * 10**9 / 2 / PEAKS["fp32"], bench.filter_bytes(qs, 50_000, 4) / 2 / PEAKS["hbm"])
    assert abs(wp["roofline_ms"] - (raster + query) * 1e3) < 1e-6 + 1e-9 * wp["roofline_ms"]
    assert abs(wp["frac"] - wp["roofline_ms"] / 51.0) < 1e-9
    # refine is charged the reference-order count; the GPU's own count rides along
    assert rl["stages"]["refine"]["gpu_tests_over_reference_order"] == 4.0


def test_cpu_sample_is_systematic_by_size_and_clustered_by_source():
    rng = np.random.default_rng(0)
    strips = []
    for b in range(2):
        ns, nt = 50, 200
        pairs = np.array(sorted({(int(s), int(t)) for s, t in zip(rng.integers(0, ns, 900), rng.integers(0, nt, 900))}),
                         np.uint32)
        strips.append({"strip": b, "s_idx": np.arange(ns, dtype=np.uint64) + 1000 * b,
                       "t_idx": np.arange(nt, dtype=np.uint64) + 5000 * b, "pairs": pairs,
                       "s_nv": rng.integers(16, 100_000, ns), "t_nv": rng.integers(16, 100_000, nt)})
    cs = bench.CpuSample(job=None, strips=strips, seed=3)
    assert len(cs.poly) == 2 * (50 + 200)
    ent, k = cs.raster_sample(50, 7)
    assert k == 10 and len(ent) == 50  # 500 polygons, every 10th
    # one polygon from every run of k in size order: the sample spans the sizes
    assert (np.diff(ent[:, 3]) >= 0).all()
    assert ent[:, 3].max() >= np.sort(cs.poly[:, 3])[-k]
    q = cs.query_sample(300)
    assert len(q) >= 300
    # every sampled source brings all of its candidate pairs
    for i in (0, 1):
        sel = q[q[:, 0] == i, 1]
        srcs = set(strips[i]["pairs"][sel, 0].tolist())
        full = [p for p in range(len(strips[i]["pairs"])) if strips[i]["pairs"][p, 0] in srcs]
        assert sorted(sel.tolist()) == full
