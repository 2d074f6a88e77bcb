"""Benchmark of the polygon-join hot path: exact intersect pairs/sec on one GB300.

Workload (configuration 2): seeded star polygons, 100,000 sources x
1,000,000 targets, vertex count log-uniform 16..100,000, mean radius
log-uniform 0.05..2.0, per-vertex radius x lognormal(0, 0.3); the domain side
is calibrated so the MBR join yields ~20M candidate pairs. The job is cut into
spatial strips by source centre: strip b holds the sources centred in it and
the targets that reach them, and all of its candidate pairs. One "step" is
one strip through the whole hot path — ring upload into the store's layout,
rasterization of every polygon of the strip (stage a), pixel-pair filter +
border refinement of every candidate (stages b, c), result bytes. Steps repeat
the strip of this rank (the inputs are GBs, far larger than the 129 MB L2, so
no L2 flush is needed).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank takes its own strip (weak scaling, no collective on
the data path); value = all ranks' pairs / max rank time.
--impl reference times the reference's CPU algorithm (the oracle port under
oracle/, all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "polygon-pair tests/sec on 1 GB300: exact vs learned-approx at 99.9% P/R"
UNIT = "pairs/s"

# configuration 2
N_SRC, N_TGT = 100_000, 1_000_000
TARGET_PAIRS = 20_000_000


def star_params(dom_hi):
    from farm_gb300.polygons import StarParams
    return StarParams(dom_lo=0.0, dom_hi=dom_hi, r_lo=0.05, r_hi=2.0, n_lo=16, n_hi=100_000, sigma=0.3)


def calibrate_domain(seed: int) -> float:
    """Domain side L giving ~20M expected MBR-overlap pairs for 100k x 1M polygons.

    For centres uniform in [0, L]^2, P(overlap) ~ E[(w_s + w_t)(h_s + h_t)] / L^2;
    the expectation is estimated from the MBRs of 4,000 polygons per side of a
    unit-domain sample (sizes do not depend on the domain)."""
    from farm_gb300 import polygons as P
    prm = star_params(1.0)
    prm.n_hi = 100_000
    a = P.generate(prm, seed + 7, 4000).mbrs()
    b = P.generate(prm, seed + 8, 4000).mbrs()
    wa, ha = a[:, 2] - a[:, 0], a[:, 3] - a[:, 1]
    wb, hb = b[:, 2] - b[:, 0], b[:, 3] - b[:, 1]
    e = float(np.mean((wa[:, None] + wb[None, :2000]) * (ha[:, None] + hb[None, :2000])))
    return math.sqrt(N_SRC * N_TGT * e / TARGET_PAIRS)


class Clocks:
    """Samples nvidia-smi clocks/throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def log(msg: str) -> None:
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


# every vertex of a generated polygon lies within this many mean radii of its
# centre unless its lognormal factor exceeds exp(0.3 * 6.5) (probability ~4e-11)
EXTENT_RADII = math.exp(0.3 * 6.5)
# configuration-4 sample for the area block: polygons per pool and domain side
AREA_POOL = 1500
AREA_SIDE = 40.0


def build_workload(seed: int, strip: int, n_strips: int, vpr: int):
    """Host (pinned) rings and candidate pairs of one strip of the job.

    The domain is cut into n_strips vertical strips by source centre. Strip b
    holds the sources centred in it and every target whose extent (centre +-
    EXTENT_RADII x mean radius) reaches the x-range of the strip's source MBRs;
    its pairs are the MBR-overlapping (source, target) pairs of those sets, so
    every candidate pair of the job belongs to exactly one strip, and only
    targets straddling a strip boundary are rasterized in two steps."""
    import torch
    from farm_gb300 import polygons as P
    from farm_gb300 import shard

    L = calibrate_domain(seed)
    prm = star_params(L)
    log(f"domain side {L:.2f}")
    s_idx = shard.strip_sources(P.centres(prm, seed, N_SRC), strip, n_strips, L)

    def gen_pinned(seed_, idx):
        counts = P.vertex_counts(prm, seed_, idx)
        off = torch.zeros(len(idx) + 1, dtype=torch.int64).pin_memory()
        offn = off.numpy().view(np.uint64)
        total = int(counts.sum(dtype=np.uint64))
        xy = torch.empty((total, 2), dtype=torch.float32).pin_memory()
        ps = P.generate_indices(prm, seed_, idx, out_off=offn, out_xy=xy.numpy())
        return ps, off, xy

    S, S_off_t, S_xy_t = gen_pinned(seed, s_idx)
    ms = S.mbrs()
    log(f"strip {strip}/{n_strips}: {S.n} sources, {S.total} vertices")
    t_idx = shard.strip_targets(ms, P.centres(prm, seed + 1, N_TGT), EXTENT_RADII)
    T, T_off_t, T_xy_t = gen_pinned(seed + 1, t_idx)
    pairs = P.mbr_join(ms, T.mbrs())
    log(f"targets: {T.n} ({T.total} vertices, {len(np.unique(pairs[:, 1]))} with candidates); "
        f"candidates: {len(pairs)}")
    return {"L": L, "S": S, "T": T, "pairs": pairs, "strip": strip, "n_strips": n_strips,
            "pinned": (S_off_t, S_xy_t, T_off_t, T_xy_t)}


def filter_bytes(stats: dict, n_pairs: int, bits: int) -> float:
    """Algorithmic bytes of the filter+refine kernel for one launch: per pair 8
    (pair ids) + 2 x 64 (raster headers) + w/8 per source window pixel and per
    target pixel visited + 1/8 (result bit)."""
    return n_pairs * (8 + 128 + 0.125) + bits / 8.0 * (stats["src_window_pixels"] + stats["tgt_window_pixels"])


# Peaks. HBM: MEASURED_PEAKS.json (a STREAM-style copy on this GPU model).
# FP64 / FP32: nominal issue rates, as no measured figure exists for them —
# GB300 issues FP64 at 2 lanes/clock/SM (1.25 TFLOP/s counts an FMA as two
# flops; these kernels cannot fuse, so every flop is one instruction) and FP32
# at 128 lanes/clock/SM; 152 SMs at 2.07 GHz.
FP64_PEAK = 2 * 152 * 2.07e9
FP32_PEAK = 128 * 152 * 2.07e9


def rooflines(rt: dict, qs: dict, n_pairs: int, stage: dict, steps: int) -> dict:
    """Roofline of each measured stage from its algorithmic work per unit
    (counts of the last step; times are the per-step means of the timed steps).

    edge walk (2 launches per edge: totals + counts, then fill): FP64, 16 flops per edge
      (endpoint cells, slope and intercept) + 16 per pixel-boundary crossing
      (both branches of one walk step), the reference's arithmetic for ONE walk;
    cell clip (count + emit): FP64, 4 flops per emitted clip point (slope and
      the two line abscissae, shared by ~2 points per edge-row);
    column clip: FP64, 2 flops per emitted point;
    cell areas: FP64, 4 flops per clip point (shoelace term + accumulation);
    filter + refine (k_intersect): FP32, 28 flops per segment-pair test
      (4 cross products x 7); its HBM bytes per filter_bytes();
    whole raster stage, HBM view: 8 B per vertex read + the raster written
      (w P / 8 + 4 (P + n) + 8 sequences + 8 nodes).
    """
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0)) * 1e9
    per = lambda k: stage[k] / steps
    walk_ms = rt["ms_walk"]
    st = {}

    def fp(name, flops, ms, peak, kind, peak_src):
        ach = flops / (ms * 1e-3) if ms > 0 else None
        st[name] = {"bound": kind, "algorithmic_flops": flops, "kernel_ms": ms,
                    "achieved": ach / 1e12 if ach else None, "peak": peak / 1e12, "unit": "TFLOP/s",
                    "frac": ach / peak if ach else None, "peak_source": peak_src}

    src64 = "nominal FP64 issue rate (no measured FP64 figure in MEASURED_PEAKS.json)"
    fp("edge_walk", 16.0 * rt["vertices"] + 16.0 * rt["crossings"], walk_ms, FP64_PEAK, "fp64", src64)
    fp("cell_clip", 4.0 * rt["clip_y_points"], rt["ms_clip_y"], FP64_PEAK, "fp64", src64)
    fp("column_clip", 2.0 * rt["clip_x_points"], rt["ms_clip_x"], FP64_PEAK, "fp64", src64)
    fp("cell_area", 4.0 * rt["clip_y_points"], rt["ms_cells"], FP64_PEAK, "fp64", src64)
    fp("refine", 28.0 * qs["segment_tests"], per("query_ms"), FP32_PEAK, "fp32",
       "nominal FP32 issue rate (no measured FP32 figure in MEASURED_PEAKS.json)")
    fb = filter_bytes(qs, n_pairs, 4)
    rb = 8.0 * rt["vertices"] + 0.5 * rt["pixels"] + 4.0 * (rt["pixels"] + rt["polygons"]) + \
        8.0 * rt["sequences"] + 8.0 * (rt["hnodes"] + rt["vnodes"])
    rms = per("raster_ms")
    st["raster_hbm_view"] = {"bound": "hbm", "algorithmic_bytes": rb, "kernel_ms": rms,
                             "achieved": rb / (rms * 1e-3) / 1e9 if rms > 0 else None, "peak": hbm / 1e9,
                             "unit": "GB/s", "frac": rb / (rms * 1e-3) / hbm if rms > 0 else None,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    st["filter_hbm_view"] = {"bound": "hbm", "algorithmic_bytes": fb, "kernel_ms": per("query_ms"),
                             "achieved": fb / (per("query_ms") * 1e-3) / 1e9 if per("query_ms") > 0 else None,
                             "peak": hbm / 1e9, "unit": "GB/s", "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    # the dominant kernel: the stage with the most device time
    cand = {k: v for k, v in st.items() if k in ("edge_walk", "cell_clip", "column_clip", "cell_area", "refine")}
    name = max(cand, key=lambda k: cand[k]["kernel_ms"] or 0.0)
    dom = dict(cand[name])
    dom["kernel"] = {"edge_walk": "k_walk_tot + k_walk_fill", "cell_clip": "k_clipy (count + emit)",
                     "column_clip": "k_clipx (count + emit)", "cell_area": "k_cells",
                     "refine": "k_intersect (filter + refine)"}[name]
    dom["traffic"] = None
    dom["peak"] = dom["peak"]
    return {"dominant": dom, "stages": st}


def choose_band(prob: np.ndarray, y: np.ndarray, budget: float, positives: int = 0) -> tuple:
    """Narrowest band (lo, hi) whose decided pairs stay within the error
    budget on held-out pairs: at most budget x positives false positives above
    hi and at most budget x positives false negatives below lo (positives: of
    the whole held-out set, default those of y). Pairs strictly inside
    (lo, hi) are refined exactly and cost no accuracy."""
    pos = max(int(positives or y.sum()), 1)
    allow = int(budget * pos)
    o = np.argsort(-prob, kind="stable")  # descending
    fp = np.cumsum(y[o] == 0)
    k = int(np.searchsorted(fp, allow, side="right"))  # first k decided-1 pairs hold <= allow negatives
    hi = float(prob[o[k - 1]]) if k > 0 else 1.01
    o2 = np.argsort(prob, kind="stable")  # ascending
    fn = np.cumsum(y[o2] == 1)
    k2 = int(np.searchsorted(fn, allow, side="right"))
    lo = float(prob[o2[k2 - 1]]) if k2 > 0 else -0.01
    if lo >= hi:  # never let the two decided sets overlap
        lo = min(lo, hi - 1e-6)
    # ties at the thresholds: decide only strictly beyond them
    return np.nextafter(np.float32(lo), np.float32(-1)).item(), np.nextafter(np.float32(hi), np.float32(2)).item()


def choose_band_cost(prob: np.ndarray, y: np.ndarray, cost: np.ndarray, budget: float, positives: int) -> tuple:
    """Lambda of the cost-aware band (decide when min(p, 1 - p) <= lambda x
    cost). Held-out pairs are decided in order of uncertainty per unit of
    refinement cost while their errors stay within budget x positives, so the
    error budget buys the most refinement. Arithmetic in float32, as on the
    device. Returns (lambda, decided fraction, decided share of cost)."""
    p = prob.astype(np.float32)
    c = cost.astype(np.float32)
    u = np.minimum(p, np.float32(1) - p)
    err = (p >= np.float32(0.5)) != (y == 1)
    allow = int(budget * max(int(positives), 1))
    r = u / c
    o = np.argsort(r, kind="stable")
    ce = np.cumsum(err[o])
    k = int(np.searchsorted(ce, allow, side="right"))
    if k == 0:
        return 0.0, 0.0, 0.0
    lam = np.float32(r[o[k - 1]])
    for _ in range(64):  # ties and rounding: shrink until the held-out errors fit
        dec = u <= lam * c
        if int(err[dec].sum()) <= allow:
            break
        lam = np.nextafter(lam, np.float32(0))
    dec = u <= lam * c
    return float(lam), float(dec.mean()), float(c[dec].sum() / c.sum())


def train_scorer(args, store, dev) -> dict:
    """Train the learned scorer on pairs of a strip drawn with a separate seed,
    labelled by the exact path, and set its band from held-out pairs."""
    import torch
    Wt = build_workload(args.seed + 1000, 0, args.strips, args.vpr)
    so, sx, to, tx = (t.to(dev) for t in Wt["pinned"])
    pairs = Wt["pairs"]
    store.load(0, so, sx)
    store.load(1, to, tx)
    store.rasterize(vpr=args.vpr, category_count=16, strict=False)
    from farm_gb300.engine import MODE_FILTER
    dp = torch.from_numpy(pairs.view(np.int32)).to(dev).view(len(pairs), 2)
    lab, _ = store.intersect(dp)
    code, cost = store.filter_costs(dp)  # the scorer only sees pairs the filter leaves (3)
    keep = torch.nonzero(lab != 2).flatten()
    g = torch.Generator(device="cpu").manual_seed(args.seed + 1001)
    keep = keep[torch.randperm(len(keep), generator=g).to(dev)][: args.learned_pairs]
    nv = max(len(keep) // 10, 1)
    val, tr = keep[:nv], keep[nv:]
    tr = tr[code[tr] == 3]
    pos_val = int((lab[val] == 1).sum())
    val = val[code[val] == 3]
    t0 = time.perf_counter()
    loss = store.mlp_train(dp[tr].contiguous(), lab[tr].contiguous(), epochs=args.learned_epochs, batch=4096,
                           lr=2e-3, seed=args.seed)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    prob = store.mlp_predict(dp[val].contiguous()).cpu().numpy()
    y = lab[val].cpu().numpy().astype(np.int64)
    vcost = cost[val].cpu().numpy()
    if args.learned_band == "cost":
        lam, dfrac, dcost = choose_band_cost(prob, y, vcost, args.learned_budget * 0.8, pos_val)
        lo, hi = -1.0, 2.0
        store.mlp_band(lo, hi, lam)
        inband = 1.0 - dfrac
        log(f"scorer trained on {len(tr)} pairs in {train_s:.1f}s (loss {loss:.4f}); cost-aware band lambda "
            f"{lam:.3g}: decides {dfrac:.3f} of {len(val)} held-out scored pairs, {dcost:.3f} of their cost")
    else:
        lo, hi = choose_band(prob, y, args.learned_budget, pos_val)
        lam, dcost = 0.0, None
        store.mlp_band(lo, hi)
        inband = float(((prob > lo) & (prob < hi)).mean()) if len(prob) else 0.0
        log(f"scorer trained on {len(tr)} pairs in {train_s:.1f}s (loss {loss:.4f}); band ({lo:.4f}, {hi:.4f}) "
            f"from {len(val)} held-out pairs, {inband:.3f} of them inside it")
    del so, sx, to, tx, dp, lab, code, cost
    torch.cuda.empty_cache()
    return {"train_pairs": int(len(tr)), "heldout_pairs": int(len(val)), "epochs": args.learned_epochs,
            "heldout_inside_band": inband, "band_kind": args.learned_band, "cost_lambda": lam,
            "heldout_decided_cost_share": dcost,
            "train_s": train_s, "final_loss": loss, "band": [lo, hi], "error_budget": args.learned_budget,
            "seed": args.seed + 1000}


def pr(out, ref):
    """Precision and recall of out against the exact results (pairs the exact
    path marks 2, unrasterizable, are left out)."""
    ok = ref != 2
    o, r = out[ok] == 1, ref[ok] == 1
    tp = int((o & r).sum())
    fp = int((o & ~r).sum())
    fn = int((~o & r).sum())
    return (tp / max(tp + fp, 1), tp / max(tp + fn, 1))


def learned_eval(store, d_pairs, exact_out, exact_query_ms: float, raster_ms: float, reps: int) -> dict:
    """Learned mode and the -a heuristic on the step's pairs, against exact."""
    import torch
    from farm_gb300.engine import MODE_APPROX, MODE_LEARNED
    res = {}
    for name, mode in (("learned", MODE_LEARNED), ("heuristic", MODE_APPROX)):
        out = torch.empty_like(exact_out)
        store.intersect(d_pairs, mode=mode, out=out)  # warm-up
        ms = 0.0
        st = {}
        for _ in range(reps):
            store.intersect(d_pairs, mode=mode, out=out)
            st = store.last_stats
            ms += st["ms_total"] if mode == MODE_APPROX else 0.0
        abst = st.get("fp64_rechecks", 0)
        if mode == MODE_LEARNED:  # timed around the whole call (predict + band + exact refinement)
            torch.cuda.synchronize()
            store.event_record(4)
            for _ in range(reps):
                store.intersect(d_pairs, mode=mode, out=out)
            store.event_record(5)
            ms = store.event_elapsed(4, 5)
        ms /= reps
        p, r = pr(out.cpu().numpy(), exact_out.cpu().numpy())
        n = d_pairs.shape[0]
        res[name] = {"precision": p, "recall": r, "query_ms": ms, "query_pairs_per_s": n / (ms * 1e-3),
                     "speedup_vs_exact_query": exact_query_ms / ms,
                     "step_pairs_per_s": n / ((raster_ms + ms) * 1e-3),
                     "speedup_vs_exact_step": (raster_ms + exact_query_ms) / (raster_ms + ms)}
        if mode == MODE_LEARNED:
            res[name]["filter_decided_pairs"] = int(n - st.get("border_pairs", 0))
            res[name]["scored_pairs"] = int(st.get("border_pairs", 0))
            res[name]["abstained_pairs"] = int(abst)
            res[name]["abstained_frac"] = abst / n
            res[name]["abstained_refine_ms"] = st.get("ms_stage", [0, 0])[1]
    return res


def run_ours(args) -> dict:
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from farm_gb300 import shard
    from farm_gb300.engine import Store

    dev = torch.device("cuda", local)
    store = Store()
    learned_train = train_scorer(args, store, dev) if args.learned else None
    mine = shard.strips_of_rank(rank, world, args.strips)
    if not mine:
        raise SystemExit(f"{world} ranks need at least {world} strips (--strips {args.strips})")
    W = build_workload(args.seed, mine[0], args.strips, args.vpr)
    S, T, pairs = W["S"], W["T"], W["pairs"]
    S_off_t, S_xy_t, T_off_t, T_xy_t = W["pinned"]
    d = {k: v.to(dev) for k, v in (("so", S_off_t), ("sx", S_xy_t), ("to", T_off_t), ("tx", T_xy_t))}
    d_pairs = torch.from_numpy(pairs.view(np.int32)).to(dev)
    d_out = torch.empty(len(pairs), dtype=torch.uint8, device=dev)
    h_out = torch.empty(len(pairs), dtype=torch.uint8).pin_memory()
    h_pairs = torch.from_numpy(pairs.view(np.int32)).pin_memory()

    stage = {"load_ms": 0.0, "raster_ms": 0.0, "query_ms": 0.0}

    def step_device(timed=False):
        store.event_record(4)
        store.load(0, d["so"], d["sx"])
        store.load(1, d["to"], d["tx"])
        store.event_record(5)
        store.rasterize(vpr=args.vpr, category_count=16, strict=False)
        if timed:
            stage["load_ms"] += store.event_elapsed(4, 5)
        store.event_record(4)
        _, found = store.intersect(d_pairs.view(len(pairs), 2), out=d_out)
        if timed:
            stage["raster_ms"] += store.event_elapsed(5, 4)
            stage["query_ms"] += store.last_stats["ms_total"]
        return found

    def step_e2e():
        store.load(0, S_off_t.numpy().view(np.uint64), S_xy_t.numpy())
        store.load(1, T_off_t.numpy().view(np.uint64), T_xy_t.numpy())
        store.rasterize(vpr=args.vpr, category_count=16, strict=False)
        _, found = store.intersect(h_pairs.numpy().view(np.uint32).reshape(-1, 2), out=h_out.numpy())
        return found

    for i in range(args.warmup):
        t = time.time()
        step_device()
        free, total = torch.cuda.mem_get_info(dev)
        log(f"warmup step {i}: {time.time() - t:.2f}s, device memory in use {(total - free) / 2**30:.1f} GiB, "
            f"raster {store.raster_totals()}, stats {store.last_stats}")
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    launches0 = store.launches
    store.event_record(0)
    founds = []
    for _ in range(args.steps):
        founds.append(step_device(timed=True))
    store.event_record(1)
    ms = store.event_elapsed(0, 1)
    torch.cuda.synchronize()
    launches = store.launches - launches0
    last = dict(store.last_stats)
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    t_dev = ms / 1000.0
    # end to end through the C ABI with host buffers
    step_e2e()
    torch.cuda.synchronize()
    store.event_record(2)
    for _ in range(args.steps):
        step_e2e()
    store.event_record(3)
    ms_e2e = store.event_elapsed(2, 3)
    t_e2e = ms_e2e / 1000.0
    t_dev, t_e2e, total_pairs = shard.reduce_job(t_dev, t_e2e, len(pairs), device=dev)
    value = total_pairs * args.steps / t_dev
    e2e_value = total_pairs * args.steps / t_e2e
    rl = rooflines(store.raster_totals(), last, len(pairs), stage, args.steps)
    h2d = int(S_xy_t.numel() * 4 + T_xy_t.numel() * 4 + S_off_t.numel() * 8 + T_off_t.numel() * 8 + pairs.nbytes)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (seeded star polygons, configuration 2 generator)",
        "config": {"workload": "intersect, configuration 2: 100k sources x 1M targets, nv log-uniform 16..100000, "
                               f"~20M MBR candidates, -v {args.vpr}, -w 16; one step = strip {W['strip']} of "
                               f"{W['n_strips']} (sources centred in it + the targets reaching them)",
                   "domain_side": W["L"], "vpr": args.vpr, "category_count": 16, "n_source": N_SRC,
                   "n_target": N_TGT, "strips": W["n_strips"], "sources_per_step": int(S.n),
                   "targets_per_step": int(T.n), "candidate_pairs_per_step": len(pairs), "found_per_step": founds[-1],
                   "vertices_per_step": int(S.total + T.total), "l2": "inputs larger than L2 (no flush needed)",
                   "seed": args.seed, "parallelism": f"weak-dp{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(len(pairs))},
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": rl["dominant"],
        "stages": rl["stages"],
        "stage_ms": {"load": stage["load_ms"] / args.steps, "raster": stage["raster_ms"] / args.steps,
                     "filter_refine": stage["query_ms"] / args.steps, "step": ms / args.steps},
    }
    if learned_train is not None and rank == 0:
        lr_ = learned_eval(store, d_pairs.view(len(pairs), 2), d_out, stage["query_ms"] / args.steps,
                           stage["raster_ms"] / args.steps, reps=3)
        lr_["train"] = learned_train
        lr_["note"] = ("query = stages b-c on the rasterized strip (learned: predict + band + exact refinement of "
                       "abstentions); step adds the strip's rasterization, which both modes need")
        result["learned"] = lr_
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(W, args, budget_s=args.cpu_seconds, threads=1, gpu_out=h_out.numpy())
    store.close()
    if rank == 0 and args.area_pairs > 0:
        result["area"] = area_eval(args)
    if world > 1:
        dist.destroy_process_group()
    return result if rank == 0 else None


def area_eval(args) -> dict:
    """Intersection area (stage d) on a configuration-4 sample, through a captured area plan.

    Configuration 4 mixes tiny and huge polygons (vertex counts log-uniform
    8..200,000 on each side) in one launch. The sample draws two pools of
    polygons from the star generator and takes args.area_pairs of their
    MBR-overlapping pairs at random, in one batch: one CUDA-graph launch of
    the persistent work-stealing kernel per pass. value = pairs / device time
    of one pass, timed with CUDA events (median of three passes after one
    warm-up pass)."""
    from farm_gb300 import polygons as P
    from farm_gb300.engine import Store

    t0 = time.time()
    prm = P.StarParams(dom_lo=0.0, dom_hi=AREA_SIDE, r_lo=0.05, r_hi=2.0, n_lo=8, n_hi=200_000, sigma=0.3)
    S = P.generate(prm, args.seed + 400, AREA_POOL)
    T = P.generate(prm, args.seed + 401, AREA_POOL)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    rng = np.random.default_rng(args.seed + 402)
    pairs = np.ascontiguousarray(pairs[rng.permutation(len(pairs))][:args.area_pairs])
    es = np.diff(S.off.astype(np.int64))[pairs[:, 0]]
    et = np.diff(T.off.astype(np.int64))[pairs[:, 1]]
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=10, strict=False)
    ras_s = st.raster_totals()["ms_total"] / 1000.0
    # items per pair at the smallest chunk the autotuner may pick (32 edges)
    plan = st.area_plan(max_pairs=len(pairs), max_items=int(((es + 31) // 32 + (et + 31) // 32).sum()) + 64)
    plan.run(pairs)
    warm_ms = plan.last_stats["ms_total"]
    ms = []
    for _ in range(3):
        out = plan.run(pairs)
        ms.append(plan.last_stats["ms_total"])
    plan.close()
    st.close()
    med = float(np.median(ms))
    log(f"area: {len(pairs)} pairs, {int(es.sum() + et.sum())} edges, {med:.1f} ms per pass "
        f"(warm-up {warm_ms:.1f} ms), {time.time() - t0:.1f} s wall")
    return {"metric": "intersection-area pairs/sec, configuration-4 sample", "value": len(pairs) / (med / 1000.0),
            "unit": "pairs/s", "ms_per_pass": med, "passes": 3, "warmup_passes": 1, "dtype": "f64",
            "edges_per_s": float(es.sum() + et.sum()) / (med / 1000.0),
            "config": {"workload": f"{len(pairs)} MBR-overlapping pairs drawn at random from two pools of "
                                   f"{AREA_POOL} star polygons, vertex counts log-uniform 8..200,000, radii "
                                   f"0.05..2 in a {AREA_SIDE:g} x {AREA_SIDE:g} domain; one batch, one "
                                   "graph launch per pass", "vpr": 10, "pairs": len(pairs),
                       "edges_in_pairs": int(es.sum() + et.sum()), "largest_pair_edges": int((es + et).max()),
                       "pool_vertices": int(S.total + T.total), "seed": args.seed + 400},
            "nonzero_areas": int((out > 0).sum()), "rasterize_s": ras_s}


def _oracle_chunk(job):
    """Worker: oracle rasterization + intersect over a list of sampled pairs."""
    import time as _t
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    rings_s, rings_t, pairs, vpr = job

    def ras(r):
        try:
            return O.Raster(r, vpr)
        except RuntimeError:  # the reference aborts on this polygon
            return None

    t0 = _t.perf_counter()
    rs = {k: ras(r) for k, r in rings_s.items()}
    rt = {k: ras(r) for k, r in rings_t.items()}
    t1 = _t.perf_counter()
    res = [2 if rs[s] is None or rt[t] is None else int(O.intersect(rs[s], rt[t])) for s, t in pairs]
    t2 = _t.perf_counter()
    verts = sum(len(r) for r in rings_s.values()) + sum(len(r) for r in rings_t.values())
    return t1 - t0, t2 - t1, verts, len(pairs), sum(v == 1 for v in res), [(s, t, int(v)) for (s, t), v in zip(pairs, res)]


def cpu_baseline(W, args, budget_s: float, threads: int, gpu_out=None) -> dict:
    """The CPU oracle (a port of the reference's algorithm) on a bounded uniform
    sample of the step's candidate pairs. Raster time is charged per vertex and
    query time per pair, then scaled to the whole step."""
    import multiprocessing as mp
    S, T, pairs = W["S"], W["T"], W["pairs"]
    rng = np.random.default_rng(args.seed + 99)
    order = rng.permutation(len(pairs))
    chunk = 8

    def job(k):
        sel = pairs[order[k:k + chunk]]
        rs = {int(s): np.ascontiguousarray(S.ring(int(s))) for s in set(sel[:, 0].tolist())}
        rt = {int(t): np.ascontiguousarray(T.ring(int(t))) for t in set(sel[:, 1].tolist())}
        return (rs, rt, [(int(a), int(b)) for a, b in sel], args.vpr)

    t_r = t_q = 0.0
    verts = npairs = found = 0
    checked = []
    t0 = time.perf_counter()
    ctx = mp.get_context("spawn")
    with ctx.Pool(threads) as pool:
        pending, k = [], 0
        while True:
            while len(pending) < 2 * threads and k < len(order) and time.perf_counter() - t0 < budget_s:
                pending.append(pool.apply_async(_oracle_chunk, (job(k),)))
                k += chunk
            if not pending:
                break
            r = pending.pop(0).get()
            t_r += r[0]
            t_q += r[1]
            verts += r[2]
            npairs += r[3]
            found += r[4]
            checked.extend(r[5])
    total_verts = S.total + T.total
    raster_s = t_r / max(verts, 1) * total_verts
    query_s = t_q / max(npairs, 1) * len(pairs)
    value = len(pairs) / (raster_s + query_s) * 1.0
    extra = {}
    if gpu_out is not None and checked:
        # the same oracle doubles as a full-size parity spot check of the GPU results
        index = {(int(a), int(b)): i for i, (a, b) in enumerate(pairs)}
        bad = sum(1 for s_, t_, v in checked if int(gpu_out[index[(s_, t_)]]) != v)
        extra = {"parity_sample_pairs": len(checked), "parity_sample_mismatches": bad}
    return {**extra, "value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{npairs} uniformly sampled candidate pairs of the step ({verts} vertices rasterized), "
                      f"{time.perf_counter() - t0:.1f} s wall on {threads} core(s); raster time scaled per vertex "
                      f"to the step's {total_verts} vertices, query time per pair to its {len(pairs)} pairs",
            "raster_s_per_step": raster_s, "query_s_per_step": query_s}


def run_reference(args) -> dict:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    W = build_workload(args.seed, 0, args.strips, args.vpr)
    threads = os.cpu_count() or 1
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.warmup + args.steps):
        vals.append(cpu_baseline(W, args, budget_s=args.ref_step_seconds, threads=threads))
    wall = time.perf_counter() - t0
    v = statistics.median([x["value"] for x in vals[args.warmup:]])
    cb = dict(vals[-1])
    cb["value"] = v
    cb["kind"] = "port"
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1000 / (args.warmup + args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded star polygons, configuration 2 generator)", "impl": "reference",
            "config": {"workload": "intersect, configuration 2 (see ours); CPU oracle port of the reference, "
                                   f"-v {args.vpr}", "vpr": args.vpr, "seed": args.seed},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--vpr", type=int, default=64)
    ap.add_argument("--strips", type=int, default=10, help="strips the job is cut into (one per step)")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--ref-step-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--area-pairs", type=int, default=0,
                    help="pairs of the configuration-4 area sample (0 = skip the area block; one pass over "
                         "1,000 pairs takes ~13 s)")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip training and evaluating the learned scorer")
    ap.add_argument("--learned-pairs", type=int, default=2_000_000, help="training + held-out pairs")
    ap.add_argument("--learned-epochs", type=int, default=12)
    ap.add_argument("--learned-band", choices=["cost", "plain"], default="cost",
                    help="cost-aware band (spend the error budget on expensive pairs) or a plain probability band")
    ap.add_argument("--learned-budget", type=float, default=5e-4,
                    help="false positives (negatives) allowed above (below) the band, per positive")
    args = ap.parse_args()
    res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
