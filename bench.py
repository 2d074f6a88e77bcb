"""Benchmark of the polygon-join hot path: exact intersect pairs/sec on one GB300.

Workload (configuration 2): seeded star polygons, 100,000 sources x
1,000,000 targets, vertex count log-uniform 16..100,000, mean radius
log-uniform 0.05..2.0, per-vertex radius x lognormal(0, 0.3); the domain side
is calibrated so the MBR join yields ~20M candidate pairs. The job is cut into
spatial strips by source centre: strip b holds the sources centred in it, the
targets whose vertices reach the x-range of those sources' MBRs (an exact
bound from the generator), and all of the strip's candidate pairs, so the
strips partition the job's pairs. One "step" is one strip through the whole
hot path — ring upload into the store's layout, rasterization of every
polygon of the strip (stage a), pixel-pair filter + border refinement of every
candidate (stages b, c), result bytes. Steps cycle through the rank's strips,
so K >= the strip count covers the whole job; every strip's rings are
resident in HBM before the timed region (the inputs are GBs, far larger than
the 129 MB L2, so no L2 flush is needed).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank takes strips r, r + N, ... (weak scaling, no
collective on the data path); value = all ranks' pairs / max rank time.
--impl reference times the reference's CPU algorithm (the oracle port under
oracle/, all host cores) on bounded samples of the same job.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
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
# configuration-4 sample for the area block: polygons per pool and domain side
AREA_POOL = 1500
AREA_SIDE = 40.0


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


# ------------------------------------------------------------------ job ----
class Job:
    """Configuration 2 cut into strips. Only centres and exact extents are held
    for the whole job; a strip's rings are generated on demand."""

    def __init__(self, seed: int, n_strips: int):
        from farm_gb300 import polygons as P
        from farm_gb300 import shard
        self.seed, self.n_strips = seed, n_strips
        self.L = calibrate_domain(seed)
        self.prm = star_params(self.L)
        t0 = time.time()
        self.src_c = P.centres(self.prm, seed, N_SRC)
        self.tgt_c = P.centres(self.prm, seed + 1, N_TGT)
        # an interval that holds every vertex of each target (the generator's
        # largest radius about the centre, widened by float rounding)
        self.tgt_ext = shard.target_extents(self.tgt_c, P.radii(self.prm, seed + 1, N_TGT))
        log(f"domain side {self.L:.2f}; exact target extents in {time.time() - t0:.1f} s")

    def strip(self, b: int, rings: bool = True) -> dict:
        """Strip b: source and target generator indices, their rings (optional)
        and the strip's candidate pairs (local indices, sorted by source)."""
        from farm_gb300 import polygons as P
        from farm_gb300 import shard
        s_idx = shard.strip_sources(self.src_c, b, self.n_strips, self.L)
        S = P.generate_indices(self.prm, self.seed, s_idx)
        ms = S.mbrs()
        t_idx = shard.strip_targets(ms, self.tgt_ext)
        T = P.generate_indices(self.prm, self.seed + 1, t_idx)
        pairs = P.mbr_join(ms, T.mbrs())
        d = {"strip": b, "s_idx": s_idx, "t_idx": t_idx, "pairs": pairs,
             "s_nv": np.diff(S.off.astype(np.int64)), "t_nv": np.diff(T.off.astype(np.int64)),
             "vertices": int(S.total + T.total)}
        if rings:
            d["S"], d["T"] = S, T
        return d


def filter_bytes(stats: dict, n_pairs: int, bits: int) -> float:
    """Algorithmic bytes of the filter+refine kernel for one launch: per pair 8
    (pair ids) + 2 x 64 (raster headers) + w/8 per source window pixel and per
    target pixel visited + 1/8 (result bit)."""
    return n_pairs * (8 + 128 + 0.125) + bits / 8.0 * (stats["src_window_pixels"] + stats["tgt_window_pixels"])


# Fallback denominators when the device's own rates cannot be measured:
# nominal issue rates, GB300 FP64 at 2 lanes/clock/SM and FP32 at 128, 152
# SMs at 2.07 GHz (no kernel here fuses, so one flop is one instruction).
FP64_NOMINAL = 2 * 152 * 2.07e9
FP32_NOMINAL = 128 * 152 * 2.07e9

# DRAM traffic per unit of the kernels that can be the dominant one, from one
# ncu capture on a small configuration-2 strip (dram__bytes_read.sum +
# dram__bytes_write.sum summed over the launches, divided by the units they
# processed); the capture command and the figures are in
# profiles/dram_traffic_small_strip.md. A step's traffic is the per-unit
# figure times the step's units.
TRAFFIC_PER_UNIT = {
    "edge_walk": 199.0,   # bytes per edge (k_walk_tot + k_walk_fill): 42.6 GB / 2.14e8 edges
    "refine": 6621.8,     # bytes per candidate pair (k_intersect): 174.3 MB / 26,320 pairs
}


def measured_peaks() -> dict:
    """HBM from MEASURED_PEAKS.json; FP64 and FP32 measured now on this GPU
    (farm_probe_issue_rates), else nominal."""
    out = {}
    try:
        pk = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        out["hbm"], out["hbm_src"] = float(pk["hbm_gbs"]) * 1e9, "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except Exception:
        out["hbm"], out["hbm_src"] = 6.8e12, "fallback 6.8 TB/s (of fallback)"
    try:
        from farm_gb300.engine import issue_rates
        r = max((issue_rates() for _ in range(2)), key=lambda d: d["fp64_ops_per_s"])
        out["fp64"], out["fp32"] = r["fp64_ops_per_s"], r["fp32_ops_per_s"]
        out["fp_src"] = "measured on this GPU by farm_probe_issue_rates (non-fused multiply/add chains; of measured)"
    except Exception as e:
        out["fp64"], out["fp32"] = FP64_NOMINAL, FP32_NOMINAL
        out["fp_src"] = f"nominal issue rate (measurement failed: {e})"
    return out


def rooflines(rt: dict, qs: dict, n_pairs: float, stage: dict, steps: int, peaks: dict,
              ref_tests: float | None) -> dict:
    """Roofline of each measured stage from its algorithmic work per unit
    (work summed over the timed steps; times are per-step means).

    edge walk (k_walk_tot + k_walk_fill): FP64, 16 flops per edge (endpoint
      cells, slope and intercept) + 16 per pixel-boundary crossing (both
      branches of one walk step), the reference's arithmetic for ONE walk;
    cell clip (count + emit): FP64, 4 flops per emitted clip point;
    column clip: FP64, 2 flops per emitted point;
    cell areas: FP64, 4 flops per clip point (shoelace term + accumulation);
    filter + refine (k_intersect): FP32, 28 flops per segment-pair test in the
      reference's order with its early exit (counted by the oracle on the
      parity sample and scaled to the step; the GPU's own test count is
      reported beside it); its HBM bytes per filter_bytes();
    whole raster stage, HBM view: 8 B per vertex read + the raster written
      (w P / 8 + 4 (P + n) + 8 sequences + 8 nodes).
    The whole path: sum over the two stages of max(bytes / HBM, flops64 /
    FP64, flops32 / FP32), over the measured step time.
    """
    hbm, p64, p32 = peaks["hbm"], peaks["fp64"], peaks["fp32"]
    per = lambda k: stage[k] / steps
    st = {}

    def fp(name, flops, ms, peak, kind):
        ach = flops / (ms * 1e-3) if ms > 0 else None
        st[name] = {"bound": kind, "algorithmic_flops_per_step": flops, "kernel_ms": ms,
                    "achieved": ach / 1e12 if ach else None, "peak": peak / 1e12, "unit": "TFLOP/s",
                    "frac": ach / peak if ach else None, "peak_source": peaks["fp_src"]}

    f_walk = (16.0 * rt["vertices"] + 16.0 * rt["crossings"]) / steps
    f_clipy = 4.0 * rt["clip_y_points"] / steps
    f_clipx = 2.0 * rt["clip_x_points"] / steps
    f_cells = 4.0 * rt["clip_y_points"] / steps
    fp("edge_walk", f_walk, rt["ms_walk"] / steps, p64, "fp64")
    fp("cell_clip", f_clipy, rt["ms_clip_y"] / steps, p64, "fp64")
    fp("column_clip", f_clipx, rt["ms_clip_x"] / steps, p64, "fp64")
    fp("cell_area", f_cells, rt["ms_cells"] / steps, p64, "fp64")
    gpu_tests = qs["segment_tests"] / steps
    tests = ref_tests / steps if ref_tests else gpu_tests
    fp("refine", 28.0 * tests, per("query_ms"), p32, "fp32")
    st["refine"]["segment_tests_reference_order"] = tests if ref_tests else None
    st["refine"]["segment_tests_gpu"] = gpu_tests
    if ref_tests:
        st["refine"]["gpu_tests_over_reference_order"] = gpu_tests / tests
    fb = filter_bytes(qs, n_pairs, 4) / steps
    rb = (8.0 * rt["vertices"] + 0.5 * rt["pixels"] + 4.0 * (rt["pixels"] + rt["polygons"]) +
          8.0 * rt["sequences"] + 8.0 * (rt["hnodes"] + rt["vnodes"])) / steps
    rms, qms = per("raster_ms"), per("query_ms")
    st["raster_hbm_view"] = {"bound": "hbm", "algorithmic_bytes_per_step": rb, "kernel_ms": rms,
                             "achieved": rb / (rms * 1e-3) / 1e9 if rms > 0 else None, "peak": hbm / 1e9,
                             "unit": "GB/s", "frac": rb / (rms * 1e-3) / hbm if rms > 0 else None,
                             "peak_source": peaks["hbm_src"]}
    st["filter_hbm_view"] = {"bound": "hbm", "algorithmic_bytes_per_step": fb, "kernel_ms": qms,
                             "achieved": fb / (qms * 1e-3) / 1e9 if qms > 0 else None,
                             "peak": hbm / 1e9, "unit": "GB/s", "frac": fb / (qms * 1e-3) / hbm if qms > 0 else None,
                             "peak_source": peaks["hbm_src"]}
    raster_floor = max(rb / hbm, (f_walk + f_clipy + f_clipx + f_cells) / p64)
    query_floor = max(fb / hbm, 28.0 * tests / p32)
    step_s = per("step_ms") * 1e-3
    st["whole_path"] = {"roofline_ms": (raster_floor + query_floor) * 1e3, "step_ms": step_s * 1e3,
                        "frac": (raster_floor + query_floor) / step_s if step_s > 0 else None,
                        "stages": {"raster": {"roofline_ms": raster_floor * 1e3, "measured_ms": rms},
                                   "filter_refine": {"roofline_ms": query_floor * 1e3, "measured_ms": qms}},
                        "formula": "sum over stages of max(bytes/HBM, flops64/FP64, flops32/FP32) / step time"}
    # the dominant kernel: the stage with the most device time
    cand = {k: v for k, v in st.items() if k in ("edge_walk", "cell_clip", "column_clip", "cell_area", "refine")}
    name = max(cand, key=lambda k: cand[k]["kernel_ms"] or 0.0)
    dom = dict(cand[name])
    dom["kernel"] = {"edge_walk": "k_walk_tot + k_walk_fill", "cell_clip": "k_clipy (count + emit)",
                     "column_clip": "k_clipx (count + emit)", "cell_area": "k_cells",
                     "refine": "k_intersect (filter + refine)"}[name]
    units = {"edge_walk": rt["vertices"] / steps, "refine": n_pairs / steps}
    tpu = TRAFFIC_PER_UNIT.get(name)
    dom["traffic"] = tpu * units[name] if tpu and name in units else None
    dom["traffic_note"] = ("ncu dram bytes per unit on a 400-strip case x units per step "
                           "(profiles/dram_traffic_small_strip.md)" if dom["traffic"] else
                           "no ncu capture of this kernel's DRAM bytes")
    return {"dominant": dom, "stages": st}


# ------------------------------------------------------- learned scorer ----
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
    Jt = Job(args.seed + 1000, args.strips)
    sd = Jt.strip(0)
    S, T, pairs = sd["S"], sd["T"], sd["pairs"]
    store.load_sets(S, T)
    store.rasterize(vpr=args.vpr, category_count=16, strict=False)
    del S, T, sd
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
    del dp, lab, code, cost
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
    """Learned mode and the -a heuristic on one strip's pairs, against exact."""
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


# ------------------------------------------------------------ GPU arm ----
def workload_config(job: Job, args, strips: list, n_pairs: int, vertices: int) -> dict:
    cfg = {"workload": "intersect, configuration 2: 100k sources x 1M targets, nv log-uniform 16..100000, "
                       f"~20M MBR candidates, -v {args.vpr}, -w 16 (category_count 16); the job is cut into "
                       f"{job.n_strips} strips by source centre, one step = one strip (sources centred in it + "
                       "every target reaching them), steps cycle through the rank's strips",
           "domain_side": job.L, "vpr": args.vpr, "category_count": 16, "n_source": N_SRC, "n_target": N_TGT,
           "strips": job.n_strips, "strips_timed": strips, "candidate_pairs_in_strips": n_pairs,
           "vertices_in_strips": vertices, "l2": "inputs larger than L2 (no flush needed)", "seed": args.seed}
    return cfg


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
    peaks = measured_peaks()
    store = Store()
    learned_train = train_scorer(args, store, dev) if args.learned else None
    mine = shard.strips_of_rank(rank, world, args.strips)
    if not mine:
        raise SystemExit(f"{world} ranks need at least {world} strips (--strips {args.strips})")
    job = Job(args.seed, args.strips)
    # the strips the warm-up and timed steps visit (all of this rank's once
    # K >= their count), resident in HBM: rings, offsets, pairs, results
    n_used = min(len(mine), max(args.steps, args.warmup, 1))
    strips = []
    t0 = time.time()
    for b in mine[:n_used]:
        sd = job.strip(b)
        S, T = sd.pop("S"), sd.pop("T")
        sd["so"], sd["to"] = S.off, T.off
        sd["d_so"] = torch.from_numpy(S.off.view(np.int64)).to(dev)
        sd["d_sx"] = torch.from_numpy(S.xy).to(dev)
        sd["d_to"] = torch.from_numpy(T.off.view(np.int64)).to(dev)
        sd["d_tx"] = torch.from_numpy(T.xy).to(dev)
        sd["d_pairs"] = torch.from_numpy(sd["pairs"].view(np.int32)).to(dev).view(len(sd["pairs"]), 2)
        sd["d_out"] = torch.empty(len(sd["pairs"]), dtype=torch.uint8, device=dev)
        sd["xy_bytes"] = (S.total + T.total) * 8
        del S, T
        strips.append(sd)
        log(f"strip {b}: {len(sd['s_idx'])} sources, {len(sd['t_idx'])} targets, {sd['vertices']} vertices, "
            f"{len(sd['pairs'])} candidates")
    log(f"{len(strips)} strips resident in HBM after {time.time() - t0:.1f} s")
    order = [strips[i % len(strips)] for i in range(max(args.steps, 1))]
    warm = [strips[i % len(strips)] for i in range(args.warmup)]

    stage = {"load_ms": 0.0, "raster_ms": 0.0, "query_ms": 0.0}
    rsum, qsum = {}, {}

    def acc(dst, src):
        for k, v in src.items():
            if isinstance(v, (int, float)):
                dst[k] = dst.get(k, 0) + v

    def step_device(sd, timed=False):
        store.event_record(4)
        store.load(0, sd["d_so"], sd["d_sx"])
        store.load(1, sd["d_to"], sd["d_tx"])
        store.event_record(5)
        store.rasterize(vpr=args.vpr, category_count=16, strict=False)
        load_ms = store.event_elapsed(4, 5)
        store.event_record(4)
        _, found = store.intersect(sd["d_pairs"], out=sd["d_out"])
        sd["raster_ms"] = store.event_elapsed(5, 4)
        sd["query_ms"] = store.last_stats["ms_total"]
        if timed:
            stage["load_ms"] += load_ms
            stage["raster_ms"] += sd["raster_ms"]
            stage["query_ms"] += sd["query_ms"]
            acc(rsum, store.raster_totals())
            acc(qsum, store.last_stats)
        sd["found"] = found
        return found

    for i, sd in enumerate(warm):
        t = time.time()
        step_device(sd)
        free, total = torch.cuda.mem_get_info(dev)
        log(f"warmup step {i} (strip {sd['strip']}): {time.time() - t:.2f}s, device memory in use "
            f"{(total - free) / 2**30:.1f} GiB, raster {store.raster_totals()}, stats {store.last_stats}")
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    launches0 = store.launches
    store.event_record(0)
    for sd in order:
        step_device(sd, timed=True)
    store.event_record(1)
    ms = store.event_elapsed(0, 1)
    torch.cuda.synchronize()
    launches = store.launches - launches0
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    stage["step_ms"] = ms
    t_dev = ms / 1000.0
    pairs_timed = sum(len(sd["pairs"]) for sd in order)

    # end to end through the C ABI with host buffers: each step's rings come
    # from pinned host memory, where they are placed before timing (one buffer
    # per distinct strip when a quarter of host memory holds them, else two
    # buffers, the next step's refilled from HBM during the current step), and
    # the result bytes go back to pinned host memory
    distinct = []
    for sd in order:
        if all(sd is not x for x in distinct):
            distinct.append(sd)
    host_bytes = os.sysconf("SC_PHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    resident = sum(sd["xy_bytes"] for sd in distinct) <= host_bytes // 4
    nbuf = len(distinct) if resident else 2
    # a source and a target buffer each (each allocation starts aligned, which
    # the copy engines need for full speed)
    caps = max(sd["d_sx"].numel() for sd in strips), max(sd["d_tx"].numel() for sd in strips)
    hbuf = [tuple(torch.empty(c, dtype=torch.float32).pin_memory() for c in caps) for _ in range(nbuf)]
    nmax = max(len(sd["pairs"]) for sd in strips)
    hout = torch.empty(nmax, dtype=torch.uint8).pin_memory()
    hpairs_out = torch.empty((nmax, 2), dtype=torch.int32).pin_memory()
    d_e2e_out = torch.empty(nmax, dtype=torch.uint8, device=dev)
    side = torch.cuda.Stream(dev)

    def refill(buf, sd):
        ns, nt = sd["d_sx"].numel(), sd["d_tx"].numel()
        with torch.cuda.stream(side):
            buf[0][:ns].copy_(sd["d_sx"].view(-1), non_blocking=True)
            buf[1][:nt].copy_(sd["d_tx"].view(-1), non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(side)
        return ev

    phase = {"load": 0.0, "join": 0.0, "raster": 0.0, "query": 0.0, "out": 0.0}

    def step_e2e(sd, buf, timed=False):
        # rings in from pinned host memory, candidates by the GPU MBR join,
        # rasterize, filter + refine, and the pairs with their results out
        # (host wall time per phase: each phase ends in a synchronisation of
        # the store's stream, except the last, which is synchronised here)
        t = [time.perf_counter()]
        ns, nt = sd["d_sx"].numel(), sd["d_tx"].numel()
        store.load(0, sd["so"], buf[0][:ns].numpy().reshape(-1, 2))
        store.load(1, sd["to"], buf[1][:nt].numpy().reshape(-1, 2))
        t.append(time.perf_counter())
        dp = store.mbr_join(device=dev, cap=nmax)
        t.append(time.perf_counter())
        store.rasterize(vpr=args.vpr, category_count=16, strict=False)
        t.append(time.perf_counter())
        n = dp.shape[0]
        _, found = store.intersect(dp, out=d_e2e_out[:n])
        t.append(time.perf_counter())
        hout[:n].copy_(d_e2e_out[:n], non_blocking=True)
        hpairs_out[:n].copy_(dp, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        t.append(time.perf_counter())
        if timed:
            for k, name in enumerate(("load", "join", "raster", "query", "out")):
                phase[name] += (t[k + 1] - t[k]) * 1000.0
        return found, n

    def buf_of(i, sd):
        return hbuf[next(k for k, x in enumerate(distinct) if x is sd)] if resident else hbuf[i % 2]

    # warm-up of the host path once over every strip the timed steps use (the
    # store's buffers reach their size before timing, and the GPU join is
    # checked against the host join on each strip)
    for k, sd in enumerate(distinct):
        b = hbuf[k] if resident else hbuf[0]
        refill(b, sd).synchronize()
        _, n0 = step_e2e(sd, b)
        # the GPU join's candidates are the host join's, in its order
        if n0 != len(sd["pairs"]) or not np.array_equal(hpairs_out[:n0].numpy().view(np.uint32), sd["pairs"]):
            raise SystemExit("the GPU MBR join differs from the host join")
    if not resident:
        refill(hbuf[0], order[0]).synchronize()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    store.event_record(2)
    t_e2e0 = time.perf_counter()
    for i, sd in enumerate(order):
        ev = None
        if not resident and i + 1 < len(order):
            ev = refill(hbuf[(i + 1) % 2], order[i + 1])
        step_e2e(sd, buf_of(i, sd), timed=True)
        if ev is not None:
            ev.synchronize()
    store.event_record(3)
    ms_e2e = store.event_elapsed(2, 3)
    wall_e2e = time.perf_counter() - t_e2e0
    t_e2e = max(ms_e2e / 1000.0, wall_e2e)
    if world > 1:
        dist.barrier()
    t_dev, t_e2e, total_pairs = shard.reduce_job(t_dev, t_e2e, pairs_timed, device=dev)
    value = total_pairs / t_dev
    e2e_value = total_pairs / t_e2e
    h2d = int(sum(sd["xy_bytes"] + 8 * (len(sd["so"]) + len(sd["to"])) for sd in order)
              / len(order))
    d2h = int(sum(9 * len(sd["pairs"]) for sd in order) / len(order))
    del hbuf
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (seeded star polygons, configuration 2 generator)",
        "config": workload_config(job, args, [sd["strip"] for sd in order], pairs_timed,
                                  sum(sd["vertices"] for sd in order)),
        "found_in_timed_steps": int(sum(sd.get("found", 0) for sd in order)),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": "per step: rings H2D from pinned host memory, the candidate pairs by the GPU MBR join (the "
                        "host join's set and order, checked once per strip in the warm-up), rasterization, filter + refine, and the pairs "
                        "with their result bytes D2H; the rings are placed in pinned host memory before timing "
                        "(one buffer per strip), or, when they do not fit a quarter of host memory, the next "
                        "step's buffer is refilled from HBM during the step (inside the timed region)",
                "host_buffers": "per strip" if resident else "two, refilled",
                "phase_wall_ms_per_step": {k: v / len(order) for k, v in phase.items()}},
        "gpu_launches": int(launches),
        "clocks": clk,
        "stage_ms": {"load": stage["load_ms"] / args.steps, "raster": stage["raster_ms"] / args.steps,
                     "filter_refine": stage["query_ms"] / args.steps, "step": ms / args.steps},
        "peaks": {"hbm_gbs": peaks["hbm"] / 1e9, "fp64_tops": peaks["fp64"] / 1e12, "fp32_tops": peaks["fp32"] / 1e12,
                  "fp_source": peaks["fp_src"]},
    }
    # learned mode on the first strip (rasterized again, outside the timed region)
    sd0 = strips[0]
    step_device(sd0)
    heavy = None
    if rank == 0:
        code, cost = store.filter_costs(sd0["d_pairs"])
        heavy = heavy_pairs(cost.cpu().numpy(), args.seed)
    if learned_train is not None and rank == 0:
        lr_ = learned_eval(store, sd0["d_pairs"], sd0["d_out"], sd0["query_ms"], sd0["raster_ms"], reps=3)
        lr_["strip"] = sd0["strip"]
        lr_["train"] = learned_train
        lr_["note"] = ("query = stages b-c on one rasterized strip (learned: predict + band + exact refinement of "
                       "abstentions); step adds the strip's rasterization, which both modes need")
        result["learned"] = lr_
    ref_tests = None
    if rank == 0 and not args.no_cpu_baseline:
        gpu_out = {sd["strip"]: sd["d_out"].cpu().numpy() for sd in strips}
        cb = cpu_baseline(job, strips, args, threads=os.cpu_count() or 1, gpu_out=gpu_out,
                          heavy=(sd0["strip"], heavy))
        # reference-order segment tests per pair (the oracle's count, early exit) scaled to the timed steps
        if cb.get("ref_tests_per_pair"):
            ref_tests = cb["ref_tests_per_pair"] * pairs_timed
        result["cpu_baseline"] = cb
    rl = rooflines(rsum, qsum, pairs_timed, stage, args.steps, peaks, ref_tests)
    result["roofline"] = rl["dominant"]
    result["stages"] = rl["stages"]
    store.close()
    del strips
    torch.cuda.empty_cache()
    if rank == 0 and args.within_strips > 0:
        result["within"] = within_eval(args)
    if rank == 0 and args.area_pairs > 0:
        result["area"] = area_eval(args)
    if world > 1:
        dist.destroy_process_group()
    return result if rank == 0 else None


def heavy_pairs(cost: np.ndarray, seed: int, frac: float = 0.01, take: int = 100) -> np.ndarray:
    """`take` pairs drawn at random from the heaviest `frac` of a strip's pairs
    by the filter's refinement cost proxy (local pair indices)."""
    n = len(cost)
    top = np.argsort(-cost, kind="stable")[:max(int(frac * n), 1)]
    rng = np.random.default_rng(seed + 98)
    return np.sort(rng.permutation(top)[:take])


def area_eval(args) -> dict:
    """Intersection area (stage d) on a configuration-4 sample, through a captured area plan.

    Configuration 4 mixes tiny and huge polygons (vertex counts log-uniform
    8..200,000 on each side) in one launch. The sample draws two pools of
    polygons from the star generator and takes args.area_pairs of their
    MBR-overlapping pairs at random, in one batch: the autotuner first picks
    the per-bucket knobs on a subsample, then one CUDA-graph launch of the
    persistent work-stealing kernel per pass. value = pairs / device time
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
    # the autotuner picks both knobs per size bucket on a 30% subsample of the
    # batch (chunk: edges per work item; window: pixels above which an edge is
    # searched by the whole warp); the plan below is captured with its tables
    t_tune = time.time()
    tune_sel = np.sort(rng.permutation(len(pairs))[:max(1, (3 * len(pairs)) // 10)])
    tuned = {}
    if args.area_tune:
        chunk_tab, wide_tab = st.area_autotune(pairs[tune_sel], with_wide=True)
        tuned = {str(b): [int(chunk_tab[b]), int(wide_tab[b])] for b in range(32) if chunk_tab[b] > 0}
    tune_s = time.time() - t_tune
    log(f"area autotune: {tune_s:.1f} s on {len(tune_sel)} pairs, bucket -> [chunk, window] {tuned or 'defaults'}")
    # items per pair at the smallest chunk the autotuner may pick (8 edges)
    plan = st.area_plan(max_pairs=len(pairs), max_items=int(((es + 7) // 8 + (et + 7) // 8).sum()) + 64)
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
            "nonzero_areas": int((out > 0).sum()), "rasterize_s": ras_s,
            "autotune": {"ran": bool(args.area_tune), "sample_pairs": int(len(tune_sel)), "seconds": tune_s,
                         "bucket_to_chunk_window": tuned,
                         "note": "bucket = floor(log2(larger edge count)); chunk = edges per work item, "
                                 "window = candidate-window pixels above which the whole warp shares an edge"}}


# ------------------------------------------------- within (config 3) ----
# Configuration 3: 200,000 star polygons in a 5,000 km square, mean radius
# log-uniform 0.05..50 km, vertex count log-uniform 32..20,000, within 10 km,
# planar (no degree scaling), self-join, the reference's default -v 10 and
# the hierarchy within needs. Coordinates are in kilometres: in metres (up to
# 5e6) the reference's Box, which starts from low = 1e5 and high = -1e5
# (Box.h:6-12), would clamp every MBR to begin at 1e5, so the join would pair
# almost everything; kilometres keep the geometry and stay inside that range.
W_N, W_SIDE, W_DIST = 200_000, 5000.0, 10.0


def within_eval(args) -> dict:
    """Within-distance pairs/sec on one strip of configuration 3: the sources
    centred in strip b of args.within_strips, every polygon that can lie
    within the distance of them, and the self-join candidates (MBRs widened
    by the distance, each source against every other polygon). One pass is
    one farm_within_mode call on device pairs, timed with CUDA events (median
    of three after a warm-up); a CPU oracle sample checks the results and
    gives the CPU rate on all host cores."""
    import torch
    from farm_gb300 import polygons as P
    from farm_gb300 import shard
    from farm_gb300.engine import Store

    t0 = time.time()
    prm = P.StarParams(dom_lo=0.0, dom_hi=W_SIDE, r_lo=0.05, r_hi=50.0, n_lo=32, n_hi=20_000, sigma=0.3)
    seed = args.seed + 300
    cen = P.centres(prm, seed, W_N)
    ext = shard.target_extents(cen, P.radii(prm, seed, W_N))
    nb = args.within_strips
    b = nb // 2
    s_idx = shard.strip_sources(cen, b, nb, W_SIDE)
    S = P.generate_indices(prm, seed, s_idx)
    ms = S.mbrs()
    lo, hi = ms[:, 0].min() - W_DIST, ms[:, 2].max() + W_DIST
    u_idx = np.nonzero((ext[:, 1] >= lo) & (ext[:, 0] <= hi))[0].astype(np.uint64)
    U = P.generate_indices(prm, seed, u_idx)
    mu = U.mbrs()
    src_pos = np.searchsorted(u_idx, s_idx)
    loc = P.mbr_join(mu[src_pos], mu, expand=W_DIST, geography=False)
    keep = src_pos[loc[:, 0]] != loc[:, 1]  # no polygon with itself
    pairs = np.ascontiguousarray(np.stack([src_pos[loc[keep, 0]], loc[keep, 1]], 1).astype(np.uint32))
    dev = torch.device("cuda", torch.cuda.current_device())
    st = Store()
    st.load(0, U.off, U.xy)
    st.rasterize(vpr=10, hierarchy=True, strict=False)
    ras_ms = st.raster_totals()["ms_total"]
    dp = torch.from_numpy(pairs.view(np.int32)).to(dev).view(len(pairs), 2)
    out = torch.empty(len(pairs), dtype=torch.uint8, device=dev)
    st.within(dp, distance=W_DIST, geography=False, self_join=True, out=out)  # warm-up
    ms, stats = [], {}
    for _ in range(3):
        torch.cuda.synchronize()
        st.event_record(4)
        st.within(dp, distance=W_DIST, geography=False, self_join=True, out=out)
        st.event_record(5)
        ms.append(st.event_elapsed(4, 5))
        stats = dict(st.last_stats)
    med = float(np.median(ms))
    gpu = out.cpu().numpy()
    st.close()
    log(f"within: strip {b}/{nb} of configuration 3: {len(s_idx)} sources, {len(u_idx)} polygons, {len(pairs)} "
        f"pairs, {med:.1f} ms per pass, {int((gpu == 1).sum())} within, {time.time() - t0:.1f} s wall")
    res = {"metric": "within-distance pairs/sec, configuration 3 strip", "value": len(pairs) / (med * 1e-3),
           "unit": "pairs/s", "ms_per_pass": med, "passes": 3, "warmup_passes": 1, "dtype": "f32+f64",
           "rasterize_ms": ras_ms,
           "config": {"workload": f"configuration 3 in km: {W_N} star polygons in a {W_SIDE:g} km square, radius "
                                  "0.05..50 km, nv log-uniform 32..20,000, within 10 km, planar, self-join, -v 10 "
                                  f"with the hierarchy; strip {b} of {nb} by source centre", "sources": int(len(s_idx)),
                      "polygons_loaded": int(len(u_idx)), "pairs": int(len(pairs)),
                      "vertices_loaded": int(U.total), "seed": seed},
           "found": int((gpu == 1).sum()), "sequence_pairs": stats.get("sequence_pairs"),
           "fp64_rechecks": stats.get("fp64_rechecks"),
           "fp64_recheck_frac": (stats.get("fp64_rechecks", 0) / stats["sequence_pairs"])
           if stats.get("sequence_pairs") else None,
           "stage_ms": {"descent": stats.get("ms_stage", [0, 0, 0, 0])[1],
                        "order_and_refine": stats.get("ms_stage", [0, 0, 0, 0])[2]}}
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = within_cpu(U, pairs, gpu, args)
    return res


def within_cpu(U, pairs, gpu: np.ndarray, args) -> dict:
    """The CPU oracle's within on all host cores over a cluster sample of the
    strip's pairs (all pairs of uniformly drawn sources), its rasterization
    phase from a systematic sample of the loaded polygons by size; also the
    parity check of the GPU's results on the sample."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(args.seed + 301)
    srcs = rng.permutation(np.unique(pairs[:, 0]))
    sel, got = [], 0
    for s_ in srcs:
        lo_, hi_ = np.searchsorted(pairs[:, 0], s_, "left"), np.searchsorted(pairs[:, 0], s_, "right")
        sel.append(np.arange(lo_, hi_))
        got += hi_ - lo_
        if got >= args.within_parity_pairs:
            break
    sel = np.concatenate(sel)
    polys = np.unique(pairs[sel].ravel())
    rings = [U.ring(int(k)) for k in polys]
    ras, _, prep_wall = timed_rasters(rings, 10, threads, hierarchy=True)
    R = {int(k): r for k, r in zip(polys, ras)}
    res = np.zeros(len(sel), np.uint8)
    chunks = [(a, min(a + 8, len(sel))) for a in range(0, len(sel), 8)]

    def run(ab):
        for k in range(*ab):
            s_, t_ = (int(v) for v in pairs[sel[k]])
            a, b_ = R[s_], R[t_]
            res[k] = 2 if a is None or b_ is None else int(O.within(a, b_, distance=W_DIST, geography=False))

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(run, chunks))
    q_wall = time.perf_counter() - t0
    # raster phase of the strip: systematic sample of the loaded polygons by size
    nv = np.diff(U.off.astype(np.int64))
    order = np.argsort(nv, kind="stable")
    k = max(len(order) // 300, 1)
    samp = order[int(rng.integers(k))::k]
    _, secs, _ = timed_rasters([U.ring(int(j)) for j in samp], 10, threads, hierarchy=True)
    raster_s = k * sum(secs) / threads
    query_s = q_wall * len(pairs) / len(sel)
    bad = int((gpu[sel] != res).sum())
    return {"value": len(pairs) / (raster_s + query_s), "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"query: {len(sel)} pairs of uniformly drawn sources (all their candidates), {q_wall:.2f} s "
                      f"wall on {threads} threads, scaled to the strip's {len(pairs)} pairs; raster: {len(samp)} "
                      f"polygons (systematic by size) x{k}",
            "raster_s": raster_s, "query_s": query_s, "parity_sample_pairs": int(len(sel)),
            "parity_sample_mismatches": bad, "prep_s": prep_wall}


# ------------------------------------------------------- CPU baseline ----
# The CPU side runs the oracle (a C port of the reference's algorithm) on
# threads: ctypes releases the GIL, so T threads use T cores at once.
class CpuSample:
    """Bounded samples of the job for the CPU oracle.

    * raster sample: a systematic sample of the strips' polygons (sources and
      targets of every strip, a target counted once per strip that holds it,
      as the job rasterizes it) in order of vertex count, so every size class
      is represented; each sampled polygon stands for `k` polygons;
    * query sample: sources drawn uniformly at random from the strips, with
      all of their candidate pairs (a cluster sample of the pairs), until at
      least `min_pairs` pairs; plus optional extra pairs (the heavy stratum),
      which are checked for parity but not used in the rate.
    """

    def __init__(self, job: Job, strips: list, seed: int):
        self.job, self.strips = job, strips
        self.rng = np.random.default_rng(seed + 99)
        # every (strip position, side, local index) with its vertex count
        self.poly = np.concatenate([
            np.stack([np.full(len(sd[key]), i), np.full(len(sd[key]), side), np.arange(len(sd[key])), sd[key]], 1)
            for i, sd in enumerate(strips) for side, key in ((0, "s_nv"), (1, "t_nv"))]).astype(np.int64)
        self.poly_sorted = self.poly[np.argsort(self.poly[:, 3], kind="stable")]
        self.n_pairs = sum(len(sd["pairs"]) for sd in strips)

    def raster_sample(self, n: int, offset_seed: int) -> tuple[np.ndarray, int]:
        N = len(self.poly_sorted)
        k = max(N // max(n, 1), 1)
        off = int(np.random.default_rng(offset_seed).integers(k))
        return self.poly_sorted[off::k], k

    def query_sample(self, min_pairs: int) -> np.ndarray:
        """(strip position, local pair index) of the cluster sample."""
        srcs = [(i, s) for i, sd in enumerate(self.strips) for s in range(len(sd["s_idx"]))]
        order = self.rng.permutation(len(srcs))
        out = []
        got = 0
        for o in order:
            i, s = srcs[o]
            pr_ = self.strips[i]["pairs"]
            lo, hi = np.searchsorted(pr_[:, 0], s, "left"), np.searchsorted(pr_[:, 0], s, "right")
            if hi > lo:
                out.append(np.stack([np.full(hi - lo, i), np.arange(lo, hi)], 1))
                got += hi - lo
            if got >= min_pairs:
                break
        return np.concatenate(out).astype(np.int64) if out else np.zeros((0, 2), np.int64)

    def rings(self, entries) -> list:
        """Rings (float32 [nv, 2]) of (strip position, side, local index) entries."""
        from farm_gb300 import polygons as P
        out = [None] * len(entries)
        for side, seed in ((0, self.job.seed), (1, self.job.seed + 1)):
            sel = [j for j, e in enumerate(entries) if e[1] == side]
            if not sel:
                continue
            key = "s_idx" if side == 0 else "t_idx"
            gids = np.array([self.strips[entries[j][0]][key][entries[j][2]] for j in sel], np.uint64)
            ps = P.generate_indices(self.job.prm, seed, gids)
            for m, j in enumerate(sel):
                out[j] = ps.ring(m)
        return out


def timed_rasters(rings: list, vpr: int, threads: int, hierarchy: bool = False) -> tuple[list, list, float]:
    """Oracle rasters of the rings on `threads` threads, largest first: the
    rasters (None where the reference fails), each polygon's own seconds
    (measured while all threads run), and the wall time."""
    from oracle import oracle as O
    O.lib()
    order = sorted(range(len(rings)), key=lambda j: -len(rings[j]))
    res, secs = [None] * len(rings), [0.0] * len(rings)

    def one(j):
        t = time.perf_counter()
        try:
            r = O.Raster(rings[j], vpr, hierarchy)
        except RuntimeError:
            r = None
        return j, r, time.perf_counter() - t

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for j, r, s in ex.map(one, order):
            res[j], secs[j] = r, s
    return res, secs, time.perf_counter() - t0


def timed_queries(rs: dict, rt: dict, keys: list, threads: int) -> tuple[np.ndarray, np.ndarray, float]:
    """Oracle intersect of (source key, target key) pairs over prebuilt rasters
    on `threads` threads (dynamic chunks of 8 pairs): results (2 where a
    raster is None), reference-order segment tests per pair, wall time."""
    from oracle import oracle as O
    n = len(keys)
    res = np.zeros(n, np.uint8)
    tests = np.zeros(n, np.uint64)
    chunks = [(a, min(a + 8, n)) for a in range(0, n, 8)]

    def run(ab):
        for k in range(*ab):
            a, b = rs[keys[k][0]], rt[keys[k][1]]
            if a is None or b is None:
                res[k] = 2
                continue
            v, c = O.intersect(a, b, counters=True)
            res[k], tests[k] = int(v), c.segment_tests

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(run, chunks))
    return res, tests, time.perf_counter() - t0


class CpuRunner:
    """Prepares the query sample's rasters once (untimed), then times steps of
    the CPU path: a raster phase on a fresh systematic polygon sample and the
    query phase on the prepared pairs."""

    def __init__(self, job: Job, strips: list, args, threads: int, min_pairs: int, heavy=None):
        self.args, self.threads = args, threads
        self.cs = CpuSample(job, strips, args.seed)
        self.strips = strips
        q = self.cs.query_sample(min_pairs)
        extra = np.zeros((0, 2), np.int64)
        if heavy is not None and heavy[1] is not None:
            pos = [i for i, sd in enumerate(strips) if sd["strip"] == heavy[0]]
            if pos:
                extra = np.stack([np.full(len(heavy[1]), pos[0]), heavy[1]], 1).astype(np.int64)
        self.q_uniform, self.q_heavy = q, extra
        allq = np.concatenate([q, extra])
        self.allq = allq
        # distinct polygons of the sampled pairs
        skeys = sorted({(int(i), 0, int(strips[i]["pairs"][p, 0])) for i, p in allq})
        tkeys = sorted({(int(i), 1, int(strips[i]["pairs"][p, 1])) for i, p in allq})
        t0 = time.perf_counter()
        rings = self.cs.rings(skeys + tkeys)
        ras, secs, wall = timed_rasters(rings, args.vpr, threads)
        self.prep_s = time.perf_counter() - t0
        self.rs = {k: ras[j] for j, k in enumerate(skeys)}
        self.rt = {k: ras[len(skeys) + j] for j, k in enumerate(tkeys)}
        self.keys = [((int(i), 0, int(strips[i]["pairs"][p, 0])), (int(i), 1, int(strips[i]["pairs"][p, 1])))
                     for i, p in allq]
        self.n_prep_polys = len(rings)
        log(f"CPU sample: {len(q)} cluster-sampled pairs + {len(extra)} heavy pairs, {len(rings)} polygons "
            f"rasterized in {self.prep_s:.1f} s on {threads} threads")

    def step(self, raster_polys: int, step_seed: int, query: bool = True) -> dict:
        cs = self.cs
        out = {}
        if raster_polys > 0:
            ent, k = cs.raster_sample(raster_polys, step_seed)
            rings = cs.rings([tuple(e[:3]) for e in ent])
            _, secs, wall = timed_rasters(rings, self.args.vpr, self.threads)
            # the job's raster phase: the sample's per-polygon seconds scaled by
            # k, spread evenly over the threads (132k+ polygons per strip keep
            # every thread busy); per-polygon seconds were measured with all
            # threads running, so shared-resource contention is included
            out["raster_s"] = k * sum(secs) / self.threads
            out["raster_sample"] = {"polygons": len(ent), "k": k, "vertices": int(ent[:, 3].sum()),
                                    "cpu_s": sum(secs), "wall_s": wall}
        if query:
            nq = len(self.q_uniform)
            res, tests, wall = timed_queries(self.rs, self.rt, self.keys[:nq], self.threads)
            out["query_s"] = wall * cs.n_pairs / max(nq, 1)
            out["query_sample"] = {"pairs": nq, "wall_s": wall}
            out["res"], out["tests"] = res, tests
        return out


def cpu_baseline(job: Job, strips: list, args, threads: int, gpu_out: dict, heavy=None) -> dict:
    """All-core CPU oracle over bounded samples of the rank's strips, and the
    full-scale parity check of the GPU's results on the query sample plus
    the heavy stratum."""
    run = CpuRunner(job, strips, args, threads, args.parity_pairs, heavy)
    st = run.step(args.raster_sample, args.seed + 500)
    # parity: the uniform sample's results come from the timed step; the heavy
    # stratum is queried here
    nq = len(run.q_uniform)
    hres, htests, _ = timed_queries(run.rs, run.rt, run.keys[nq:], threads) if len(run.q_heavy) else \
        (np.zeros(0, np.uint8), np.zeros(0, np.uint64), 0.0)
    exp = np.concatenate([st["res"], hres])
    got = np.array([gpu_out[strips[i]["strip"]][p] for i, p in run.allq], np.uint8)
    bad = int((got != exp).sum())
    value = run.cs.n_pairs / (st["raster_s"] + st["query_s"])
    ok = st["res"] != 2
    tpp = float(st["tests"][ok].astype(np.float64).mean()) if ok.any() else None
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"raster phase: {st['raster_sample']['polygons']} polygons (systematic sample by vertex "
                       f"count of the {len(run.cs.poly)} polygon rasterizations of the timed strips), "
                       f"{st['raster_sample']['cpu_s']:.1f} thread-seconds over {threads} threads, scaled x "
                       f"{st['raster_sample']['k']:.0f}; query phase: {nq} pairs of uniformly drawn sources "
                       f"(all their candidates), {st['query_sample']['wall_s']:.2f} s wall on {threads} threads, "
                       f"scaled to the strips' {run.cs.n_pairs} pairs"),
            "raster_s_per_job": st["raster_s"], "query_s_per_job": st["query_s"],
            "pairs_in_job": run.cs.n_pairs,
            "parity_sample_pairs": int(len(exp)), "parity_sample_mismatches": bad,
            "parity_heavy_pairs": int(len(run.q_heavy)),
            "parity_heavy_rule": "100 pairs drawn at random from the heaviest 1% of one strip's pairs by the "
                                 "filter's refinement cost proxy",
            "ref_tests_per_pair": tpp, "prep_s": run.prep_s}


def run_reference(args) -> dict:
    """The reference's CPU algorithm (the oracle port, all host cores) on the
    same job: every step times a fresh raster-phase sample and the query
    sample; value is the median over the timed steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    from farm_gb300 import shard
    world = int(os.environ.get("WORLD_SIZE", "1"))
    job = Job(args.seed, args.strips)
    mine = shard.strips_of_rank(0, 1, args.strips)
    order_strips = [mine[i % len(mine)] for i in range(max(args.steps, 1))]
    strips = [job.strip(b, rings=False) for b in sorted(set(order_strips))]
    by_strip = {sd["strip"]: sd for sd in strips}
    pairs_timed = sum(len(by_strip[b]["pairs"]) for b in order_strips)
    threads = os.cpu_count() or 1
    run = CpuRunner(job, strips, args, threads, args.parity_pairs)
    for i in range(args.warmup):
        run.step(0, args.seed + 600 + i)
    vals, steps = [], []
    t0 = time.perf_counter()
    for i in range(args.steps):
        st = run.step(args.ref_raster_sample, args.seed + 700 + i)
        vals.append(run.cs.n_pairs / (st["raster_s"] + st["query_s"]))
        steps.append({k: v for k, v in st.items() if k not in ("res", "tests")})
        log(f"reference step {i}: {vals[-1]:.1f} pairs/s (raster {st['raster_s']:.0f} s, query "
            f"{st['query_s']:.0f} s per job)")
    wall = time.perf_counter() - t0
    v = statistics.median(vals)
    last = steps[-1]
    cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": (f"per step: {last['raster_sample']['polygons']} polygons (systematic sample by vertex count, "
                     f"x{last['raster_sample']['k']:.0f}) and {last['query_sample']['pairs']} cluster-sampled "
                     f"pairs, on {threads} threads; median of {args.steps} steps"),
          "raster_s_per_job": statistics.median(s["raster_s"] for s in steps),
          "query_s_per_job": statistics.median(s["query_s"] for s in steps)}
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1000 / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded star polygons, configuration 2 generator)", "impl": "reference",
            "config": workload_config(job, args, order_strips, pairs_timed,
                                      sum(by_strip[b]["vertices"] for b in order_strips)),
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
    ap.add_argument("--parity-pairs", type=int, default=2000,
                    help="pairs of the CPU query sample (cluster sample by source; also the parity sample)")
    ap.add_argument("--raster-sample", type=int, default=600,
                    help="polygons of the CPU raster-phase sample in the GPU arm's cpu_baseline")
    ap.add_argument("--ref-raster-sample", type=int, default=150,
                    help="polygons of the raster-phase sample per step of --impl reference")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--area-pairs", type=int, default=1000,
                    help="pairs of the configuration-4 area sample (0 = skip the area block)")
    ap.add_argument("--no-area-tune", dest="area_tune", action="store_false",
                    help="time the area block with the default knobs (skip the autotuner)")
    ap.add_argument("--within-strips", type=int, default=40,
                    help="configuration 3 is cut into this many strips and the middle one is timed (0 = skip)")
    ap.add_argument("--within-parity-pairs", type=int, default=1000)
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip training and evaluating the learned scorer")
    ap.add_argument("--learned-pairs", type=int, default=2_000_000, help="training + held-out pairs")
    ap.add_argument("--learned-epochs", type=int, default=12)
    ap.add_argument("--learned-band", choices=["cost", "plain"], default="cost",
                    help="cost-aware band (spend the error budget on expensive pairs) or a plain probability band")
    ap.add_argument("--learned-budget", type=float, default=1e-3,
                    help="false positives (negatives) allowed above (below) the band, per positive")
    args = ap.parse_args()
    res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
