"""Times the reference's own CPU program (oracle/_ref/intersect_cpu, compiled
from the reference's sources by this directory's Makefile) against the CPU
oracle port on the same polygons and the same number of threads.

The GPU machines that run the benchmark have neither the reference's sources
nor an x86 build of it, so the benchmark's CPU figures come from the port;
this script measures, on a machine that has the reference, how the port's
speed compares with the reference's for the two phases the reference logs
("preprocess finished": rasterization of every polygon; "query finished":
the per-pair decisions). Polygons follow the configuration-2 generator with
at most 20,000 vertices (the reference asserts on more edge sequences than
65,535 per polygon at -v 64 above that).

The two "found" counts differ by design: the stock program reads one vertex
past each ring for a single-pixel edge sequence (Ideal.cpp:523-529) and gets
whatever the allocator left there, while the port (and the harness the parity
fixtures come from) reads a copy of the first vertex. Only the times are the
comparison; parity is pinned by the harness.

  python oracle/ref/time_reference.py [--threads N] [--sources 150] [--targets 1500]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def phase_seconds(log: str, name: str) -> float:
    m = re.search(r"\t" + re.escape(name) + r" takes ([0-9.]+) (s|ms)", log)
    if not m:
        raise RuntimeError(f"no '{name}' in the reference's log:\n{log[-2000:]}")
    v = float(m.group(1))
    return v if m.group(2) == "s" else v / 1000.0


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--sources", type=int, default=150)
    ap.add_argument("--targets", type=int, default=1500)
    ap.add_argument("--vpr", type=int, default=64)
    ap.add_argument("--seed", type=int, default=77)
    args = ap.parse_args()
    exe = ROOT / "oracle" / "_ref" / "intersect_cpu"
    if not exe.exists():
        raise SystemExit(f"{exe} is not built (python -c 'import __graft_entry__ as g; g.build()')")
    import numpy as np
    from farm_gb300 import polygons as P
    from oracle import oracle as O

    # the configuration-2 generator, density kept as in configuration 2's job
    side = 419.17 * (args.sources / 100_000) ** 0.5
    prm = P.StarParams(dom_lo=0.0, dom_hi=side, r_lo=0.05, r_hi=2.0, n_lo=16, n_hi=20_000, sigma=0.3)
    S = P.generate(prm, args.seed, args.sources)
    T = P.generate(prm, args.seed + 1, args.targets)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    with tempfile.TemporaryDirectory() as tmp:
        s_dt, t_dt = os.path.join(tmp, "S.dt"), os.path.join(tmp, "T.dt")
        S.write_dt(s_dt)
        T.write_dt(t_dt)
        r = subprocess.run([str(exe), "-s", s_dt, "-t", t_dt, "-r", "-v", str(args.vpr), "-n", str(args.threads)],
                           stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:
            raise SystemExit(f"the reference failed ({r.returncode}):\n{r.stderr[-2000:]}")
        ref_pre, ref_query = phase_seconds(r.stderr, "preprocess finished"), phase_seconds(r.stderr, "query finished")
        m = re.search(r"count-found:\s*(\d+)", r.stdout + r.stderr)
        ref_found = int(m.group(1)) if m else None
    t0 = time.perf_counter()
    RS = O.rasterize_many([S.ring(k) for k in range(S.n)], args.vpr, threads=args.threads)
    RT = O.rasterize_many([T.ring(k) for k in range(T.n)], args.vpr, threads=args.threads)
    port_pre = time.perf_counter() - t0
    t0 = time.perf_counter()
    res = O.intersect_many(RS, RT, pairs, threads=args.threads)
    port_query = time.perf_counter() - t0
    out = {"threads": args.threads, "sources": S.n, "targets": T.n, "vertices": int(S.total + T.total),
           "pairs": int(len(pairs)), "vpr": args.vpr,
           "reference": {"preprocess_s": ref_pre, "query_s": ref_query, "found": ref_found},
           "port": {"preprocess_s": port_pre, "query_s": port_query, "found": int((res == 1).sum())},
           "port_over_reference_time": {"preprocess": port_pre / ref_pre, "query": port_query / ref_query}}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
