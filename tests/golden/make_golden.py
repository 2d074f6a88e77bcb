"""Generate the golden fixtures from the reference's own CPU code.

Runs where the reference sources are present: it builds oracle/_ref (the
reference's unmodified CPU sources + the harness, see oracle/ref/Makefile),
generates seeded star polygons with the engine's generator, writes them as .dt
files, and records what the reference computes for them:

* ``<case>.rast.bin.gz`` — every polygon's raster (status, edge-sequence CSR,
  grid-line nodes, FP64 fill areas, hierarchy layers), dumped by
  ``ref_harness raster``;
* ``<case>.pairs.bin.gz`` — every MBR-candidate pair with the reference's
  decision, from ``ref_harness intersect|within``;
* ``degree_table.json`` — the reference's longitude degree table (util.h:73) as
  a SHA-256 of its printed values, which the regenerated table must match;
* ``<case>.pairs.bin.gz`` under the manifest's ``contain`` and
  ``contain_point`` keys — ``Ideal::contain`` of polygon pairs (large sources
  holding small targets) and of (polygon, point) pairs, with the points (float32,
  vertices and edge midpoints of the polygons among uniform ones) in
  ``<case>_P.bin``;
* ``wkt_cases.wkt`` / ``wkt_cases.dt`` — WKT lines covering the parser's rules
  (prefixes, holes, MULTIPOLYGON, spacing, exponents, many digits, an empty
  line, a large ring) and the .dt the reference's ``dump_polygons`` tool
  writes for them.

The .dt inputs are committed next to the outputs, so the tests never need the
reference or the generator's libm to reproduce them. Usage:

    python tests/golden/make_golden.py        # everything
    python tests/golden/make_golden.py wkt    # the WKT fixture only
    python tests/golden/make_golden.py contain  # the contain fixtures only
    python tests/golden/make_golden.py sweep    # the -v 128 / 256 fixtures only
"""
from __future__ import annotations

import gzip
import hashlib
import json
import re
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from farm_gb300 import build  # noqa: E402
from farm_gb300.polygons import StarParams, generate  # noqa: E402

REF_SRC = build.ref_src()

# (name, params, seed, count, vpr, hierarchy)
RASTER_CASES = [
    ("r_cfg1_v10", StarParams(dom_hi=20.0), 101, 80, 10, 0),
    ("r_cfg1_v4_h", StarParams(dom_hi=20.0), 102, 60, 4, 1),
    ("r_cfg1_v64", StarParams(dom_hi=20.0), 103, 60, 64, 0),
    ("r_small_v1", StarParams(dom_hi=5.0, r_lo=0.01, r_hi=0.5, n_lo=16, n_hi=200), 104, 60, 1, 1),
    # the bench's -v 64 on polygons of 2k-20k vertices (below the 65,536-sequence assert)
    ("r_big_v64", StarParams(dom_hi=30.0, n_lo=2000, n_hi=20000), 105, 10, 64, 0),
]
# configuration 2's -v sweep beyond 64 (128 and 256 vertices per pixel): its
# generator's polygons up to the size below the 65,536-sequence assert
SWEEP_RASTER_CASES = [
    ("r_big_v128", StarParams(dom_hi=30.0, n_lo=2000, n_hi=22000), 107, 10, 128, 0),
    ("r_big_v256", StarParams(dom_hi=30.0, n_lo=2000, n_hi=26000), 108, 10, 256, 0),
]
SWEEP_PAIR_CASES = [
    ("p_intersect_v128", StarParams(dom_hi=12.0, n_lo=16, n_hi=22000), 207, 24, 90, 128, "intersect"),
    ("p_intersect_v256", StarParams(dom_hi=12.0, n_lo=16, n_hi=26000), 208, 24, 90, 256, "intersect"),
]

# (name, params, seed, n_source, n_target (0 = self-join), vpr, mode)
PAIR_CASES = [
    ("p_intersect_v10", StarParams(dom_hi=20.0), 201, 60, 240, 10, "intersect"),
    ("p_intersect_v4", StarParams(dom_hi=20.0), 202, 50, 200, 4, "intersect"),
    ("p_within_v10", StarParams(dom_hi=20.0), 203, 260, 0, 10, "within"),
    ("p_within_v64", StarParams(dom_hi=30.0), 204, 260, 0, 64, "within"),
    # -v 64 with configuration 2's heavy tail, cut at 20k vertices
    ("p_intersect_v64_big", StarParams(dom_hi=12.0, n_lo=16, n_hi=20000), 205, 24, 90, 64, "intersect"),
    ("p_within_v64_big", StarParams(dom_hi=12.0, n_lo=16, n_hi=5000), 206, 100, 0, 64, "within"),
]

# (name, source params, target params, seed, n_source, n_target, vpr): large
# sources and small targets in one domain, so that containment occurs
_BIG = dict(dom_hi=20.0, r_lo=1.0, r_hi=3.0)
_SMALL = dict(dom_hi=20.0, r_lo=0.02, r_hi=0.6, n_lo=8)
CONTAIN_CASES = [
    ("k_contain_v10", StarParams(**_BIG, n_hi=2000), StarParams(**_SMALL, n_hi=400), 301, 40, 500, 10),
    ("k_contain_v4", StarParams(**_BIG, n_hi=1000), StarParams(**_SMALL, n_hi=200), 302, 30, 400, 4),
    ("k_contain_v64", StarParams(dom_hi=20.0, r_lo=2.0, r_hi=4.0, n_lo=2000, n_hi=20000),
     StarParams(dom_hi=20.0, r_lo=0.02, r_hi=0.4, n_lo=8, n_hi=1500), 303, 12, 200, 64),
]
# (name, params, seed, n_polygons, n_uniform_points, vpr)
CONTAIN_POINT_CASES = [
    ("q_point_v10", StarParams(dom_hi=20.0, r_lo=0.5, r_hi=3.0, n_hi=2000), 311, 40, 6000, 10),
    ("q_point_v64", StarParams(dom_hi=20.0, r_lo=0.5, r_hi=3.0, n_lo=2000, n_hi=20000), 312, 10, 6000, 64),
]


def contain_points(ps, seed: int, n_uniform: int, lo: float, hi: float):
    """Query points: uniform ones, every 7th vertex of each polygon, and the
    float32 midpoints of every 11th edge (points on or next to the boundary)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    pts = [rng.uniform(lo, hi, (n_uniform, 2)).astype(np.float32)]
    for k in range(ps.n):
        r = ps.ring(k).astype(np.float32)
        pts.append(r[::7])
        a, b = r[:-1:11].astype(np.float64), r[1::11].astype(np.float64)
        m = len(b)
        pts.append(((a[:m] + b) / 2).astype(np.float32))
    return np.ascontiguousarray(np.concatenate(pts), dtype=np.float32)


def write_points(path: Path, pts) -> None:
    import numpy as np
    with open(path, "wb") as f:
        f.write(np.uint64(len(pts)).tobytes())
        f.write(np.ascontiguousarray(pts, dtype=np.float32).tobytes())


def make_contain() -> None:
    harness = build.build_ref()
    if harness is None:
        raise SystemExit("reference sources not found (set FARM_REF_SRC to the reference's src/)")
    build.build_host()
    tmp = Path("/tmp/farm_golden")
    tmp.mkdir(exist_ok=True)
    mf = HERE / "manifest.json"
    manifest = json.loads(mf.read_text()) if mf.exists() else {}
    manifest["contain"], manifest["contain_point"] = [], []
    for name, sp, tp, seed, ns, nt, vpr in CONTAIN_CASES:
        S, T = generate(sp, seed, ns), generate(tp, seed + 5000, nt)
        sdt, tdt = HERE / f"{name}_S.dt", HERE / f"{name}_T.dt"
        S.write_dt(str(sdt))
        T.write_dt(str(tdt))
        out = tmp / f"{name}.pairs.bin"
        subprocess.run([str(harness), "contain", str(sdt), str(tdt), str(vpr), str(out)], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env={"FARM_REF_THREADS": "4"})
        gz(out, HERE / f"{name}.pairs.bin.gz")
        manifest["contain"].append({"name": name, "mode": "contain", "vpr": vpr, "seed": seed, "n_source": ns,
                                    "n_target": nt, "self_join": False, "params": sp.__dict__,
                                    "target_params": tp.__dict__})
    for name, prm, seed, n, npts, vpr in CONTAIN_POINT_CASES:
        S = generate(prm, seed, n)
        sdt = HERE / f"{name}_S.dt"
        S.write_dt(str(sdt))
        pts = contain_points(S, seed, npts, prm.dom_lo - 1.0, prm.dom_hi + 1.0)
        pbin = HERE / f"{name}_P.bin"
        write_points(pbin, pts)
        out = tmp / f"{name}.pairs.bin"
        subprocess.run([str(harness), "contain_point", str(sdt), str(pbin), str(vpr), str(out)], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env={"FARM_REF_THREADS": "4"})
        gz(out, HERE / f"{name}.pairs.bin.gz")
        manifest["contain_point"].append({"name": name, "vpr": vpr, "seed": seed, "n_source": n,
                                          "n_points": int(len(pts)), "params": prm.__dict__})
    mf.write_text(json.dumps(manifest, indent=1))
    print("wrote", len(CONTAIN_CASES), "contain and", len(CONTAIN_POINT_CASES), "contain-point fixtures")


def gz(src: Path, dst: Path) -> None:
    # mtime=0 keeps the fixture bytes reproducible
    with open(src, "rb") as f, open(dst, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9,
                                                                    mtime=0) as g:
        shutil.copyfileobj(f, g)


def sha(p: Path) -> str:
    return hashlib.sha256(p.read_bytes()).hexdigest()


def wkt_lines() -> list[str]:
    """WKT text for the dump_polygons fixture: one case per line."""
    import numpy as np
    rng = np.random.default_rng(9)
    lines = [
        "POLYGON((0 0, 4 0, 4 3, 0 3, 0 0))",
        "POLYGON ((10 10, 20 10, 20 20, 10 20, 10 10), (12 12, 12 14, 14 14, 14 12, 12 12))",
        "SRID=4326;POLYGON((-5.5 -5.5,-1.25 -5.5,-1.25 -1.125,-5.5 -1.125,-5.5 -5.5),"
        "(-5 -5,-5 -4,-4 -4,-4 -5,-5 -5), (-3 -3, -3 -2.5, -2.5 -2.5, -3 -3))",
        "MULTIPOLYGON(((30 30, 31 30, 31 31, 30 30)), ((40 40, 42 40, 42 42, 40 40)))",
        "POLYGON(( 1.5e-3 2.25e1 ,\t3.000000000000001 22.5 , 3 25.75 , 1.5e-3 2.25e1 ))",
        "",
        "POLYGON((0.1 0.2, 0.30000000000000004 0.2, 0.30000000000000004 0.7, 0.1 0.7, 0.1 0.2))",
        "polygon((-179.999999 -89.5, 179.999999 -89.5, 179.999999 89.5, -179.999999 89.5, -179.999999 -89.5))",
    ]
    # a large ring: a star of 3,000 vertices written with 17 significant digits
    n = 3000
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    rad = 5.0 * np.exp(rng.normal(0, 0.2, n))
    pts = [(50 + r * np.cos(a), 60 + r * np.sin(a)) for a, r in zip(ang, rad)]
    pts.append(pts[0])
    lines.append("POLYGON((" + ", ".join(f"{x:.17g} {y:.17g}" for x, y in pts) + "))")
    return lines


def make_wkt() -> None:
    exe = REF_SRC and build.build_ref() and (ROOT / "oracle" / "_ref" / "dump_polygons")
    if not exe or not exe.exists():
        raise SystemExit("reference sources not found (set FARM_REF_SRC to the reference's src/)")
    wkt = HERE / "wkt_cases.wkt"
    wkt.write_text("\n".join(wkt_lines()) + "\n")
    subprocess.run([str(exe), str(wkt), str(HERE / "wkt_cases.dt")], check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    mf = HERE / "manifest.json"
    manifest = json.loads(mf.read_text()) if mf.exists() else {}
    manifest["wkt"] = {"wkt": wkt.name, "dt": "wkt_cases.dt", "lines": len(wkt_lines()),
                       "dt_sha256": sha(HERE / "wkt_cases.dt")}
    mf.write_text(json.dumps(manifest, indent=1))
    print("wrote the WKT fixture")


def raster_fixture(harness: Path, tmp: Path, name, prm, seed, n, vpr, hier) -> dict:
    ps = generate(prm, seed, n)
    dt = HERE / f"{name}.dt"
    ps.write_dt(str(dt))
    out = tmp / f"{name}.rast.bin"
    subprocess.run([str(harness), "raster", str(dt), str(vpr), str(hier), str(out)], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env={"FARM_REF_THREADS": "4"})
    gz(out, HERE / f"{name}.rast.bin.gz")
    return {"name": name, "vpr": vpr, "hierarchy": hier, "seed": seed, "count": n, "params": prm.__dict__,
            "dt_sha256": sha(dt)}


def pair_fixture(harness: Path, tmp: Path, name, prm, seed, ns, nt, vpr, mode) -> dict:
    S = generate(prm, seed, ns)
    sdt = HERE / f"{name}_S.dt"
    S.write_dt(str(sdt))
    if nt:
        T = generate(prm, seed + 5000, nt)
        tdt = HERE / f"{name}_T.dt"
        T.write_dt(str(tdt))
        targ = str(tdt)
    else:
        targ = "-"
    out = tmp / f"{name}.pairs.bin"
    subprocess.run([str(harness), mode, str(sdt), targ, str(vpr), str(out)], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env={"FARM_REF_THREADS": "4"})
    gz(out, HERE / f"{name}.pairs.bin.gz")
    return {"name": name, "mode": mode, "vpr": vpr, "seed": seed, "n_source": ns, "n_target": nt,
            "self_join": nt == 0, "params": prm.__dict__}


def make_sweep() -> None:
    """The -v 128 and 256 cases alone, replacing their manifest entries."""
    harness = build.build_ref()
    if harness is None:
        raise SystemExit("reference sources not found (set FARM_REF_SRC to the reference's src/)")
    build.build_host()
    tmp = Path("/tmp/farm_golden")
    tmp.mkdir(exist_ok=True)
    mf = HERE / "manifest.json"
    manifest = json.loads(mf.read_text())
    names = {c[0] for c in SWEEP_RASTER_CASES + SWEEP_PAIR_CASES}
    manifest["raster"] = [c for c in manifest["raster"] if c["name"] not in names]
    manifest["pairs"] = [c for c in manifest["pairs"] if c["name"] not in names]
    for case in SWEEP_RASTER_CASES:
        manifest["raster"].append(raster_fixture(harness, tmp, *case))
    for case in SWEEP_PAIR_CASES:
        manifest["pairs"].append(pair_fixture(harness, tmp, *case))
    mf.write_text(json.dumps(manifest, indent=1))
    print("wrote", len(SWEEP_RASTER_CASES), "raster and", len(SWEEP_PAIR_CASES), "pair fixtures of the -v sweep")


def main() -> None:
    harness = build.build_ref()
    if harness is None:
        raise SystemExit("reference sources not found (set FARM_REF_SRC to the reference's src/)")
    build.build_host()
    manifest = {"raster": [], "pairs": []}
    tmp = Path("/tmp/farm_golden")
    tmp.mkdir(exist_ok=True)
    for case in RASTER_CASES + SWEEP_RASTER_CASES:
        manifest["raster"].append(raster_fixture(harness, tmp, *case))
    for case in PAIR_CASES + SWEEP_PAIR_CASES:
        manifest["pairs"].append(pair_fixture(harness, tmp, *case))
    # the reference's longitude table, as printed in util.h
    util = (REF_SRC / "include" / "util.h").read_text()
    m = re.search(r"degree_per_kilometer_longitude_arr\[\] = \{([^}]*)\}", util)
    vals = [v.strip() for v in m.group(1).split(",")]
    manifest["degree_table"] = {"count": len(vals), "sha256_of_6_decimal_text": hashlib.sha256(
        ",".join(vals).encode()).hexdigest()}
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1))
    print("wrote", len(RASTER_CASES) + len(SWEEP_RASTER_CASES), "raster and",
          len(PAIR_CASES) + len(SWEEP_PAIR_CASES), "pair fixtures")
    make_wkt()
    make_contain()


if __name__ == "__main__":
    if sys.argv[1:] == ["wkt"]:
        make_wkt()
    elif sys.argv[1:] == ["contain"]:
        make_contain()
    elif sys.argv[1:] == ["sweep"]:
        make_sweep()
    else:
        main()
