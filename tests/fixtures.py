"""Access to the committed golden fixtures (tests/golden)."""
import gzip
import json
import tempfile
from pathlib import Path

from farm_gb300.polygons import read_dt
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def manifest() -> dict:
    return json.loads((GOLDEN / "manifest.json").read_text())


def _gunzip(name: str) -> str:
    data = gzip.open(GOLDEN / name, "rb").read()
    f = tempfile.NamedTemporaryFile(delete=False, suffix=".bin")
    f.write(data)
    f.close()
    return f.name


def raster_case(case: dict):
    ps = read_dt(str(GOLDEN / f"{case['name']}.dt"))
    ref = O.read_ref_rasters(_gunzip(f"{case['name']}.rast.bin.gz"))
    return ps, ref


def pair_case(case: dict):
    S = read_dt(str(GOLDEN / f"{case['name']}_S.dt"))
    T = S if case["self_join"] else read_dt(str(GOLDEN / f"{case['name']}_T.dt"))
    ref = O.read_ref_pairs(_gunzip(f"{case['name']}.pairs.bin.gz"))
    return S, T, ref


def point_case(case: dict):
    """A contain-point fixture: the polygons, the points and the reference's
    (polygon, point, result) rows."""
    S = read_dt(str(GOLDEN / f"{case['name']}_S.dt"))
    pts = O.read_points(str(GOLDEN / f"{case['name']}_P.bin"))
    ref = O.read_ref_pairs(_gunzip(f"{case['name']}.pairs.bin.gz"))
    return S, pts, ref


RASTER_FIELDS = ["mbr", "dimx", "dimy", "step", "status", "offset", "seq", "hoff", "hnodes", "voff", "vnodes", "areas",
                 "num_layers"]


def raster_mismatches(a: dict, b: dict, fields=RASTER_FIELDS) -> list:
    import numpy as np
    bad = []
    for f in fields:
        x, y = a[f], b[f]
        if isinstance(x, np.ndarray) or isinstance(y, np.ndarray):
            x = np.asarray(x)
            y = np.asarray(y)
            if x.shape != y.shape or not np.array_equal(x, y):
                bad.append(f)
        elif x != y:
            bad.append(f)
    return bad
