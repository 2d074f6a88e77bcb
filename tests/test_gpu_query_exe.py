"""The drop-in query programs (intersect, within_polygon) print the reference's
count-found on the golden .dt fixtures."""
import re
import subprocess
from pathlib import Path

import pytest

from fixtures import GOLDEN, manifest, pair_case

pytestmark = pytest.mark.gpu
LIB = Path(__file__).resolve().parents[1] / "farm_gb300" / "lib"
M = manifest()


@pytest.fixture(scope="module", autouse=True)
def query_built(gpu_lib):
    from farm_gb300 import build
    build.build_query_exe()


def run(prog, *args):
    p = subprocess.run([str(LIB / prog), *args], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    m = re.search(r"count-found:\t(\d+)", p.stderr)
    assert m, p.stderr
    return int(m.group(1))


@pytest.mark.parametrize("case", M["pairs"], ids=[c["name"] for c in M["pairs"]])
def test_query_program_count_matches_reference(gpu_lib, case):
    _, _, ref = pair_case(case)
    expected = int((ref[:, 2] == 1).sum())
    s = str(GOLDEN / f"{case['name']}_S.dt")
    if case["mode"] == "intersect":
        got = run("intersect", "-s", s, "-t", str(GOLDEN / f"{case['name']}_T.dt"), "-r", "-g", "-v",
                  str(case["vpr"]))
    else:
        got = run("within_polygon", "-s", s, "-r", "-h", "-g", "-v", str(case["vpr"]))
    assert got == expected


def test_query_program_batches_add_up(gpu_lib):
    case = next(c for c in M["pairs"] if c["mode"] == "intersect")
    s, t = str(GOLDEN / f"{case['name']}_S.dt"), str(GOLDEN / f"{case['name']}_T.dt")
    whole = run("intersect", "-s", s, "-t", t, "-r", "-g", "-v", str(case["vpr"]))
    assert run("intersect", "-s", s, "-t", t, "-r", "-g", "-v", str(case["vpr"]), "-b", "37") == whole


def test_within_program_approximation(gpu_lib, tmp_path):
    # within_polygon -a counts the pairs the within -a rule accepts
    import numpy as np
    from farm_gb300 import polygons as P
    from oracle import oracle as O
    S = P.generate(P.StarParams(dom_hi=2.0, r_lo=0.005, r_hi=0.06, n_hi=1500), 45, 220)
    f = tmp_path / "s.dt"
    S.write_dt(str(f))
    pairs = P.mbr_join(S.mbrs(), S.mbrs(), expand=10.0, geography=True, skip_same=True)
    RS = O.rasterize_set(S, 10, True)
    expected = sum(O.within_heuristic(RS[s], RS[t]) for s, t in pairs)
    assert run("within_polygon", "-s", str(f), "-r", "-h", "-g", "-a", "-v", "10") == expected
    assert run("within_polygon", "-s", str(f), "-r", "-h", "-g", "-v", "10") == sum(
        O.within(RS[s], RS[t]) for s, t in pairs)
