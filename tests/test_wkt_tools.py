"""The data tools: WKT -> .dt (the reference's dump_polygons) and the
generator CLI. CPU only.

The fixture pair tests/golden/wkt_cases.{wkt,dt} was made by the reference's
own dump_polygons tool (tests/golden/make_golden.py); the engine's parser must
write the same bytes.
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from farm_gb300 import polygons as P

GOLDEN = Path(__file__).resolve().parent / "golden"
LIB = Path(__file__).resolve().parents[1] / "farm_gb300" / "lib"


@pytest.fixture(scope="module")
def tools(host_built):
    from farm_gb300 import build
    build.build_tools_exe()
    from farm_gb300 import _native
    return _native.host()


def wkt_to_dt(lib, src, dst):
    n = C.c_uint64(0)
    rc = lib.farm_wkt_to_dt(str(src).encode(), str(dst).encode(), C.byref(n))
    return rc, n.value


def test_wkt_to_dt_matches_reference_dump(tools, tmp_path):
    out = tmp_path / "w.dt"
    rc, n = wkt_to_dt(tools, GOLDEN / "wkt_cases.wkt", out)
    assert rc == 0, tools.farm_host_last_error()
    assert n == 8  # nine lines, one of them empty
    assert out.read_bytes() == (GOLDEN / "wkt_cases.dt").read_bytes()


def test_dump_polygons_cli_matches_reference_dump(tools, tmp_path):
    out = tmp_path / "c.dt"
    r = subprocess.run([str(LIB / "dump_polygons"), str(GOLDEN / "wkt_cases.wkt"), str(out)],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == (GOLDEN / "wkt_cases.dt").read_bytes()


def test_wkt_read_gives_the_boundaries(tools):
    n, tot = C.c_uint64(0), C.c_uint64(0)
    path = str(GOLDEN / "wkt_cases.wkt").encode()
    assert tools.farm_wkt_read(path, C.byref(n), C.byref(tot), None, None) == 0
    off = np.zeros(n.value + 1, np.uint64)
    xy = np.zeros(2 * tot.value, np.float32)
    assert tools.farm_wkt_read(path, C.byref(n), C.byref(tot), off.ctypes.data_as(C.POINTER(C.c_uint64)),
                               xy.ctypes.data_as(C.POINTER(C.c_float))) == 0
    ps = P.read_dt(str(GOLDEN / "wkt_cases.dt"))
    assert np.array_equal(off, ps.off)
    assert np.array_equal(xy.view(np.uint32), ps.xy.reshape(-1).view(np.uint32))
    # rules: the MULTIPOLYGON gives its first polygon, a hole is not a boundary,
    # the prefix before '(' is ignored, digits round to float32 through double
    r3 = xy[2 * off[3]: 2 * off[4]].reshape(-1, 2)
    assert r3.tolist() == [[30, 30], [31, 30], [31, 31], [30, 30]]
    r1 = xy[2 * off[1]: 2 * off[2]].reshape(-1, 2)
    assert r1[0].tolist() == [10, 10] and len(r1) == 5
    r4 = xy[2 * off[4]: 2 * off[5]].reshape(-1, 2)
    assert r4[1, 0] == np.float32(3.000000000000001) and r4[0, 0] == np.float32(1.5e-3)


@pytest.mark.parametrize("text", [
    "POLYGON EMPTY",                       # no '(' at all: the reference reads past the line
    "POLYGON((0 0, 1 0, 1 1, 0 0)",         # the closing parenthesis is missing
    "POLYGON((0 0, 1e+05 0, 1 1, 0 0))",   # 'e+' splits a number: one coordinate too many
    "POLYGON((0 0, 1 0, 1 1) x",           # a ring is fine but the polygon is not closed
])
def test_wkt_malformed_lines_are_format_errors(tools, tmp_path, text):
    src = tmp_path / "bad.wkt"
    src.write_text("POLYGON((0 0, 1 0, 1 1, 0 0))\n" + text + "\n")
    rc, _ = wkt_to_dt(tools, src, tmp_path / "bad.dt")
    assert rc == -7  # FARM_EFORMAT
    assert b"bad.wkt:2" in tools.farm_host_last_error()


def test_generate_polygons_cli(tools, tmp_path):
    prm = P.StarParams(dom_lo=0.0, dom_hi=30.0, r_lo=0.1, r_hi=1.5, n_lo=16, n_hi=400, sigma=0.3)
    out, wkt = tmp_path / "g.dt", tmp_path / "g.wkt"
    args = [str(LIB / "generate_polygons"), "-o", str(out), "--wkt", str(wkt), "-n", "40", "--seed", "17",
            "--first", "100", "--dom-lo", "0", "--dom-hi", "30", "--r-lo", "0.1", "--r-hi", "1.5",
            "--n-lo", "16", "--n-hi", "400", "--sigma", "0.3", "--threads", "2"]
    r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    # polygons 100..139 of seed 17 are those of the library's generator
    whole = P.generate(prm, 17, 140)
    got = P.read_dt(str(out))
    assert got.n == 40
    for k in range(40):
        assert np.array_equal(got.ring(k), whole.ring(100 + k))
    # the WKT it writes reads back to the same float32 vertices
    back = tmp_path / "back.dt"
    rc, n = wkt_to_dt(tools, wkt, back)
    assert rc == 0 and n == 40
    again = P.read_dt(str(back))
    assert np.array_equal(again.off, got.off) and np.array_equal(again.xy, got.xy)
