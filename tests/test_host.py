"""Host services: .dt I/O, generator determinism, MBR join, error paths."""
import numpy as np
import pytest

from farm_gb300 import polygons as P
from farm_gb300._native import FarmError


def test_dt_roundtrip_and_generator_determinism(host_built, tmp_path):
    prm = P.StarParams(dom_hi=10.0)
    a = P.generate(prm, 7, 50)
    b = P.generate(prm, 7, 50)
    assert np.array_equal(a.off, b.off) and np.array_equal(a.xy, b.xy)
    c = P.generate(prm, 7, 20, first=30)  # sub-ranges are independent
    assert np.array_equal(c.xy, a.subset(range(30, 50)).xy)
    for k in range(a.n):
        r = a.ring(k)
        assert (r[0] == r[-1]).all() and 16 <= len(r) - 1 <= 1024
    f = tmp_path / "a.dt"
    a.write_dt(str(f))
    r = P.read_dt(str(f))
    assert np.array_equal(r.off, a.off) and np.array_equal(r.xy, a.xy)


def test_mbr_join_matches_brute_force(host_built):
    prm = P.StarParams(dom_hi=15.0)
    S, T = P.generate(prm, 1, 120), P.generate(prm, 2, 300)
    ms, mt = S.mbrs(), T.mbrs()
    got = P.mbr_join(ms, mt)
    ov = ~((ms[:, None, 0] > mt[None, :, 2]) | (mt[None, :, 0] > ms[:, None, 2]) |
           (ms[:, None, 1] > mt[None, :, 3]) | (mt[None, :, 1] > ms[:, None, 3]))
    s, t = np.nonzero(ov)
    exp = np.stack([s, t], 1).astype(np.uint32)
    assert np.array_equal(got, exp)
    # self join without the diagonal
    g2 = P.mbr_join(ms, ms, skip_same=True)
    assert (g2[:, 0] != g2[:, 1]).all()


def test_corrupt_dt_is_an_error(host_built, tmp_path):
    f = tmp_path / "bad.dt"
    f.write_bytes(b"\x01\x02")
    with pytest.raises(FarmError):
        P.read_dt(str(f))
    a = P.generate(P.StarParams(), 3, 5)
    good = tmp_path / "g.dt"
    a.write_dt(str(good))
    data = bytearray(good.read_bytes())
    data[-8:] = (10 ** 9).to_bytes(8, "little")  # impossible polygon count
    f.write_bytes(bytes(data))
    with pytest.raises(FarmError):
        P.read_dt(str(f))
    with pytest.raises(FarmError):
        P.read_dt(str(tmp_path / "missing.dt"))
