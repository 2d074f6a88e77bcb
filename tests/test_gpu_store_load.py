"""farm_store_load from the three places rings can live: pageable host memory
(staged through a device buffer), pinned host memory (read by the padding
kernel over the host link, no staging copy) and device memory. The store must
hold the same rings each way: rasters and intersect results are compared
byte for byte."""
import numpy as np
import pytest

from farm_gb300 import polygons as P
from farm_gb300.engine import Store

pytestmark = pytest.mark.gpu


def test_store_load_pinned_pageable_and_device_agree(gpu_lib):
    import torch
    prm = P.StarParams(dom_hi=30.0, n_lo=16, n_hi=20000)
    S, T = P.generate(prm, 81, 300), P.generate(prm, 82, 900)
    pairs = np.ascontiguousarray(P.mbr_join(S.mbrs(), T.mbrs()), dtype=np.uint32)
    dev = torch.device("cuda:0")
    # pinned buffers with a leading pad, so the rings start inside the allocation
    pinned = []
    for X in (S, T):
        buf = torch.zeros(X.xy.size + 6, dtype=torch.float32).pin_memory()
        buf[6:] = torch.from_numpy(X.xy.reshape(-1))
        pinned.append(buf[6:].numpy().reshape(-1, 2))
    results = []
    for how in ("pageable", "pinned", "device"):
        with Store() as st:
            if how == "pageable":
                st.load_sets(S, T)
            elif how == "pinned":
                st.load(0, S.off, pinned[0])
                st.load(1, T.off, pinned[1])
            else:
                st.load(0, torch.from_numpy(S.off.view(np.int64)).to(dev), torch.from_numpy(S.xy).to(dev))
                st.load(1, torch.from_numpy(T.off.view(np.int64)).to(dev), torch.from_numpy(T.xy).to(dev))
            st.rasterize(vpr=64, strict=False)
            rasters = [st.fetch_raster(side, k) for side, k in ((0, 0), (0, S.n - 1), (1, 3), (1, T.n - 1))]
            out, found = st.intersect(pairs)
            results.append((rasters, out, found))
    base = results[0]
    for rasters, out, found in results[1:]:
        for ra, rb in zip(base[0], rasters):
            for key in ("status", "offset", "seq", "vnodes", "hnodes", "areas"):
                assert np.array_equal(ra[key], rb[key]), key
        assert np.array_equal(base[1], out) and base[2] == found


def test_store_load_alignment(gpu_lib):
    """Vertices at a 4-byte (not 8-byte) boundary: pinned host ones go
    through the staging copy and load the same rings; device ones are
    refused before any device work."""
    import torch
    prm = P.StarParams(dom_hi=10.0, n_lo=16, n_hi=2000)
    S = P.generate(prm, 83, 40)
    buf = torch.zeros(S.xy.size + 1, dtype=torch.float32).pin_memory()
    buf[1:] = torch.from_numpy(S.xy.reshape(-1))
    odd = buf[1:].numpy().reshape(-1, 2)  # starts 4 bytes into the allocation
    assert odd.ctypes.data % 8 == 4
    with Store() as a, Store() as b:
        a.load(0, S.off, odd)
        b.load(0, S.off, S.xy)
        a.rasterize(vpr=10, strict=False)
        b.rasterize(vpr=10, strict=False)
        for k in (0, S.n - 1):
            ra, rb = a.fetch_raster(0, k), b.fetch_raster(0, k)
            for key in ("status", "offset", "seq", "vnodes", "areas"):
                assert np.array_equal(ra[key], rb[key]), key
    dev = torch.device("cuda:0")
    d = torch.zeros(S.xy.size + 1, dtype=torch.float32, device=dev)
    d[1:] = torch.from_numpy(S.xy.reshape(-1)).to(dev)
    with Store() as c:
        with pytest.raises(Exception, match="8-byte"):
            c.load(0, torch.from_numpy(S.off.view(np.int64)).to(dev), d[1:].view(-1, 2))
