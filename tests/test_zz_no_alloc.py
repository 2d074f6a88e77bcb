"""farm_intersect_static: the allocation-free intersect entry point.

Some callers cannot allocate device memory when they query: their device
memory belongs to another allocator (a framework's caching allocator holding
the HBM), or they must not trigger the device-wide synchronisation of a
cudaMalloc while other streams run. farm_intersect_static serves them from a
fixed device array compiled into the library (at most 1,048,576 pairs per
call). This test calls it through the C ABI on a freshly rasterized store,
before farm_intersect has ever grown the store's query buffers, and checks
that two calls in a row allocate nothing in the store and give exactly what
farm_intersect gives (results are bytes: exact equality). It also checks that
a pair list over the limit, and a pair index out of range, are rejected.

The file sorts last so a failure here cannot hide any other test's outcome.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_static_intersect_matches_farm_intersect_twice(gpu_lib):
    from farm_gb300 import polygons as P
    from farm_gb300.engine import Store

    prm = P.StarParams(dom_hi=20.0, n_hi=1200)
    S, T = P.generate(prm, 31, 120), P.generate(prm, 32, 400)
    pairs = np.ascontiguousarray(P.mbr_join(S.mbrs(), T.mbrs()), dtype=np.uint32)
    assert len(pairs) > 100
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=10)
    lib = gpu_lib
    held = st.device_bytes()
    launches = st.launches
    results = []
    for _ in range(2):
        got = np.full(len(pairs), 0xEE, dtype=np.uint8)
        found = C.c_uint64(0)
        rc = lib.farm_intersect_static(st._h, C.c_void_p(pairs.ctypes.data), len(pairs),
                                       C.c_void_p(got.ctypes.data), C.byref(found))
        assert rc == 0, lib.farm_last_error().decode()
        results.append((got, found.value))
        # the static path grew none of the store's buffers
        assert st.device_bytes() == held
    assert st.launches == launches + 2
    want, want_found = st.intersect(pairs)
    for got, f in results:
        assert np.array_equal(got, want)
        assert f == want_found
    # farm_intersect does allocate its staging buffers (so the check above can see growth)
    assert st.device_bytes() > held
    # over the limit: rejected before any device work
    big = np.zeros(((1 << 20) + 1, 2), dtype=np.uint32)
    out = np.zeros(len(big), dtype=np.uint8)
    rc = lib.farm_intersect_static(st._h, C.c_void_p(big.ctypes.data), len(big), C.c_void_p(out.ctypes.data), None)
    assert rc == -1 and b"exceed" in lib.farm_last_error()
    # a target index past the target side: rejected on the host, no launch
    bad = pairs[:8].copy()
    bad[3, 1] = T.n
    launches = st.launches
    rc = lib.farm_intersect_static(st._h, C.c_void_p(bad.ctypes.data), len(bad), C.c_void_p(out.ctypes.data), None)
    assert rc == -1 and b"out of range" in lib.farm_last_error()
    assert st.launches == launches
    st.close()
