"""The GPU MBR join gives the host join's candidate pairs, in the same
(source, target) order: the set the reference's R-tree search returns
(RTree.h:581-600, intersect_cpu.cpp:18-36), for intersect candidates, the
within query's widened boxes (planar and in degrees) and self-joins."""
import numpy as np
import pytest

from farm_gb300 import polygons as P
from farm_gb300.engine import Store

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [3, 4])
def test_gpu_join_matches_host_join(gpu_lib, seed):
    prm = P.StarParams(dom_hi=60.0, r_lo=0.05, r_hi=2.0, n_lo=16, n_hi=3000)
    S, T = P.generate(prm, seed, 700), P.generate(prm, seed + 50, 4000)
    want = P.mbr_join(S.mbrs(), T.mbrs())
    st = Store()
    st.load_sets(S, T)
    got = st.mbr_join()
    assert len(want) > 1000 and np.array_equal(got, want)
    import torch
    dev = st.mbr_join(device=torch.device("cuda"))
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), want)
    # too small a buffer is refused with the count
    from farm_gb300._native import FarmError
    with pytest.raises(FarmError, match="exceed"):
        st.mbr_join(cap=len(want) - 1)
    st.close()


@pytest.mark.parametrize("geography,expand,dom", [(False, 1.5, 60.0), (True, 10.0, 60.0), (True, 25.0, 80.0)])
def test_gpu_join_widened_self_join(gpu_lib, geography, expand, dom):
    prm = P.StarParams(dom_lo=-dom / 2, dom_hi=dom, r_lo=0.05, r_hi=1.0, n_lo=16, n_hi=800)
    S = P.generate(prm, 21, 2500)
    want = P.mbr_join(S.mbrs(), S.mbrs(), expand=expand, geography=geography, skip_same=True)
    st = Store()
    st.load(0, S.off, S.xy)
    got = st.mbr_join(expand=expand, geography=geography, self_join=True)
    assert len(want) > 500 and np.array_equal(got, want)
    st.close()
