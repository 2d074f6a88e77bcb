"""The learned scorer's hand-written tcgen05 kernels."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,BN", [(128, 64, 64, 64), (256, 256, 576, 256), (384, 128, 256, 128),
                                      (256, 512, 192, 256), (128, 192, 128, 64)])
def test_tc_gemm_matches_fp32_reference(gpu_lib, M, N, K, BN):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    Cm = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    rc = gpu_lib.farm_tc_gemm_test(C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), C.c_void_p(Cm.data_ptr()),
                                   M, N, K, BN)
    assert rc == 0, gpu_lib.farm_last_error().decode()
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T  # plain fp32 reference of the same bf16 operands
    err = (Cm - ref).abs().max().item()
    assert err <= 1e-3 * max(1.0, ref.abs().max().item()), err


def _bf16(a):
    import torch
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).float().numpy().astype(np.float64)


def _gelu(x):
    from scipy.special import erf
    return 0.5 * x * (1 + erf(x / np.sqrt(2)))


def _gelu_grad(x):
    from scipy.special import erf
    return 0.5 * (1 + erf(x / np.sqrt(2))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


def test_mlp_gradients_match_fp64_cpu_reference(gpu_lib):
    """Forward + backward of the tcgen05 MLP against an FP64 CPU computation
    with the same bf16 rounding points (operands of every GEMM)."""
    import torch
    from farm_gb300 import polygons as P
    from farm_gb300.engine import Store

    st = Store()
    S = P.generate(P.StarParams(dom_hi=10.0), 1, 4)
    st.load_sets(S, S)
    st.rasterize(vpr=10)
    st.mlp_init(seed=3)
    rows, n = 256, 200
    g = torch.Generator(device="cuda").manual_seed(5)
    X = torch.rand(rows, 576, device="cuda", generator=g)
    X[:, 520:] = 0
    X = X.to(torch.bfloat16)
    y = (torch.rand(rows, device="cuda", generator=g) < 0.4).to(torch.uint8)
    loss, grad = st.mlp_grad(X, y, n)
    p = st.mlp_params().astype(np.float64)
    o = 0
    W1 = p[o:o + 256 * 576].reshape(256, 576); o += 256 * 576
    W2 = p[o:o + 256 * 256].reshape(256, 256); o += 256 * 256
    b1 = p[o:o + 256]; o += 256
    b2 = p[o:o + 256]; o += 256
    w3 = p[o:o + 256]; o += 256
    b3 = p[o]
    Xc = X.float().cpu().numpy().astype(np.float64)
    yc = y.cpu().numpy().astype(np.float64)
    W1b, W2b = _bf16(W1), _bf16(W2)
    z1 = Xc @ W1b.T + b1
    h1 = _bf16(_gelu(z1))
    z2 = h1 @ W2b.T + b2
    h2 = _bf16(_gelu(z2))
    logit = h2 @ w3 + b3
    pr = 1 / (1 + np.exp(-logit))
    m = np.arange(rows) < n
    ref_loss = np.mean((np.maximum(logit, 0) - logit * yc + np.log1p(np.exp(-np.abs(logit))))[m])
    dl = np.where(m, (pr - yc) / n, 0.0)
    dw3 = h2.T @ dl
    db3 = dl.sum()
    dz2 = dl[:, None] * w3[None, :] * _gelu_grad(z2)
    db2 = dz2.sum(0)
    dz2b = _bf16(dz2)
    dW2 = dz2b.T @ h1
    dz1 = (dz2b @ W2b) * _gelu_grad(z1)
    db1 = dz1.sum(0)
    dW1 = _bf16(dz1).T @ Xc
    ref = np.concatenate([dW1.ravel(), dW2.ravel(), db1, db2, dw3, [db3]])
    assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss))
    o = 0
    for name, size in [("W1", 256 * 576), ("W2", 256 * 256), ("b1", 256), ("b2", 256), ("w3", 256), ("b3", 1)]:
        a, b = grad[o:o + size].astype(np.float64), ref[o:o + size]
        o += size
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert rel < 1e-2, (name, rel)
    st.close()


def test_learned_mode_beats_the_reference_heuristic(gpu_lib):
    """Train the scorer on exact labels; on held-out pairs its decisions (no
    abstention) are more accurate than the reference's -a heuristic, and the
    learned mode with an abstain band returns exact results for every pair it
    refers to refinement."""
    import torch
    from farm_gb300 import polygons as P
    from farm_gb300.engine import MODE_LEARNED, Store
    from oracle import oracle as O

    prm = P.StarParams(dom_hi=60.0, n_hi=600)
    S, T = P.generate(prm, 71, 1500), P.generate(prm, 72, 6000)
    pairs = P.mbr_join(S.mbrs(), T.mbrs())
    st = Store()
    st.load_sets(S, T)
    st.rasterize(vpr=10)
    exact, _ = st.intersect(pairs)
    rng = np.random.default_rng(0)
    idx = rng.permutation(len(pairs))
    ntr = int(0.7 * len(pairs))
    tr, te = idx[:ntr], idx[ntr:]
    dp = torch.from_numpy(pairs[tr].view(np.int32)).cuda()
    dy = torch.from_numpy(exact[tr]).cuda()
    l0 = None
    st.mlp_init(seed=2)
    l1 = st.mlp_train(dp, dy, epochs=1, batch=1024, lr=2e-3)
    l2 = st.mlp_train(dp, dy, epochs=12, batch=1024, lr=2e-3)
    assert l2 < l1 < 0.7
    prob = st.mlp_predict(torch.from_numpy(pairs[te].view(np.int32)).cuda()).cpu().numpy()
    learned = (prob >= 0.5).astype(np.uint8)
    truth = exact[te]
    RS, RT = O.rasterize_set(S, 10), O.rasterize_set(T, 10)
    heur = np.array([O.intersect_heuristic(RS[s], RT[t]) for s, t in pairs[te]], np.uint8)
    acc_l = (learned == truth).mean()
    acc_h = (heur == truth).mean()
    assert acc_l > acc_h, (acc_l, acc_h)
    # learned mode with a band: the exact filter decides what it can, the
    # scorer decides its confident pairs among the rest, and the band's pairs
    # are refined exactly
    from farm_gb300.engine import MODE_FILTER
    dte = torch.from_numpy(np.ascontiguousarray(pairs[te]).view(np.int32)).cuda().view(-1, 2)
    code, _ = st.intersect(dte, mode=MODE_FILTER)
    code = code.cpu().numpy()
    assert set(np.unique(code)) <= {0, 1, 3}
    decided = code != 3
    assert np.array_equal(code[decided], truth[decided])
    st.mlp_band(0.05, 0.95)
    out, found = st.intersect(np.ascontiguousarray(pairs[te]), mode=MODE_LEARNED)
    refined = (code == 3) & (prob > 0.05) & (prob < 0.95)
    assert np.array_equal(out[decided], truth[decided])
    assert np.array_equal(out[refined], truth[refined])
    assert st.last_stats["fp64_rechecks"] == int(refined.sum())
    assert st.last_stats["border_pairs"] == int((code == 3).sum())
    # cost-aware band: a pair is also decided when min(p, 1 - p) <= lambda x
    # its refinement cost proxy; every other scored pair is refined
    code2, cost = st.filter_costs(dte)
    assert np.array_equal(code2.cpu().numpy(), code)
    cost = cost.cpu().numpy().astype(np.float32)
    p32 = prob.astype(np.float32)
    u = np.minimum(p32, np.float32(1) - p32)
    lam = np.float32(np.median(u[code == 3] / cost[code == 3]))
    st.mlp_band(0.05, 0.95, cost_lambda=float(lam))
    out2, _ = st.intersect(np.ascontiguousarray(pairs[te]), mode=MODE_LEARNED)
    cheap = u <= lam * cost
    refined2 = (code == 3) & (p32 > 0.05) & (p32 < 0.95) & ~cheap
    assert np.array_equal(out2[decided], truth[decided])
    assert np.array_equal(out2[refined2], truth[refined2])
    assert st.last_stats["fp64_rechecks"] == int(refined2.sum())
    assert refined2.sum() < refined.sum()
    st.close()
