"""Surrogate network kernels on the GPU against torch / float64 CPU references."""
import ctypes as C

import numpy as np
import pytest

from mcluminescence_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("epi", [0, 1, 2])
@pytest.mark.parametrize("M,N,K", [(64, 64, 32), (128, 256, 64), (256, 64, 4096)])
def test_gemm_nt_matches_torch(epi, M, N, K):
    import torch
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(M + N + K + epi)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    Cm = torch.empty(M, N, device="cuda")
    Y = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
    Yt = torch.zeros(N, M, dtype=torch.bfloat16, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = lib.mcl_gemm_nt(epi, M, N, K, p(A), K, p(B), K, p(bias), p(Cm), N, p(Y), N, p(Yt), M, s)
    assert rc == 0
    torch.cuda.synchronize()
    ref = A.float() @ B.float().t()
    if epi:
        ref = ref + bias
    torch.testing.assert_close(Cm, ref, rtol=1e-4, atol=1e-3 * K ** 0.5)
    if epi == 2:
        gy = torch.nn.functional.gelu(Cm).to(torch.bfloat16)
        assert torch.equal(Y, gy)
        assert torch.equal(Yt, gy.t().contiguous())


@pytest.mark.parametrize("path", ["fused", "tcgen05", "mma_sync"])
def test_gradients_match_float64_reference(path):
    """Forward, loss and every parameter gradient against a float64 autograd
    reference of the same network (bf16 weights, inputs and hidden
    activations): the fused whole-network kernel, the layer-by-layer tcgen05
    GEMMs and the mma.sync GEMMs."""
    import torch
    from mcluminescence_gb300 import surrogate as S
    m = S.SurrogateMLP(batch=256, seed=3)
    m.use_fused = path == "fused"
    m.use_tcgen05 = path != "mma_sync"
    rng = np.random.default_rng(0)
    x = S.standardize(S.sample_params(256, rng))
    y = rng.normal(-2.0, 0.5, (256, 200)).astype(np.float32)
    m.set_inputs(torch.tensor(x, dtype=torch.float32, device="cuda"))
    m.set_targets(torch.tensor(y, device="cuda"))
    out = m.forward().float().cpu().numpy()
    m.backward()
    torch.cuda.synchronize()
    m.check_errors()
    loss_ref, gW, gb, out_ref = S.reference_forward_backward(m, x, y)
    assert np.abs(out - out_ref).max() < 0.05 * np.abs(out_ref).max()
    loss_gpu = float(m.loss.item()) / (256 * 200)
    assert abs(loss_gpu - loss_ref) < 2e-2 * loss_ref
    for L, gw_ref, gb_ref in zip(m.layers, gW, gb):
        gw = L.gW.cpu().numpy()
        assert np.linalg.norm(gw - gw_ref) < 2e-2 * np.linalg.norm(gw_ref) + 1e-9
        gbg = L.gb.cpu().numpy()
        assert np.linalg.norm(gbg - gb_ref) < 2e-2 * np.linalg.norm(gb_ref) + 1e-9


def test_adam_matches_formula():
    import torch
    lib = _lib.load()
    rows, cols = 64, 96
    g = torch.Generator(device="cuda").manual_seed(1)
    p0 = torch.randn(rows, cols, device="cuda", generator=g)
    p = p0.clone()
    m1 = torch.zeros_like(p)
    m2 = torch.zeros_like(p)
    W = torch.zeros(rows, cols, dtype=torch.bfloat16, device="cuda")
    Wt = torch.zeros(cols, rows, dtype=torch.bfloat16, device="cuda")
    ref = torch.nn.Parameter(p0.clone())
    opt = torch.optim.Adam([ref], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: C.c_void_p(t.data_ptr())
    for step in range(1, 6):
        grad = torch.randn(rows, cols, device="cuda", generator=g)
        assert lib.mcl_adam(rows, cols, P(p), P(grad), P(m1), P(m2), C.c_float(1e-2), C.c_float(0.9),
                            C.c_float(0.999), C.c_float(1e-8), step, P(W), P(Wt), s) == 0
        ref.grad = grad.clone()
        opt.step()
    torch.cuda.synchronize()
    torch.testing.assert_close(p, ref.detach(), rtol=1e-5, atol=1e-6)
    assert torch.equal(W, p.to(torch.bfloat16))
    assert torch.equal(Wt, p.t().contiguous().to(torch.bfloat16))


def test_training_learns_monte_carlo_curves():
    """Trained on device-generated Monte Carlo curves, the network predicts
    held-out curves far better than the untrained network, with per-bin errors
    of the order of the Monte Carlo standard error."""
    from mcluminescence_gb300 import surrogate as S
    P, Ct = S.generate_dataset(60000, seed=11)
    Ph, Ch = S.generate_dataset(2000, seed=12, id0=10 ** 6)
    m = S.SurrogateMLP(batch=1024, seed=0)
    y_h = S.curve_to_target(Ch)
    before = float(np.mean((S.predict(m, Ph) - y_h) ** 2))
    hist = S.train(m, P, Ct, steps=1500, log_every=500)
    after = float(np.mean((S.predict(m, Ph) - y_h) ** 2))
    assert after < 0.1 * before, (before, after, hist)
    # linear domain: error against the MC realisation relative to its SE
    pred = S.target_to_curve(S.predict(m, Ph))
    big = Ch > 20
    ratio = np.sqrt(np.mean((pred[big] - Ch[big]) ** 2 / Ch[big]))
    assert ratio < 4.0, ratio


@pytest.mark.parametrize("epi", [0, 1, 2])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 256, 256), (4096, 64, 256), (256, 64, 4096)])
def test_gemm_tcgen05_matches_torch(epi, M, N, K):
    """The tcgen05 / tensor-memory GEMM against torch and against the mma.sync kernel."""
    import torch
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(7 * M + N + K + epi)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    outs = []
    for fn in ("mcl_gemm_nt_tc", "mcl_gemm_nt"):
        Cm = torch.full((M, N), float("nan"), device="cuda")
        Y = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
        Yt = torch.zeros(N, M, dtype=torch.bfloat16, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        p = lambda t: C.c_void_p(t.data_ptr())
        args = [epi, M, N, K, p(A), K, p(B), K, p(bias), p(Cm), N, p(Y), N, p(Yt), M]
        rc = getattr(lib, fn)(*args, p(err), s) if fn.endswith("_tc") else getattr(lib, fn)(*args, s)
        assert rc == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        outs.append((Cm, Y, Yt))
    ref = A.float() @ B.float().t()
    if epi:
        ref = ref + bias
    Cm, Y, Yt = outs[0]
    torch.testing.assert_close(Cm, ref, rtol=1e-4, atol=1e-3 * K ** 0.5)
    torch.testing.assert_close(Cm, outs[1][0], rtol=1e-4, atol=1e-3 * K ** 0.5)
    if epi == 2:
        assert torch.equal(Yt, Y.t().contiguous())
        assert (Y.float() - torch.nn.functional.gelu(Cm).to(torch.bfloat16).float()).abs().max() == 0


def _train_pass(m, x, y):
    import torch
    m.set_inputs(torch.tensor(x, dtype=torch.float32, device="cuda"))
    m.set_targets(torch.tensor(y, device="cuda"))
    out = m.forward().float().clone()
    m.backward()
    torch.cuda.synchronize()
    m.check_errors()
    return (out, float(m.loss.item()), [L.gW.clone() for L in m.layers], [L.gb.clone() for L in m.layers])


_FUSED_OUT = {}


@pytest.mark.parametrize("split", [0, 1, 2, 4])
def test_fused_step_matches_layer_by_layer(split):
    """At batch 4,096 (32 tiles; weight gradients split over 8-CTA clusters)
    the fused launch, with each tile on a cluster of 1, 2 or 4 CTAs (0: the
    library's pick), and the grouped weight-gradient launch give what the
    layer-by-layer tcgen05 kernels give: same GEMMs, same bf16 roundings, the
    sums in another order.  The forward outputs do not depend on the split."""
    import torch
    from mcluminescence_gb300 import surrogate as S
    B = 4096
    rng = np.random.default_rng(5)
    x = S.standardize(S.sample_params(B, rng))
    y = rng.normal(-2.0, 0.5, (B, 200)).astype(np.float32)
    fused = S.SurrogateMLP(batch=B, seed=7)
    fused.fused_split = split
    plain = S.SurrogateMLP(batch=B, seed=7)
    plain.use_fused = False
    a = _train_pass(fused, x, y)
    b = _train_pass(plain, x, y)
    torch.testing.assert_close(a[0], b[0], rtol=1e-3, atol=1e-3)
    assert abs(a[1] - b[1]) <= 1e-4 * abs(b[1])
    for ga, gb_ in zip(a[2] + a[3], b[2] + b[3]):
        assert float(torch.linalg.norm(ga - gb_)) <= 1e-3 * float(torch.linalg.norm(gb_)) + 1e-12
    first = _FUSED_OUT.setdefault("out", a[0])
    assert torch.equal(first, a[0])


@pytest.mark.parametrize("B,split", [(128, 4), (1152, 0), (1152, 2), (8192, 0)])
def test_fused_step_other_batches(B, split):
    """One tile, an odd number of tiles (9), and 64 tiles: the fused pass
    against the layer-by-layer kernels."""
    import torch
    from mcluminescence_gb300 import surrogate as S
    rng = np.random.default_rng(B)
    x = S.standardize(S.sample_params(B, rng))
    y = rng.normal(-2.0, 0.5, (B, 200)).astype(np.float32)
    fused = S.SurrogateMLP(batch=B, seed=3)
    fused.fused_split = split
    plain = S.SurrogateMLP(batch=B, seed=3)
    plain.use_fused = False
    a = _train_pass(fused, x, y)
    b = _train_pass(plain, x, y)
    torch.testing.assert_close(a[0], b[0], rtol=1e-3, atol=1e-3)
    assert abs(a[1] - b[1]) <= 1e-4 * abs(b[1])
    for ga, gb_ in zip(a[2] + a[3], b[2] + b[3]):
        assert float(torch.linalg.norm(ga - gb_)) <= 1e-3 * float(torch.linalg.norm(gb_)) + 1e-12


@pytest.mark.parametrize("split", [0, 1, 2, 4])
def test_fused_inference_matches_layer_by_layer(split):
    import torch
    from mcluminescence_gb300 import surrogate as S
    m = S.SurrogateMLP(batch=512, seed=9)
    inf_f = m.inference_copy(1024)
    inf_f.fused_split = split
    inf_p = m.inference_copy(1024)
    inf_p.use_fused = False
    p = torch.tensor(S.sample_params(1000, np.random.default_rng(2)), dtype=torch.float32, device="cuda")
    a, b = S.predict_t(inf_f, p), S.predict_t(inf_p, p)
    torch.cuda.synchronize()
    torch.testing.assert_close(a, b, rtol=1e-3, atol=1e-3)
