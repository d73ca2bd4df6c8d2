"""The one-launch weight-gradient + Adam kernel (mcl_wgrad_adam) against the
grouped weight-gradient GEMM, torch, and the multi-tensor Adam (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fused_model(B=4096, seed=3):
    import torch
    from mcluminescence_gb300 import surrogate as S
    rng = np.random.default_rng(seed)
    m = S.SurrogateMLP(batch=B, seed=seed)
    x = torch.tensor(S.standardize(S.sample_params(B, rng)), dtype=torch.float32, device="cuda")
    y = torch.tensor(rng.normal(-2.0, 0.5, (B, 200)).astype(np.float32), device="cuda")
    # a few plain steps first, so that the Adam moments are not zero
    lr = torch.full((8,), 1e-3, device="cuda")
    base = torch.zeros(1, dtype=torch.int32, device="cuda")
    for j in range(3):
        m.fused_pass(x, y, target_ld=200)
        m.weight_grads()
        m.adam_step_dev(lr[j:].data_ptr(), base.data_ptr(), j + 1)
    m.fused_pass(x, y, target_ld=200)
    torch.cuda.synchronize()
    m.check_errors()
    return m, lr, base


def _state(m):
    out = []
    for L in m.layers:
        out += [L.W.clone(), L.mW.clone(), L.vW.clone(), L.Wb.clone(), L.Wt.clone(),
                L.b.clone(), L.mb.clone(), L.vb.clone()]
    return out


def _load(m, st):
    for i, L in enumerate(m.layers):
        for t, v in zip([L.W, L.mW, L.vW, L.Wb, L.Wt, L.b, L.mb, L.vb], st[8 * i:8 * i + 8]):
            t.copy_(v)


@pytest.mark.parametrize("B", [4096, 256, 8192])
def test_gradients_match_grouped_gemm_and_torch(B):
    import torch
    m, lr, base = _fused_model(B=B)
    m.weight_grads()
    torch.cuda.synchronize()
    ref = [L.gW.clone() for L in m.layers]
    m.wgrad_adam_dev(lr[3:].data_ptr(), base.data_ptr(), 4)
    torch.cuda.synchronize()
    m.check_errors()
    for l, L in enumerate(m.layers):
        Xt = m.Yt[l - 1] if l > 0 else m.x0t
        exact = m.dZt[l].float() @ Xt.float().t()
        scale = float(torch.linalg.norm(exact)) + 1e-30
        assert float(torch.linalg.norm(L.gW - exact)) <= 1e-5 * scale
        assert float(torch.linalg.norm(L.gW - ref[l])) <= 1e-5 * scale


def test_adam_matches_multi_tensor_adam_bit_for_bit():
    """Given the gradients it computed, the kernel's Adam step equals
    mcl_adam_multi_dev's on the same state: weights, moments, bf16 copies
    and the transposed copies, biases."""
    import torch
    m, lr, base = _fused_model(seed=4)
    before = _state(m)
    m.wgrad_adam_dev(lr[3:].data_ptr(), base.data_ptr(), 4)
    torch.cuda.synchronize()
    m.check_errors()
    after = _state(m)
    _load(m, before)                      # the gradients gW / gb stay
    m.adam_step_dev(lr[3:].data_ptr(), base.data_ptr(), 4)
    torch.cuda.synchronize()
    want = _state(m)
    for a, w in zip(after, want):
        assert torch.equal(a, w)
    assert any(not torch.equal(a, b) for a, b in zip(after, before))


def test_training_step_with_one_launch_update_matches_two_launch_update():
    """Graph-replayed training steps: the one-launch update and the grouped
    GEMM + multi-tensor Adam give the same losses to rounding."""
    from mcluminescence_gb300 import surrogate as S
    P, Cn = S.generate_dataset(20000, seed=5)
    a = S.SurrogateMLP(batch=4096, seed=2)
    b = S.SurrogateMLP(batch=4096, seed=2)
    b.use_wgrad_adam = False
    ha = S.train(a, P, Cn, steps=100, log_every=25, seed=1)
    hb = S.train(b, P, Cn, steps=100, log_every=25, seed=1)
    np.testing.assert_allclose(ha, hb, rtol=1e-2)
