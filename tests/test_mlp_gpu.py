"""Radiance-cache MLP on the tensor cores: operand-layout products, forward and gradients
against a numpy FP32 statement of the same network (the CPU oracle of the learned part)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_umma_operand_layouts(ctx, mode):
    """One tcgen05 product per operand arrangement equals the FP32 product of the bf16 inputs."""
    rng = np.random.default_rng(mode)
    shapes = {0: ((128, 64), (64, 64)), 1: ((128, 64), (64, 96)), 2: ((128, 96), (128, 64))}
    (ar, ac), (br, bc) = shapes[mode]
    a = to_bf16_bits(rng.standard_normal((ar, ac)).astype(np.float32))
    b = to_bf16_bits(rng.standard_normal((br, bc)).astype(np.float32))
    af, bf = from_bf16_bits(a).astype(np.float64), from_bf16_bits(b).astype(np.float64)
    want = {0: lambda: af @ bf.T, 1: lambda: af @ bf, 2: lambda: af.T @ bf}[mode]()
    res = {}
    for swap in (0, 1):
        d = np.zeros((128, 96 if mode == 1 else 64), np.float32)
        ctx.check(ctx.lib.lts_debug_umma_probe(ctx.h, mode, swap, a.ctypes.data_as(ctypes.c_void_p),
                                                b.ctypes.data_as(ctypes.c_void_p), d.ctypes.data_as(ctypes.c_void_p)))
        got = d[:want.shape[0]]
        res[swap] = np.max(np.abs(got - want)) / np.max(np.abs(want))
    print(f"mode {mode}: max rel err, offsets as documented {res[0]:.2e}, swapped {res[1]:.2e}")
    assert res[0] < 1e-5


def _batch(n, seed):
    from oracle import mlp_np
    rng = np.random.default_rng(seed)
    p = rng.random((n, 3), dtype=np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.standard_normal((n, 3)).astype(np.float32)
    nn /= np.linalg.norm(nn, axis=1, keepdims=True)
    feat = mlp_np.encode(p, d, nn, rng.random(n, dtype=np.float32), rng.random((n, 3), dtype=np.float32),
                         rng.random((n, 3), dtype=np.float32))
    # a smooth positive target of position and normal
    target = np.exp(0.5 * np.sin(3 * p[:, :1] + nn[:, 1:2]) + 0.3 * np.cos(2 * p[:, 1:2]) * np.array([1, 0.8, 0.6]))
    return feat, target.astype(np.float32)


@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_mlp_forward_matches_oracle(ctx, n):
    """Tensor-core inference equals the numpy network with the same bf16 rounding points."""
    import lighttransportsimulation_gb300 as lts
    from oracle import mlp_np
    mlp = lts.RadianceCacheMLP(ctx, seed=3)
    p = mlp_np.he_init(5)
    mlp.set_params(p)
    feat, _ = _batch(n, 1)
    got = mlp.forward(feat)
    want = mlp_np.forward(p, feat)
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-6)
    print(f"n={n}: forward max rel {rel.max():.2e}, median {np.median(rel):.2e}")
    assert np.median(rel) < 1e-4
    assert np.mean(rel < 1e-2) > 0.999


def test_mlp_gradients_match_oracle(ctx):
    """Gradient check: the tensor-core backward pass (input gradients and TMEM-accumulated weight
    gradients over persistent CTAs) against the numpy oracle, per layer."""
    import lighttransportsimulation_gb300 as lts
    from oracle import mlp_np
    mlp = lts.RadianceCacheMLP(ctx, seed=3)
    p = mlp_np.he_init(7)
    mlp.set_params(p)
    feat, target = _batch(5000, 2)
    loss, g = mlp.train_step(feat, target, lr=0.0, want_grad=True)
    loss_ref, g_ref = mlp_np.loss_and_grad(p, feat, target)
    print(f"loss {loss:.6f} oracle {loss_ref:.6f}")
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref)
    for L, (off, (o, i)) in enumerate(zip(mlp_np.OFFSETS, mlp_np.LAYERS)):
        a, b = g[off:off + o * i], g_ref[off:off + o * i]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        print(f"layer {L}: |dW| {np.linalg.norm(b):.3e}, rel err {rel:.2e}")
        assert rel < 1e-2


def test_mlp_learns(ctx):
    """Adam on the tensor-core gradients fits a smooth target: the relative L2 loss falls by more
    than 10x in 400 steps, and the fit holds on held-out samples."""
    import lighttransportsimulation_gb300 as lts
    mlp = lts.RadianceCacheMLP(ctx, seed=11)
    feat, target = _batch(16384, 3)
    losses = []
    for step in range(400):
        loss, _ = mlp.train_step(feat, target, lr=1e-2 if step < 300 else 3e-3)
        losses.append(loss)
    fh, th = _batch(4096, 4)
    pred = mlp.forward(fh)
    held = float(np.mean((pred - th) ** 2 / (pred ** 2 + 0.01)))
    print(f"loss {losses[0]:.4f} -> {losses[-1]:.5f}, held-out {held:.5f}")
    assert losses[-1] < losses[0] / 10
    assert held < 3 * losses[-1] + 1e-3


def test_device_pointer_entry_points_match_host_ones(ctx):
    """lts_mlp_forward_device_async / lts_mlp_train_step_device_async give the host entry points'
    outputs, loss and updated parameters on the same data."""
    import torch

    import lighttransportsimulation_gb300 as lts
    rng = np.random.default_rng(11)
    n = 3000
    feat = to_bf16_bits(rng.uniform(-1, 1, (n, 96)).astype(np.float32))
    targ = rng.uniform(0.01, 1.0, (n, 3)).astype(np.float32)
    net = lts.RadianceCacheMLP(ctx, seed=3)
    p0 = net.params()
    ref_out = net.forward(feat)
    ref_loss, _ = net.train_step(feat, targ, 1e-3)
    p_host = net.params()
    net.set_params(p0)  # same weights, fresh Adam state
    d_feat = torch.from_numpy(feat.view(np.int16)).cuda()
    d_targ = torch.from_numpy(targ).cuda()
    d_out = torch.empty((n, 3), device="cuda")
    d_loss = torch.zeros(1, device="cuda")
    torch.cuda.synchronize()
    net.forward_device_async(d_feat.data_ptr(), n, d_out.data_ptr())
    net.train_step_device_async(d_feat.data_ptr(), d_targ.data_ptr(), n, 1e-3, d_loss.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), ref_out)  # inference: no atomics, bit-exact
    # training sums the per-CTA gradients and losses with float atomics (order varies): the loss to
    # 1e-5; Adam's first step moves each weight by ~lr * sign(g), so weights agree to float
    # rounding except where a gradient is ~0 and its sign may differ (at most 2 lr apart)
    assert d_loss.item() == pytest.approx(ref_loss, rel=1e-5)
    p_dev = net.params()
    assert np.mean(np.abs(p_dev - p_host) <= 1e-6) >= 0.999
    assert np.max(np.abs(p_dev - p_host)) <= 2.1e-3
