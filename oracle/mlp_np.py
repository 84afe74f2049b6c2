"""CPU oracle of the radiance-cache MLP (test infrastructure): numpy FP32/FP64 statement of the
network the tensor-core kernels run, with the same BF16 rounding points, so gradients and outputs
of lighttransportsimulation_gb300/csrc/mlp.cu can be checked element by element.

Network: features (96, bf16) -> 5 hidden layers of 64 with ReLU (activations rounded to bf16) ->
3 outputs through exp; no biases.  Loss: mean over samples and channels of
(pred - t)^2 / (pred^2 + 0.01), the denominator treated as a constant.  The output gradient and
the masked hidden gradients are rounded to bf16 where the kernels store them in shared memory.
"""
import numpy as np

N_IN, N_HID, N_OUT_PAD, N_OUT = 96, 64, 16, 3
LAYERS = [(64, 96), (64, 64), (64, 64), (64, 64), (64, 64), (16, 64)]  # (out, in)
OFFSETS = np.cumsum([0] + [o * i for o, i in LAYERS])[:-1]
N_PARAMS = int(sum(o * i for o, i in LAYERS))


def bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b).astype(np.uint32) << 16).view(np.float32)


def bf16(x):
    return from_bits(bf16_bits(x))


def unpack(params):
    params = np.asarray(params, np.float32)
    return [params[off:off + o * i].reshape(o, i) for off, (o, i) in zip(OFFSETS, LAYERS)]


def encode(p, d, n, rough, kd, ks):
    """Feature vector of shading points: 12-frequency sin/cos encoding of the position p (in the
    unit cube: scene bounds normalised), direction, normal, roughness, diffuse and specular albedo,
    a constant 1, zeros to 96.  Returns bf16 bit patterns (n x 96)."""
    p = np.asarray(p, np.float32)
    m = p.shape[0]
    f = np.zeros((m, N_IN), np.float32)
    freq = (np.float32(np.pi) * (2.0 ** np.arange(12))).astype(np.float32)
    arg = (p[:, :, None] * freq[None, None, :]).astype(np.float32)  # m x 3 x 12
    f[:, 0:36] = np.sin(arg).reshape(m, 36)
    f[:, 36:72] = np.cos(arg).reshape(m, 36)
    f[:, 72:75] = d
    f[:, 75:78] = n
    f[:, 78] = rough
    f[:, 79:82] = kd
    f[:, 82:85] = ks
    f[:, 85] = 1.0
    return bf16_bits(f)


def forward(params, feat_bits, keep=False):
    W = [bf16(w).astype(np.float64) for w in unpack(params)]
    h = from_bits(feat_bits).astype(np.float64)
    hs = [h]
    for L in range(5):
        h = bf16(np.maximum((h @ W[L].T).astype(np.float32), 0.0)).astype(np.float64)
        hs.append(h)
    z = (h @ W[5].T).astype(np.float32)
    pred = np.exp(z[:, :N_OUT])
    return (pred, hs, W) if keep else pred


def loss_and_grad(params, feat_bits, target):
    pred, hs, W = forward(params, feat_bits, keep=True)
    t = np.asarray(target, np.float32).reshape(-1, 3)
    n = t.shape[0]
    d = pred - t
    den = pred * pred + np.float32(0.01)
    loss = float(np.sum(d * d / den) / (3 * n))
    gz = np.zeros((n, N_OUT_PAD), np.float32)
    gz[:, :N_OUT] = 2.0 * d / den * pred * np.float32(1.0 / (3 * n))
    gz = bf16(gz).astype(np.float64)
    grads = [None] * 6
    grads[5] = gz.T @ hs[5]
    grads[5][N_OUT:] = 0.0
    gh = gz @ W[5]
    for L in range(4, -1, -1):
        ga = bf16((gh * (hs[L + 1] > 0)).astype(np.float32)).astype(np.float64)
        grads[L] = ga.T @ hs[L]
        if L > 0:
            gh = ga @ W[L]
    return loss, np.concatenate([g.reshape(-1) for g in grads]).astype(np.float32)


def he_init(seed):
    rng = np.random.default_rng(seed)
    out = []
    for L, (o, i) in enumerate(LAYERS):
        a = np.sqrt(6.0 / i) * (0.1 if L == 5 else 1.0)
        w = rng.uniform(-a, a, (o, i)).astype(np.float32)
        if L == 5:
            w[N_OUT:] = 0.0
        out.append(w.reshape(-1))
    return np.concatenate(out)
