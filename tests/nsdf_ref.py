"""NumPy forward pass of the learned collision proxy (tfx_nsdf): the same features, BF16 rounding
of inputs, weights and activations, and FP32 accumulation, for checking the tensor-core kernels."""
from __future__ import annotations

import numpy as np

KIN, HID, OUTN, NFEAT = 112, 64, 8, 102
P_W1 = 0
P_B1 = P_W1 + KIN * HID
P_W2 = P_B1 + HID
P_B2 = P_W2 + HID * HID
P_W3 = P_B2 + HID
P_B3 = P_W3 + HID * HID
P_W4 = P_B3 + HID
P_B4 = P_W4 + HID * HID
P_W5 = P_B4 + HID
P_B5 = P_W5 + HID * OUTN
NPARAM = P_B5 + OUTN
FREQ = (2.0 ** (np.arange(16) / 3.0)).astype(np.float32)


def bf16(x) -> np.ndarray:
    """Round float32 to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def frame(box_min, box_max, pose_scale):
    lo, hi = np.asarray(box_min, np.float32), np.asarray(box_max, np.float32)
    c = (np.float32(0.5) * (lo + hi)).astype(np.float32)
    ih = (np.float32(2.0) / (hi - lo)).astype(np.float32)
    return c, ih, np.float32(pose_scale)


def features(points: np.ndarray, pose, fr) -> np.ndarray:
    c, ih, ps = fr
    u = ((points.astype(np.float32) - c) * ih).astype(np.float32)
    f = np.zeros((len(points), KIN), np.float32)
    f[:, 0:3] = u
    f[:, 3:6] = np.asarray(pose, np.float32) * ps
    for k in range(16):
        arg = (FREQ[k] * u).astype(np.float64)
        f[:, 6 + 6 * k:6 + 6 * k + 6:2] = np.sin(np.pi * arg)
        f[:, 7 + 6 * k:7 + 6 * k + 6:2] = np.cos(np.pi * arg)
    return bf16(f)


def silu(z):
    """The kernels' activation: 0.5 z (1 + tanh(z / 2)) on bf16 values (h = bf16(z / 2), bf16(h t + h))."""
    h = bf16(np.float32(0.5) * z)
    t = bf16(np.tanh(h.astype(np.float64)).astype(np.float32))
    return bf16(h * t + h)


def forward(params: np.ndarray, feats: np.ndarray) -> np.ndarray:
    """Network output (cells) of every feature row."""
    p = params.astype(np.float32)
    W1 = bf16(p[P_W1:P_B1].reshape(KIN, HID))
    h = bf16(silu(feats @ W1 + p[P_B1:P_W2]))
    for w, b in ((P_W2, P_B2), (P_W3, P_B3)):
        h = bf16(silu(h @ bf16(p[w:w + HID * HID].reshape(HID, HID)) + p[b:b + HID]))
    h = bf16(silu(h @ bf16(p[P_W4:P_B4].reshape(HID, HID)) + p[P_B4:P_W5]))
    W5 = bf16(p[P_W5:P_B5].reshape(HID, OUTN))
    return (h @ W5[:, 0] + p[P_B5]).astype(np.float32)


# ------------------------------------------------------------------------------------------ training
def hash32(x: np.ndarray) -> np.ndarray:
    """lowbias32 (C. Wellons), the kernels' sample hash, on uint32 arrays."""
    x = np.asarray(x, dtype=np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def drawn_samples(seed: int, step: int, batch: int, pool_size: int) -> np.ndarray:
    """Indices of the pool samples training step `step` (1-based) uses: sample b of the batch is
    hash32(s ^ hash32(b * 2654435761)) scaled to the pool, s = seed * 2654435761 + step * 40503."""
    s = (seed * 2654435761 + step * 40503) & 0xFFFFFFFF
    b = np.arange(batch, dtype=np.uint64)
    h = hash32(np.uint64(s) ^ hash32((b * 2654435761) & 0xFFFFFFFF))
    return ((h * np.uint64(pool_size)) >> np.uint64(32)).astype(np.int64)


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z.astype(np.float64)))
    return (s * (1.0 + z * (1.0 - s))).astype(np.float32)


def train_gradients(params: np.ndarray, samples: np.ndarray, fr) -> tuple[np.ndarray, float]:
    """Loss sum and gradient (parameter layout) of one batch, as the training kernels form them: bf16
    features, weights and activations, fp32 pre-activations, loss = sum w (y - t)^2 / B, each layer's
    pre-activation gradient rounded to bf16 before it meets the weights and the activations."""
    p = params.astype(np.float32)
    B = len(samples)
    feats = np.stack([features(samples[i:i + 1, :3], samples[i, 4:7], fr)[0] for i in range(B)])
    Ws = [bf16(p[P_W1:P_B1].reshape(KIN, HID)), bf16(p[P_W2:P_B2].reshape(HID, HID)),
          bf16(p[P_W3:P_B3].reshape(HID, HID)), bf16(p[P_W4:P_B4].reshape(HID, HID))]
    bs = [p[P_B1:P_W2], p[P_B2:P_W3], p[P_B3:P_W4], p[P_B4:P_W5]]
    W5 = bf16(p[P_W5:P_B5].reshape(HID, OUTN))[:, 0]
    H, Z = [feats], []
    for W, b in zip(Ws, bs):
        z = (H[-1].astype(np.float64) @ W.astype(np.float64) + b).astype(np.float32)
        Z.append(z)
        H.append(bf16(silu(z)))
    y = (H[4].astype(np.float64) @ W5 + p[P_B5]).astype(np.float32)
    t, w = samples[:, 3], samples[:, 7]
    e = y - t
    loss = float((w * e * e).sum())
    dy = (2.0 * w * e / B).astype(np.float32)
    g = np.zeros(NPARAM, np.float32)
    dz5 = bf16(dy)
    g[P_W5:P_B5].reshape(HID, OUTN)[:, 0] = (H[4].astype(np.float64).T @ dz5).astype(np.float32)
    g[P_B5] = dz5.sum()
    d = (dy[:, None] * W5[None, :]).astype(np.float32) * silu_grad(Z[3])
    offs = [(P_W1, P_B1, P_W2), (P_W2, P_B2, P_W3), (P_W3, P_B3, P_W4), (P_W4, P_B4, P_W5)]
    for l in range(3, -1, -1):
        db = bf16(d)
        pw, pb, pe = offs[l]
        g[pw:pb] = (H[l].astype(np.float64).T @ db).reshape(-1).astype(np.float32)
        g[pb:pe] = db.sum(0)
        if l > 0:
            d = (db.astype(np.float64) @ Ws[l].astype(np.float64).T).astype(np.float32) * silu_grad(Z[l - 1])
    return g, loss


def adam_first_step(params: np.ndarray, grads: np.ndarray, lr) -> np.ndarray:
    """Adam's first step (m = v = 0 before it) in fp32 in the kernel's operation order (b1 = 0.9,
    b2 = 0.999, eps = 1e-8 as float constants), with the padding parameters (unused input rows, output
    columns 1..7) held at zero.  `lr` is the step's learning rate as a float32."""
    f = np.float32
    b1, b2 = f(0.9), f(0.999)
    g = grads.astype(np.float32)
    m = (f(1.0) - b1) * g
    v = ((f(1.0) - b2) * g) * g
    mh = m / (f(1.0) - b1)
    vh = v / (f(1.0) - b2)
    w = params.astype(np.float32) - (f(lr) * mh) / (np.sqrt(vh) + f(1e-8))
    idx = np.arange(NPARAM)
    pad = ((idx < P_B1) & (idx // HID >= NFEAT)) | ((idx >= P_W5) & (idx < P_B5) & ((idx - P_W5) % OUTN != 0)) | \
          ((idx >= P_B5) & (idx != P_B5))
    w[pad] = 0.0
    return w
