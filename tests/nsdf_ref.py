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
