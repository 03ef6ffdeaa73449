"""CPU oracle of the learned part (test infrastructure only).

Restates, in numpy, the BF16 MLP of help_gb300/csrc/mlp.cu with the same
rounding points -- inputs, weights and stored activations rounded to BF16
(round to nearest even), products accumulated in FP32 -- its weighted
squared-error loss and the gradients the backward kernel forms, so GPU
results can be compared to it at FP32 summation-order tolerance.  With
``exact=True`` every rounding is skipped and the arithmetic is float64: that
form is checked against finite differences, which pins the back-propagation
formulas themselves.

The MLP has no counterpart in the reference; parameter layout and semantics
follow include/help_gpu.h (HELP_MLP_*).
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 16, 64, 2
OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3, OFF_MEAN, OFF_SCALE, NPARAMS = (
    0, 1024, 1088, 5184, 5248, 5376, 5378, 5394, 5410)


def bf16(a) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p)
    return (p[OFF_W1:OFF_B1].reshape(HID, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(HID, HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(OUT, HID), p[OFF_B3:OFF_MEAN])


def forward(p, x, exact=False):
    """out [rows x 2] and the stored activations (H1, H2)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    if exact:
        f = lambda a: np.asarray(a, np.float64)
        x, W1, b1, W2, b2, W3, b3 = map(f, (x, W1, b1, W2, b2, W3, b3))
        H1 = np.maximum(x @ W1.T + b1, 0.0)
        H2 = np.maximum(H1 @ W2.T + b2, 0.0)
        return H2 @ W3.T + b3, H1, H2
    x = bf16(x)
    W1, W2, W3 = bf16(W1), bf16(W2), bf16(W3)
    b1, b2, b3 = (np.asarray(b, np.float32) for b in (b1, b2, b3))
    H1 = bf16(np.maximum(x @ W1.T + b1, 0.0))
    H2 = bf16(np.maximum(H1 @ W2.T + b2, 0.0))
    return (H2 @ W3.T + b3).astype(np.float32), H1, H2


def loss_grad(p, x, t, w, exact=False):
    """Loss sum w (out - t)^2 / sum w and its gradient (trainable layout, OFF_MEAN floats)."""
    out, H1, H2 = forward(p, x, exact)
    W1, b1, W2, b2, W3, b3 = unpack(p)
    wsum = float(np.sum(np.asarray(w, np.float64)))
    if exact:
        e = out - t
        loss = float(np.sum(w * e * e) / wsum)
        G3 = 2.0 * w * e / wsum
        dZ2 = (G3 @ W3) * (H2 > 0)
        dZ1 = (dZ2 @ W2) * (H1 > 0)
        xx = np.asarray(x, np.float64)
    else:
        inv = np.float32(1.0 / wsum) if wsum > 0 else np.float32(0.0)
        e = (out - np.asarray(t, np.float32)).astype(np.float32)
        wf = np.asarray(w, np.float32)
        loss = float(np.sum((wf * e * e * inv).astype(np.float64)))
        G3 = bf16((np.float32(2.0) * wf * e * inv).astype(np.float32))
        W3b, W2b = bf16(W3), bf16(W2)
        dZ2 = bf16((G3 @ W3b) * (H2 > 0))
        dZ1 = bf16((dZ2 @ W2b) * (H1 > 0))
        xx = bf16(x)
    g = np.zeros(OFF_MEAN, np.float64)
    g[OFF_W1:OFF_B1] = (dZ1.T @ xx).ravel()
    g[OFF_B1:OFF_W2] = dZ1.sum(0)
    g[OFF_W2:OFF_B2] = (dZ2.T @ H1).ravel()
    g[OFF_B2:OFF_W3] = dZ2.sum(0)
    g[OFF_W3:OFF_B3] = (G3.T @ H2).ravel()
    g[OFF_B3:OFF_MEAN] = G3.sum(0)
    return loss, g


def init_params(seed: int, mean=None, scale=None) -> np.ndarray:
    """He-style initialisation; normalisation constants default to (0, 1)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    p[OFF_W1:OFF_B1] = rng.normal(0, np.sqrt(2.0 / IN), HID * IN)
    p[OFF_W2:OFF_B2] = rng.normal(0, np.sqrt(2.0 / HID), HID * HID)
    p[OFF_W3:OFF_B3] = rng.normal(0, np.sqrt(1.0 / HID), OUT * HID)
    p[OFF_MEAN:OFF_SCALE] = 0.0 if mean is None else mean
    p[OFF_SCALE:NPARAMS] = 1.0 if scale is None else scale
    return p
