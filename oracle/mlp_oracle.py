"""TEST INFRASTRUCTURE — float64 CPU restatement of the score predictor (csrc/mlp_kernel.cu).

The predictor has no counterpart in the reference; this module is its oracle: the same
features, the same network with the same bf16 roundings at the same places (inputs, W1, W2
and the layer-1 activations are bf16 on the GPU; accumulation is fp32 there and float64
here), and the analytic gradient of the mean squared error on log(1 + |score|) targets.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 32, 64
OFF_W1 = 0
OFF_B1 = N_IN * N_HID
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID
N_PARAMS = OFF_B3 + 1


def bf16_round(x) -> np.ndarray:
    """Round to the nearest bf16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    bits = a.view(np.uint32).astype(np.uint64)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return rounded.view(np.float32).astype(np.float64)


def bf16_bits_to_float(bits: np.ndarray) -> np.ndarray:
    return (np.asarray(bits, np.uint32) << 16).astype(np.uint32).view(np.float32).astype(np.float64)


def kmer_bin(d: np.ndarray) -> np.ndarray:
    d = np.asarray(d, np.int64)
    out = d.copy()
    big = d >= 16
    lg = np.floor(np.log2(np.maximum(d, 1))).astype(np.int64)
    out[big] = np.minimum(27, 16 + (lg[big] - 4))
    return out


def features(pattern: bytes, text: bytes) -> np.ndarray:
    """The 32 features of one pair (float64, before bf16 rounding)."""
    def counts(s: bytes) -> np.ndarray:
        c = np.zeros(256, np.int64)
        a = (np.frombuffer(s, np.uint8).astype(np.int64) >> 1) & 3
        if a.size >= 4:
            codes = (a[:-3] << 6) | (a[1:-2] << 4) | (a[2:-1] << 2) | a[3:]
            np.add.at(c, codes, 1)
        return c
    cp, ct = counts(pattern), counts(text)
    d = np.abs(cp - ct)
    hist = np.bincount(kmer_bin(d), minlength=28)[:28]
    plen, tlen = len(pattern), len(text)
    tot = plen + tlen + 1
    f = np.empty(N_IN)
    f[0] = np.log2(plen + 1.0) / 16
    f[1] = np.log2(tlen + 1.0) / 16
    f[2] = (plen - tlen) / tot
    f[3:31] = hist / 256.0
    f[31] = d.sum() / tot
    return f


def unpack(params: np.ndarray):
    p = np.asarray(params, np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(N_IN, N_HID)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(N_HID, N_HID)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, w3, b3


def forward(params: np.ndarray, X: np.ndarray):
    """X: bf16-valued features (n x 32). Returns y and the activations."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    # bias/w3 are fp32 on the device
    b1, b2, w3 = (np.float32(b1).astype(np.float64), np.float32(b2).astype(np.float64),
                  np.float32(w3).astype(np.float64))
    b3 = float(np.float32(b3))
    h1 = bf16_round(np.maximum(X @ bf16_round(W1) + b1, 0.0))
    h2 = np.maximum(h1 @ bf16_round(W2) + b2, 0.0)
    y = h2 @ w3 + b3
    return y, h1, h2


def loss_and_grad(params: np.ndarray, X: np.ndarray, t: np.ndarray):
    """Mean squared error and its gradient (the device's backward: fp32 W2 in dH1)."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    w3 = np.float32(w3).astype(np.float64)
    W2f = np.float32(W2).astype(np.float64)
    y, h1, h2 = forward(params, X)
    n = X.shape[0]
    e = y - t
    loss = float(np.mean(e * e))
    dy = 2.0 * e / n
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    dh2 = dy[:, None] * w3[None, :] * (h2 > 0)
    g[OFF_W2:OFF_B2] = (h1.T @ dh2).reshape(-1)
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = (dh2 @ W2f.T) * (h1 > 0)
    g[OFF_W1:OFF_B1] = (X.T @ dh1).reshape(-1)
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    return loss, g
