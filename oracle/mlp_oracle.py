"""Oracle test infrastructure -- not part of the product.

CPU (numpy, FP32) restatement of the learned candidate filter that the GPU
library trains and runs with its own tensor-core kernels: an MLP
40 -> 128 -> 128 -> 128 -> 1 with GELU (erf form), BF16 operands and FP32
accumulation, a logistic output and a (positive-weighted) binary
cross-entropy loss, trained with Adam.

The rounding points are the GPU kernels' own: every GEMM operand is rounded
to BF16 (round to nearest even) and every product is accumulated in FP32;
pre-activations, the output layer, the loss and the optimizer stay FP32.
With the same inputs and weights the GPU gradients then differ from these
only by FP32 summation order.  Only tests/ may import this module.
"""
from __future__ import annotations

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover
    _erf = np.vectorize(__import__("math").erf)

N_FEAT = 40
K_IN = 64          # the first layer's input width as the kernels see it (zero padded)
HID = 128
SQRT1_2 = np.float32(0.7071067811865476)
INV_SQRT_2PI = np.float32(0.3989422804014327)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 to the nearest BF16 (ties to even), returned as FP32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def gelu(z):
    return (0.5 * z * (1.0 + _erf(z * SQRT1_2))).astype(np.float32)


def gelu_grad(z):
    cdf = 0.5 * (1.0 + _erf(z * SQRT1_2))
    pdf = INV_SQRT_2PI * np.exp(-0.5 * z * z)
    return (cdf + z * pdf).astype(np.float32)


def init_params(seed: int = 0) -> dict:
    """The library's initialisation is its own; tests copy weights across."""
    rng = np.random.default_rng(seed)
    p = {}
    dims = [(HID, K_IN, N_FEAT), (HID, HID, HID), (HID, HID, HID)]
    for i, (o, kin, fan) in enumerate(dims, 1):
        w = np.zeros((o, kin), np.float32)
        w[:, :fan] = rng.normal(0, np.sqrt(2.0 / fan), (o, fan))
        p[f"W{i}"] = w
        p[f"b{i}"] = np.zeros(o, np.float32)
    p["w4"] = rng.normal(0, np.sqrt(1.0 / HID), HID).astype(np.float32)
    p["b4"] = np.zeros(1, np.float32)
    return p


def pad_features(x: np.ndarray) -> np.ndarray:
    out = np.zeros((x.shape[0], K_IN), np.float32)
    out[:, :x.shape[1]] = x
    return out


def forward(p: dict, x: np.ndarray, exact: bool = False):
    """x: (B, 40) features.  Returns logits (B,) and the cache for backward.
    exact=True skips the BF16 rounding (for finite-difference checks)."""
    r = (lambda a: np.asarray(a, np.float32)) if exact else bf16
    h = r(pad_features(x))
    cache = {"H0": h, "exact": exact}
    for i in (1, 2, 3):
        z = (h @ r(p[f"W{i}"]).T + p[f"b{i}"]).astype(np.float32)
        h = r(gelu(z))
        cache[f"Z{i}"] = z
        cache[f"H{i}"] = h
    logit = (h @ p["w4"] + p["b4"][0]).astype(np.float32)
    return logit, cache


def loss_and_dlogit(logit: np.ndarray, y: np.ndarray, pos_weight: float = 1.0):
    """Mean weighted BCE with logits and its gradient w.r.t. the logits."""
    y = y.astype(np.float32)
    w = np.where(y > 0.5, np.float32(pos_weight), np.float32(1.0))
    sp = np.logaddexp(0, logit)  # softplus
    loss = float(np.mean(w * (sp - y * logit)))
    sig = 1.0 / (1.0 + np.exp(-logit))
    d = (w * (sig - y) / logit.shape[0]).astype(np.float32)
    return loss, d


def backward(p: dict, cache: dict, dlogit: np.ndarray) -> dict:
    r = (lambda a: np.asarray(a, np.float32)) if cache.get("exact") else bf16
    g = {}
    h3 = cache["H3"]
    g["w4"] = (dlogit @ h3).astype(np.float32)
    g["b4"] = np.array([dlogit.sum()], np.float32)
    dz = r((dlogit[:, None] * p["w4"][None, :]) * gelu_grad(cache["Z3"]))
    for i in (3, 2, 1):
        hp = cache[f"H{i - 1}"]
        g[f"W{i}"] = (dz.T @ hp).astype(np.float32)
        g[f"b{i}"] = dz.astype(np.float32).sum(axis=0)
        if i > 1:
            dh = (dz @ r(p[f"W{i}"])).astype(np.float32)
            dz = r(dh * gelu_grad(cache[f"Z{i - 1}"]))
    g["W1"][:, N_FEAT:] = 0.0
    return g


def adam_step(p: dict, g: dict, state: dict, lr: float, t: int, b1=0.9, b2=0.999, eps=1e-8):
    for k in p:
        m = state.setdefault("m_" + k, np.zeros_like(p[k]))
        v = state.setdefault("v_" + k, np.zeros_like(p[k]))
        m[:] = b1 * m + (1 - b1) * g[k]
        v[:] = b2 * v + (1 - b2) * g[k] * g[k]
        mh = m / (1 - b1 ** t)
        vh = v / (1 - b2 ** t)
        p[k] -= (lr * mh / (np.sqrt(vh) + eps)).astype(np.float32)
    p["W1"][:, N_FEAT:] = 0.0
