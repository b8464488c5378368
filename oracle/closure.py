"""CPU oracle of the KS closure network -- TEST INFRASTRUCTURE ONLY.

The network corrects a coarse KS step: delta = f(u), u one periodic coarse
domain, f = conv5(32->1) . GELU . conv5(32->32) . GELU . conv5(1->32), circular
padding 2 on every layer, GELU in its tanh form.  Parameters are kept in FP32 and rounded to BF16
for the forward pass; the 32->32 layer multiplies BF16 activations by BF16
weights with FP32 accumulation (the tensor-core layer), the outer layers run
in FP32 with the BF16-rounded weights.  This module restates that arithmetic
in float64 (with the same BF16 rounding points) and its gradients, so the GPU
kernels' forward outputs and weight gradients can be checked against it.

Parameter layout (flat FP32 vector, PARAMS = 5506 values):
  w1[32][5] b1[32] | w2[32][32][5] b2[32] | w3[32][5] b3[1] | s[1]
  w[out][in][tap], tap t multiplies u[x + t - 2]; delta = s * net(u), the
  output scale s is fixed (not trained).  The loss is on the scaled defect:
  mean (net(u) - target / s)^2.
"""
from __future__ import annotations

import math

import numpy as np

C = 32
K = 5
SIZES = [("w1", (C, K)), ("b1", (C,)), ("w2", (C, C, K)), ("b2", (C,)), ("w3", (C, K)), ("b3", (1,)),
         ("scale", (1,))]
PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(theta: np.ndarray) -> dict:
    out, at = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(theta[at:at + n], dtype=np.float64).reshape(shape)
        at += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest, ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    nan = np.isnan(f)
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


def init(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """He-style initialisation; the last layer starts near zero so the
    untrained closure leaves the coarse step unchanged."""
    rng = np.random.default_rng(seed)
    d = {
        "w1": rng.standard_normal((C, K)) * math.sqrt(2.0 / K) * scale,
        "b1": np.zeros(C),
        "w2": rng.standard_normal((C, C, K)) * math.sqrt(2.0 / (C * K)) * scale,
        "b2": np.zeros(C),
        "w3": rng.standard_normal((C, K)) * 1e-3,
        "b3": np.zeros(1),
        "scale": np.ones(1),
    }
    return pack(d).astype(np.float32)


# GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units",
# 2016): x/2 (1 + tanh(c (x + a x^3))), c = sqrt(2/pi), a = 0.044715 -- the
# form the kernels evaluate (with the SFU's tanh.approx.f32; here an exact tanh).
GELU_C, GELU_A = math.sqrt(2.0 / math.pi), 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(GELU_C * (x + GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * x * x)


def _taps(a: np.ndarray) -> np.ndarray:
    """a[..., ch, n] -> stacked shifted copies [..., ch, K, n], tap t = a[x + t - 2] (periodic)."""
    return np.stack([np.roll(a, 2 - t, axis=-1) for t in range(K)], axis=-2)


def forward(theta: np.ndarray, u: np.ndarray, keep: bool = False):
    """u: (batch, n) coarse states.  Returns delta (batch, n) [and the activations]."""
    p = unpack(theta)
    w1, w2, w3 = bf16(p["w1"]), bf16(p["w2"]), bf16(p["w3"])
    u = np.asarray(u, dtype=np.float64)
    if u.ndim == 1:
        u = u[None]
    # layer 1 (FP32 cores): z1[b, o, x] = sum_t w1[o,t] u[x+t-2] + b1[o]
    tu = _taps(u[:, None, :])[:, 0]                      # (b, K, n)
    z1 = np.einsum("ot,btn->bon", w1, tu) + p["b1"][None, :, None]
    a1 = gelu(z1)
    a1q = bf16(a1)                                       # BF16 operand of the tensor-core layer
    t1 = _taps(a1q)                                      # (b, C, K, n)
    z2 = np.einsum("oit,bitn->bon", w2, t1) + p["b2"][None, :, None]
    a2 = gelu(z2)
    t2 = _taps(a2)                                       # (b, C, K, n)
    raw = np.einsum("it,bitn->bn", w3, t2) + p["b3"][0]
    if keep:
        return raw, dict(u=u, tu=tu, z1=z1, a1q=a1q, t1=t1, z2=z2, a2=a2, t2=t2)
    return np.float32(p["scale"][0]) * raw


def loss_and_grad(theta: np.ndarray, u: np.ndarray, target: np.ndarray):
    """Mean squared scaled defect, mean (net(u) - target/s)^2, and its gradient
    with respect to the FP32 parameters (straight-through for the BF16
    roundings; zero for the fixed scale s)."""
    raw, s = forward(theta, u, keep=True)
    target = np.asarray(target, dtype=np.float64).reshape(raw.shape)
    scl = float(np.float32(unpack(theta)["scale"][0]))
    npts = raw.size
    err = raw - np.asarray(np.asarray(target, dtype=np.float32) / np.float32(scl), dtype=np.float64)
    loss = float(np.sum(err * err) / npts)
    g = 2.0 * err / npts                                  # dL/ddelta (b, n)
    p = unpack(theta)
    w2, w3 = bf16(p["w2"]), bf16(p["w3"])
    grads = {"b3": np.array([g.sum()]), "w3": np.einsum("bn,bitn->it", g, s["t2"])}
    # dL/da2[b,i,x] = sum_t w3[i,t] g[x - t + 2]
    da2 = np.zeros_like(s["a2"])
    for t in range(K):
        da2 += w3[None, :, t, None] * np.roll(g, t - 2, axis=-1)[:, None, :]
    dz2 = da2 * gelu_grad(s["z2"])
    grads["b2"] = dz2.sum(axis=(0, 2))
    grads["w2"] = np.einsum("bon,bitn->oit", dz2, s["t1"])
    da1 = np.zeros_like(s["z1"])
    for t in range(K):
        da1 += np.einsum("oi,bon->bin", w2[:, :, t], np.roll(dz2, t - 2, axis=-1))
    dz1 = da1 * gelu_grad(s["z1"])
    grads["b1"] = dz1.sum(axis=(0, 2))
    grads["w1"] = np.einsum("bon,btn->ot", dz1, s["tu"])
    grads["scale"] = np.zeros(1)
    return loss, pack(grads)


def coarse_grain(fine: np.ndarray, factor: int = 4) -> np.ndarray:
    """Cell averages of `factor` consecutive fine cells (periodic domains)."""
    fine = np.asarray(fine)
    return fine.reshape(*fine.shape[:-1], fine.shape[-1] // factor, factor).mean(axis=-1)
