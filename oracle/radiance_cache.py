"""FP64 numpy restatement of the radiance-cache network — test infrastructure.

The oracle for the tensor-core MLP kernels (zig_ornament_gb300/csrc/
radiance_cache.cu): the same encoding, layer shapes, loss and Adam update,
in float64.  The reference renderer has no learned cache; this network is an
extension, so there is no reference file to follow — the oracle states the
mathematics the kernels implement and is itself checked by central finite
differences (tests/test_cache_oracle.py).

`emulate=True` additionally rounds the operands the way the kernels store
them (FP16 forward operands and activations, BF16 backward operands), which
narrows the tolerance of the GPU comparison to the accumulation order.
"""
from __future__ import annotations

import numpy as np

INPUTS, BANDS, FEATURES, HIDDEN, OUTPUTS, OUT_PAD = 10, 12, 256, 64, 3, 16
SHAPES = [(HIDDEN, FEATURES)] + [(HIDDEN, HIDDEN)] * 4 + [(OUT_PAD, HIDDEN)]
OFFSETS = np.cumsum([0] + [o * i for o, i in SHAPES]).tolist()
PARAM_COUNT = OFFSETS[-1]   # 33792
GRAD_CLAMP = 1.0e4


def unpack(params: np.ndarray) -> list[np.ndarray]:
    p = np.asarray(params, dtype=np.float64).ravel()
    assert p.size == PARAM_COUNT
    return [p[OFFSETS[l]:OFFSETS[l + 1]].reshape(SHAPES[l]) for l in range(len(SHAPES))]


def pack(mats: list[np.ndarray]) -> np.ndarray:
    return np.concatenate([np.asarray(m, dtype=np.float64).ravel() for m in mats])


def round_f16(a: np.ndarray) -> np.ndarray:
    return np.asarray(a, dtype=np.float64).astype(np.float16).astype(np.float64)


def round_bf16(a: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (round to nearest, ties to even) through float32."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isfinite(f), out, f.astype(np.float64))


def encode(x: np.ndarray) -> np.ndarray:
    """(n, 10) inputs -> (n, 256) features: for input j and band b,
    feature 24j + 2b = sin(2^b pi x_j), 24j + 2b + 1 = cos(2^b pi x_j);
    then the 10 raw inputs, a constant 1 and 5 zeros."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, INPUTS)
    n = len(x)
    out = np.zeros((n, FEATURES))
    for j in range(INPUTS):
        for b in range(BANDS):
            a = np.pi * (2.0 ** b) * x[:, j]
            out[:, 24 * j + 2 * b] = np.sin(a)
            out[:, 24 * j + 2 * b + 1] = np.cos(a)
    out[:, 240:250] = x
    out[:, 250] = 1.0
    return out


def forward(params: np.ndarray, x: np.ndarray, emulate: bool = False):
    """Returns (outputs (n, 3), per-layer inputs a_0..a_5, pre-activations)."""
    W = unpack(params)
    a = encode(x)
    if emulate:
        a = round_f16(a)
        W = [round_f16(w) for w in W]
    acts, zs = [], []
    for l, w in enumerate(W):
        acts.append(a)
        z = a @ w.T
        zs.append(z)
        if l < len(W) - 1:
            a = np.maximum(z, 0.0)
            if emulate:
                a = round_f16(a)
    return zs[-1][:, :OUTPUTS], acts, zs


def loss_and_grads(params: np.ndarray, x: np.ndarray, targets: np.ndarray, emulate: bool = False):
    """Summed relative-L2 loss sum_i,c (y - r)^2 / (y^2 + 0.01) (y held
    constant in the denominator) over samples with r[0] >= 0, and its
    gradient with respect to every parameter (flat, params' layout)."""
    W = unpack(params)
    y, acts, zs = forward(params, x, emulate)
    t = np.asarray(targets, dtype=np.float64).reshape(-1, OUTPUTS)
    valid = t[:, 0] >= 0.0
    den = y * y + 0.01
    diff = y - np.where(valid[:, None], t, 0.0)
    loss = float(np.sum(np.where(valid[:, None], diff * diff / den, 0.0)))
    dy = np.clip(2.0 * diff / den, -GRAD_CLAMP, GRAD_CLAMP)
    dy[~valid] = 0.0
    dz = np.zeros((len(y), OUT_PAD))
    dz[:, :OUTPUTS] = dy
    if emulate:
        dz = round_bf16(dz)
        Wb = [round_bf16(w) for w in W]
    grads = [None] * len(W)
    for l in range(len(W) - 1, -1, -1):
        a = acts[l]
        if emulate:
            # layer 1's features are rounded to BF16 straight from FP32
            a = round_bf16(encode(x) if l == 0 else a)
        grads[l] = dz.T @ a
        if l > 0:
            da = dz @ (Wb[l] if emulate else W[l])
            dz = da * (acts[l] > 0.0)
            if emulate:
                dz = round_bf16(dz)
    g = pack(grads)
    # padded output rows carry no gradient
    g[OFFSETS[5] + OUTPUTS * HIDDEN:OFFSETS[6]] = 0.0
    return loss, g


def adam_step(params, m, v, grads, step, lr=1e-3, beta1=0.9, beta2=0.99, eps=1e-8, grad_scale=1.0):
    """One Adam update (the kernels' rc_adam, in float64)."""
    g = np.asarray(grads, dtype=np.float64) * grad_scale
    m = beta1 * m + (1.0 - beta1) * g
    v = beta2 * v + (1.0 - beta2) * g * g
    mh = m / (1.0 - beta1 ** step)
    vh = v / (1.0 - beta2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v
