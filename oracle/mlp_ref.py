"""FP64 reference of the shading surrogate's network.  TEST INFRASTRUCTURE ONLY.

Forward and backward passes of the 10 -> 4 x 64 -> 12 ReLU network (arch 0,
the twelve lobes) and of the compact 10 -> 2 x 32 -> 3 network (arch 1, the
per-light BSDF rgb) that libhairgb.so trains and evaluates
(bevy_hair_gb300/csrc/hg_mlp.cuh, hg_mlp_small.cuh, surrogate.cu).  With ``half=True`` the weights, the normalised
inputs and the post-ReLU activations are rounded to FP16 exactly where the
kernels round them, and everything else is FP64; the gradients are not
rounded (the kernels round the backward pass's fragments to FP16, so the
comparison uses a tolerance).  With ``half=False`` the network is smooth FP64
for finite-difference checks of the analytic gradient.

Loss: sum over samples and the used outputs of (y - target)^2.  Targets are
the twelve transformed lobes log1p(lobe / 1e-3) in both cases; arch 1's three
targets are log1p(bsdf / 1e-3) with bsdf = R + TT + TRT + 0.7 B formed from
them (``bsdf_targets``).
"""
from __future__ import annotations

import numpy as np

LAYERS = ((64, 16), (64, 64), (64, 64), (64, 64), (16, 64))
N_PARAMS = 14608
COMPACT_LAYERS = ((32, 16), (32, 32), (16, 32))
COMPACT_PARAMS = 2128
N_OUT = 12


def layers_of(arch: int):
    return COMPACT_LAYERS if arch == 1 else LAYERS


def outputs_of(arch: int) -> int:
    return 3 if arch == 1 else N_OUT


def bsdf_targets(targets12: np.ndarray) -> np.ndarray:
    """(n, 12) transformed lobes -> (n, 3) transformed BSDF channels (FP64)."""
    e = np.expm1(np.asarray(targets12, dtype=np.float64).reshape(-1, 12))
    return np.log1p(e[:, 0:3] + e[:, 3:6] + e[:, 6:9] + 0.7 * e[:, 9:12])


def split(params: np.ndarray, arch: int = 0):
    out, o = [], 0
    for rows, cols in layers_of(arch):
        w = params[o:o + rows * cols].reshape(rows, cols)
        o += rows * cols
        b = params[o:o + rows]
        o += rows
        out.append((w, b))
    assert o == (COMPACT_PARAMS if arch == 1 else N_PARAMS) == len(params)
    return out


def _h(a: np.ndarray, half: bool) -> np.ndarray:
    return a.astype(np.float16).astype(np.float64) if half else np.asarray(a, dtype=np.float64)


def normalise(raw: np.ndarray) -> np.ndarray:
    """hg_mlp.cuh normalise(): (n, 10) raw inputs -> (n, 16) network inputs (FP32 like the kernel)."""
    r = np.asarray(raw, dtype=np.float32).reshape(-1, 10)
    x = np.zeros((len(r), 16), dtype=np.float32)
    x[:, 0:4] = r[:, 0:4]
    x[:, 4:7] = (np.log(np.maximum(r[:, 4:7], np.float32(1e-6))) - np.float32(-0.91629073)) * np.float32(0.33380820)
    x[:, 7] = (r[:, 7] - np.float32(0.165)) * np.float32(7.4074074)
    x[:, 8] = (r[:, 8] - np.float32(0.5)) * np.float32(3.3333333)
    x[:, 9] = (r[:, 9] - np.float32(1.55)) * np.float32(10.0)
    return x


def forward(params: np.ndarray, raw: np.ndarray, half: bool = True, arch: int = 0):
    """Network outputs (n, 16; columns 12..15 are padding) and the activations."""
    # The kernels round the FP32 master weights to FP16; the smooth network keeps FP64.
    base = np.asarray(params, np.float32) if half else np.asarray(params, np.float64)
    layers = [(_h(w, half), np.asarray(b, dtype=np.float64)) for w, b in split(base, arch)]
    x = _h(normalise(raw), half)
    acts = [x]
    h = x
    for k, (w, b) in enumerate(layers):
        z = h @ w.T + b
        if k < len(layers) - 1:
            h = _h(np.maximum(z, 0.0), half)
            acts.append(h)
        else:
            h = z
    return h, acts, layers


def gradients(params: np.ndarray, raw: np.ndarray, targets: np.ndarray, half: bool = True, arch: int = 0):
    """(flat gradient float64[len(params)], loss) of sum((y - t)^2) over the 12 outputs."""
    y, acts, layers = forward(params, raw, half, arch)
    t = np.asarray(targets, dtype=np.float64).reshape(-1, N_OUT)
    if arch == 1:
        t = bsdf_targets(t)
    k = outputs_of(arch)
    d = np.zeros_like(y)
    d[:, :k] = y[:, :k] - t
    loss = float((d * d).sum())
    dz = 2.0 * d
    grads = [None] * len(layers)
    for k in range(len(layers) - 1, -1, -1):
        w, _ = layers[k]
        grads[k] = (dz.T @ acts[k], dz.sum(axis=0))
        if k > 0:
            dh = dz @ w
            dz = dh * (acts[k] > 0.0)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return flat, loss
