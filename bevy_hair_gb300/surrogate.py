"""The learned shading surrogate: host side of the ``hg_mlp_*`` entry points.

A ReLU network (FP16 weights and activations, FP32 accumulation on the
tensor cores) that stands in for the Karis-fit lobes of
``shade.wesl:94-190``: 10 -> 4 x 64 -> 12 lobes (``MLP_ARCH_DEEP``, shade
models 1 and 2) or the compact 10 -> 2 x 32 -> 3 (``MLP_ARCH_COMPACT``, shade
model 3), which predicts the per-light BSDF R + TT + TRT + 0.7 B directly.  It is trained on FP64 samples of the exact lobes
(Gauss-Legendre integration of the Marschner/d'Eon azimuthal scattering plus
the Zinke back-scattering term), generated on the GPU by ``hg_mlp_samples``.

Device buffers for training are torch CUDA tensors (allocation only); every
computation runs in libhairgb.so.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from pathlib import Path

import numpy as np

from . import abi
from .pipeline import HairRenderer, _check

WEIGHTS = Path(__file__).resolve().parent / "surrogate_weights.npy"
COMPACT_WEIGHTS = Path(__file__).resolve().parent / "surrogate_compact_weights.npy"
TILT = 0.08                 # longitudinal tilt the network is trained at (all configs use it)
SAMPLE_SEED = 0x5EED0005    # seed of the training set (16M samples)
HOLDOUT_FIRST = 1 << 40     # sample index where the held-out set starts

# Parameter layouts: hg_mlp.cuh W1[64][16] b1 W2[64][64] b2 W3 b3 W4 b4 W5[16][64] b5;
# hg_mlp_small.cuh W1[32][16] b1 W2[32][32] b2 W3[16][32] b3.
LAYERS = ((64, 16), (64, 64), (64, 64), (64, 64), (16, 64))
COMPACT_LAYERS = ((32, 16), (32, 32), (16, 32))


def layers_of(arch: int = abi.MLP_ARCH_DEEP):
    return COMPACT_LAYERS if arch == abi.MLP_ARCH_COMPACT else LAYERS


def param_count(arch: int = abi.MLP_ARCH_DEEP) -> int:
    return abi.MLP_COMPACT_PARAMS if arch == abi.MLP_ARCH_COMPACT else abi.MLP_PARAMS


def output_count(arch: int = abi.MLP_ARCH_DEEP) -> int:
    return abi.MLP_COMPACT_OUTPUTS if arch == abi.MLP_ARCH_COMPACT else abi.MLP_OUTPUTS


def split(params: np.ndarray, arch: int = abi.MLP_ARCH_DEEP) -> list[tuple[np.ndarray, np.ndarray]]:
    """Views (W[out][in], b[out]) of each layer of a flat parameter vector."""
    out, o = [], 0
    for rows, cols in layers_of(arch):
        w = params[o:o + rows * cols].reshape(rows, cols)
        o += rows * cols
        b = params[o:o + rows]
        o += rows
        out.append((w, b))
    assert o == param_count(arch) == len(params)
    return out


def init_params(seed: int = 0, arch: int = abi.MLP_ARCH_DEEP) -> np.ndarray:
    """He-normal hidden layers, a small output layer, zero biases and zero padding."""
    rng = np.random.default_rng(seed)
    p = np.zeros(param_count(arch), dtype=np.float32)
    layers = split(p, arch)
    for k, (w, _b) in enumerate(layers):
        fan_in = abi.MLP_INPUTS if k == 0 else w.shape[1]
        std = math.sqrt(2.0 / fan_in) * (0.5 if k == len(layers) - 1 else 1.0)
        w[...] = rng.normal(0.0, std, size=w.shape).astype(np.float32)
    layers[0][0][:, abi.MLP_INPUTS:] = 0.0
    w_out, b_out = layers[-1]
    w_out[output_count(arch):, :] = 0.0
    b_out[...] = 0.0
    return p


def weights_path(arch: int = abi.MLP_ARCH_DEEP) -> Path:
    return COMPACT_WEIGHTS if arch == abi.MLP_ARCH_COMPACT else WEIGHTS


def load_params(arch: int = abi.MLP_ARCH_DEEP) -> np.ndarray:
    """The trained parameters shipped with the package."""
    path = weights_path(arch)
    p = np.load(path).astype(np.float32)
    if p.shape != (param_count(arch),):
        raise ValueError(f"{path} holds {p.shape}, expected ({param_count(arch)},)")
    return p


def _ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr() if hasattr(t, "data_ptr") else int(t)


class Surrogate:
    """One hg_mlp on a renderer's context."""

    def __init__(self, renderer: HairRenderer, params: np.ndarray | None = None, arch: int = abi.MLP_ARCH_DEEP):
        self.renderer = renderer
        self.lib = renderer.lib
        self.arch = int(arch)
        h = C.c_void_p()
        _check(self.lib, renderer.ctx, self.lib.hg_mlp_create_arch(renderer.ctx, self.arch, C.byref(h)))
        self.handle = h
        self.n_params = int(self.lib.hg_mlp_param_count(h))
        self.n_out = int(self.lib.hg_mlp_output_count(h))
        if not hasattr(renderer, "_surrogates"):
            renderer._surrogates = []
        renderer._surrogates.append(self)
        if params is not None:
            self.set_params(params)

    def _check(self, status: int) -> None:
        _check(self.lib, self.renderer.ctx, status)

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.hg_mlp_set_params(self.handle, p.ctypes.data, p.size))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n_params, dtype=np.float32)
        self._check(self.lib.hg_mlp_get_params(self.handle, p.ctypes.data, p.size))
        return p

    def infer(self, inputs, n: int, lobes=None, net=None) -> None:
        """Device float[n][10] inputs -> device float[n][n_out] decoded outputs and/or raw outputs
        (12 lobes, or the compact network's 3 BSDF channels)."""
        self._check(self.lib.hg_mlp_infer(self.handle, _ptr(inputs), n, _ptr(lobes), _ptr(net)))

    def infer_tc(self, inputs, n: int, lobes=None, net=None) -> None:
        """The same evaluation on the tcgen05 tensor cores (128 rows per MMA, TMEM accumulators);
        4 x 64 network only."""
        self._check(self.lib.hg_mlp_infer_tc(self.handle, _ptr(inputs), n, _ptr(lobes), _ptr(net)))

    def gradients(self, inputs, targets, n: int) -> tuple[np.ndarray, float]:
        """Gradient of sum((net - target)^2) over one device batch, and that sum."""
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float()
        self._check(self.lib.hg_mlp_gradients(self.handle, _ptr(inputs), _ptr(targets), n, g.ctypes.data,
                                              C.byref(loss)))
        return g, float(loss.value)

    def train_step(self, inputs, targets, n: int, lr: float, loss_sum=None) -> None:
        self._check(self.lib.hg_mlp_train_step(self.handle, _ptr(inputs), _ptr(targets), n, float(lr),
                                               _ptr(loss_sum)))

    def close(self) -> None:
        if self.handle:
            self.lib.hg_mlp_destroy(self.handle)
            self.handle = None
            if self in getattr(self.renderer, "_surrogates", []):
                self.renderer._surrogates.remove(self)


def samples(renderer: HairRenderer, seed: int, first: int, n: int, inputs, targets=None, lobes=None,
            tilt: float = TILT) -> None:
    """Fill device buffers with n FP64-integrated training samples (hg_mlp_samples)."""
    _check(renderer.lib, renderer.ctx,
           renderer.lib.hg_mlp_samples(renderer.ctx, seed, first, n, tilt, _ptr(inputs), _ptr(targets),
                                       _ptr(lobes)))


def karis_lobes(renderer: HairRenderer, inputs, n: int, lobes, tilt: float = TILT) -> None:
    """The same 12 lobes from the Karis fits as the shade pass evaluates them (hg_karis_lobes)."""
    _check(renderer.lib, renderer.ctx,
           renderer.lib.hg_karis_lobes(renderer.ctx, _ptr(inputs), n, tilt, _ptr(lobes)))


def bsdf(lobes: np.ndarray) -> np.ndarray:
    """Per-light BSDF the shade pass adds at zero DOM depth: R + TT + TRT + 0.7 B (rgb)."""
    l = np.asarray(lobes, dtype=np.float64).reshape(-1, 12)
    return l[:, 0:3] + l[:, 3:6] + l[:, 6:9] + 0.7 * l[:, 9:12]


def relative_l1(pred: np.ndarray, ref: np.ndarray) -> float:
    """sum |pred - ref| / sum |ref|."""
    pred = np.asarray(pred, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(pred - ref).sum() / max(np.abs(ref).sum(), 1e-300))


def evaluate(renderer: HairRenderer, surrogate: Surrogate, n: int = 1 << 16, seed: int = SAMPLE_SEED) -> dict:
    """Errors of the surrogate and of the Karis fit against FP64 lobes on a
    held-out set: relative L1 of the per-light BSDF and of each lobe."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.empty((n, 10), dtype=torch.float32, device=dev)
    exact = torch.empty((n, 12), dtype=torch.float64, device=dev)
    pred = torch.empty((n, surrogate.n_out), dtype=torch.float32, device=dev)
    kar = torch.empty((n, 12), dtype=torch.float32, device=dev)
    samples(renderer, seed, HOLDOUT_FIRST, n, x, None, exact)
    surrogate.infer(x, n, pred)
    karis_lobes(renderer, x, n, kar)
    renderer.synchronize()
    e, p, k = exact.cpu().numpy(), pred.cpu().numpy(), kar.cpu().numpy()
    per_light = p if surrogate.n_out == 3 else bsdf(p)
    out = {"samples": n, "surrogate_bsdf": relative_l1(per_light, bsdf(e)),
           "karis_bsdf": relative_l1(bsdf(k), bsdf(e))}
    for i, name in enumerate(("R", "TT", "TRT", "B")):
        sl = slice(3 * i, 3 * i + 3)
        if surrogate.n_out == 12:
            out[f"surrogate_{name}"] = relative_l1(p[:, sl], e[:, sl])
        out[f"karis_{name}"] = relative_l1(k[:, sl], e[:, sl])
    return out


def train(renderer: HairRenderer, n_samples: int = 16 << 20, batch: int = 16384, epochs: int = 150,
          lr_max: float = 3e-3, lr_min: float = 1e-5, warmup: int = 200, seed: int = SAMPLE_SEED,
          init_seed: int = 0, log=print, arch: int = abi.MLP_ARCH_DEEP) -> tuple[np.ndarray, dict]:
    """Generate n_samples FP64 samples on the GPU and fit the network with Adam
    (linear warm-up, cosine decay).  Returns the parameters and a history."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.perf_counter()
    x = torch.empty((n_samples, 10), dtype=torch.float32, device=dev)
    y = torch.empty((n_samples, 12), dtype=torch.float32, device=dev)
    chunk = 1 << 22
    for first in range(0, n_samples, chunk):
        m = min(chunk, n_samples - first)
        samples(renderer, seed, first, m, x[first:first + m], y[first:first + m])
    renderer.synchronize()
    t_gen = time.perf_counter() - t0
    log(f"generated {n_samples} FP64 samples in {t_gen:.1f} s")

    s = Surrogate(renderer, init_params(init_seed, arch), arch)
    n_batches = n_samples // batch
    steps = n_batches * epochs
    losses = torch.zeros(steps, dtype=torch.float32, device=dev)
    rng = np.random.default_rng(seed)
    t1 = time.perf_counter()
    step = 0
    for ep in range(epochs):
        for b in rng.permutation(n_batches):
            if step < warmup:
                lr = lr_max * (step + 1) / warmup
            else:
                q = (step - warmup) / max(steps - warmup, 1)
                lr = lr_min + 0.5 * (lr_max - lr_min) * (1.0 + math.cos(math.pi * q))
            lo = int(b) * batch
            s.train_step(x[lo:lo + batch], y[lo:lo + batch], batch, lr, losses[step:step + 1])
            step += 1
        if log and (ep % 5 == 4 or ep == epochs - 1):
            renderer.synchronize()
            recent = losses[step - n_batches:step].mean().item() / (batch * 12)
            log(f"epoch {ep + 1}/{epochs}: mse {recent:.3e} ({time.perf_counter() - t1:.1f} s)")
    renderer.synchronize()
    t_train = time.perf_counter() - t1
    params = s.get_params()
    hist = {"arch": "2x32" if arch == abi.MLP_ARCH_COMPACT else "4x64", "generate_s": t_gen, "train_s": t_train,
            "steps": steps, "batch": batch, "epochs": epochs,
            "samples": n_samples, "final_mse": losses[-n_batches:].mean().item() / (batch * 12),
            "first_mse": losses[:min(50, steps)].mean().item() / (batch * 12)}
    hist["heldout"] = evaluate(renderer, s)
    s.close()
    return params, hist


def main(argv=None) -> int:
    """Train the surrogate and write its parameters (and a JSON history)."""
    import argparse
    import json

    ap = argparse.ArgumentParser(description="Train the shading surrogate on FP64 samples generated on the GPU.")
    ap.add_argument("--samples", type=int, default=16 << 20)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--arch", choices=("4x64", "2x32"), default="4x64")
    ap.add_argument("--out", type=Path, default=None)
    ap.add_argument("--history", type=Path, default=None)
    a = ap.parse_args(argv)
    arch = abi.MLP_ARCH_COMPACT if a.arch == "2x32" else abi.MLP_ARCH_DEEP
    if a.out is None:
        a.out = weights_path(arch)
    with HairRenderer(0) as r:
        params, hist = train(r, n_samples=a.samples, batch=a.batch, epochs=a.epochs, lr_max=a.lr, arch=arch)
    a.out.parent.mkdir(parents=True, exist_ok=True)
    np.save(a.out, params)
    text = json.dumps(hist, indent=1)
    print(text)
    if a.history:
        a.history.write_text(text + "\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
