"""ORACLE -- test infrastructure only (tests and the smoke check; never the product).

FP64 restatement of the surrogate network of mfree_iwf_gb300/csrc/mf_mlp.cu, used to
check its BF16 tensor-core forward and backward passes.  The network is a stack of
dense layers z = h W^T + b with ReLU between them and a linear last layer; the loss is
the mean over rows and outputs of (z_L - y)^2.  The reference has no such part (the
learned screen is this project's own), so nothing here is pinned to the reference;
the gradients are pinned to central finite differences instead (tests).

``emulate=True`` rounds to BF16 where the CUDA kernels store BF16 (the inputs, the
weights, every hidden activation after its ReLU, and the output-side gradient fed to
the two backward products) and computes everything else in FP64, so it isolates the
FP32 accumulation of the kernels; ``emulate=False`` is the exact network on
BF16-rounded weights and inputs.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value, ties to even (as __float2bfloat16), returned as FP64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    nan = np.isnan(f)
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


def unpack(params: np.ndarray, dims: Sequence[int]) -> List[Tuple[np.ndarray, np.ndarray]]:
    """Flat parameters (per layer: W [out][in] row-major, then b [out]) -> [(W, b)]."""
    layers, o = [], 0
    p = np.asarray(params, np.float64)
    for l in range(len(dims) - 1):
        i, n = dims[l], dims[l + 1]
        W = p[o:o + i * n].reshape(n, i)
        o += i * n
        b = p[o:o + n]
        o += n
        layers.append((W, b))
    assert o == p.size
    return layers


def pack(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers])


def forward(params: np.ndarray, dims: Sequence[int], x: np.ndarray, emulate: bool = True):
    """Returns (outputs [rows, out], activations [h_0 .. h_{L-1}])."""
    layers = unpack(params, dims)
    rnd = bf16_round if emulate else (lambda a: np.asarray(a, np.float64))
    h = bf16_round(x)
    acts = [h]
    for l, (W, b) in enumerate(layers):
        z = h @ bf16_round(W).T + b
        if l + 1 < len(layers):
            h = rnd(np.maximum(z, 0.0))
            acts.append(h)
        else:
            return z, acts
    raise AssertionError("no layers")


def gradients(params: np.ndarray, dims: Sequence[int], x: np.ndarray, y: np.ndarray,
              emulate: bool = True) -> Tuple[np.ndarray, float]:
    """(flat gradient of the mean squared error, loss) for one member's batch."""
    layers = unpack(params, dims)
    rnd = bf16_round if emulate else (lambda a: np.asarray(a, np.float64))
    z, acts = forward(params, dims, x, emulate)
    rows, out = z.shape
    diff = z - np.asarray(y, np.float64)
    loss = float(np.mean(diff * diff))
    dz = 2.0 * diff / (rows * out)  # FP64; the kernels keep an FP32 copy for the bias gradient
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        dzr = rnd(dz)
        gW = dzr.T @ acts[l]
        gb = dz.sum(axis=0)
        grads[l] = (gW, gb)
        if l == 0:
            break
        dh = dzr @ bf16_round(W)
        dz = np.where(acts[l] > 0.0, dh, 0.0)
    return pack(grads), loss


def numeric_gradients(params: np.ndarray, dims: Sequence[int], x: np.ndarray, y: np.ndarray,
                      idx: Sequence[int], eps: float = 1e-6) -> np.ndarray:
    """Central differences of the exact FP64 loss (no BF16 rounding anywhere)."""
    def loss(p):
        h = np.asarray(x, np.float64)
        for l, (W, b) in enumerate(unpack(p, dims)):
            z = h @ W.T + b
            h = np.maximum(z, 0.0) if l + 1 < len(dims) - 1 else z
        d = h - y
        return float(np.mean(d * d))

    p = np.array(params, np.float64)
    g = np.zeros(len(idx))
    for k, i in enumerate(idx):
        a, b_ = p.copy(), p.copy()
        a[i] += eps
        b_[i] -= eps
        g[k] = (loss(a) - loss(b_)) / (2 * eps)
    return g


def exact_gradients(params: np.ndarray, dims: Sequence[int], x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Analytic gradients of the exact FP64 network (no rounding): the finite-difference pin."""
    layers = unpack(params, dims)
    h = np.asarray(x, np.float64)
    acts = [h]
    for l, (W, b) in enumerate(layers):
        z = h @ W.T + b
        if l + 1 < len(layers):
            h = np.maximum(z, 0.0)
            acts.append(h)
    rows, out = z.shape
    dz = 2.0 * (z - y) / (rows * out)
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        grads[l] = (dz.T @ acts[l], dz.sum(axis=0))
        if l:
            dz = np.where(acts[l] > 0.0, dz @ W, 0.0)
    return pack(grads)
