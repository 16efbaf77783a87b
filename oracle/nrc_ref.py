"""CPU restatement of the neural radiance cache (TEST INFRASTRUCTURE ONLY).

numpy float64 forward and backward passes of the hash-grid encoding + MLP
implemented in kiraray_gb300/csrc/nrc.cu, used to check the CUDA path's
predictions and gradients.  `bf16=True` rounds at the same points as the GPU
(layer inputs, weights, backward operands) so that the comparison isolates
accumulation-order differences.
"""
from __future__ import annotations

import numpy as np

PRIME_Y, PRIME_Z = 2654435761, 805459861
IN, WIDTH, OUT_PAD = 64, 64, 16


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float values to bfloat16 (round to nearest even), as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


class Grid:
    def __init__(self, info, lo, hi, table_size):
        self.levels = info.n_levels
        self.res = [info.resolution[l] for l in range(self.levels)]
        self.offset = [info.level_offset[l] for l in range(self.levels)]
        self.size = [info.level_size[l] for l in range(self.levels)]
        self.table_size = table_size
        self.lo = np.asarray(lo, np.float32)
        ext = np.asarray(hi, np.float32) - self.lo
        self.inv = np.where(ext > 0, (1.0 / np.where(ext > 0, ext, 1)).astype(np.float32), 1.0)

    def corners(self, pos):
        """Per level: (indices [n, 8], weights [n, 8])."""
        p = np.clip((pos.astype(np.float32) - self.lo) * self.inv.astype(np.float32), 0, 1)
        out = []
        for l in range(self.levels):
            r = self.res[l]
            s = p * np.float32(r)
            fl = np.clip(np.floor(s), 0, r - 1)
            fr = np.clip(s - fl, 0, 1).astype(np.float64)
            base = fl.astype(np.int64)
            idx = np.zeros((p.shape[0], 8), np.int64)
            w = np.ones((p.shape[0], 8), np.float64)
            n1 = r + 1
            dense = n1 ** 3 <= self.table_size
            for k in range(8):
                x = base[:, 0] + (k & 1)
                y = base[:, 1] + ((k >> 1) & 1)
                z = base[:, 2] + ((k >> 2) & 1)
                if dense:
                    ii = x + n1 * (y + n1 * z)
                else:
                    ii = (x ^ ((y * PRIME_Y) & 0xFFFFFFFF) ^ ((z * PRIME_Z) & 0xFFFFFFFF)) & (self.table_size - 1)
                idx[:, k] = self.offset[l] + ii
                for a in range(3):
                    bit = (k >> a) & 1
                    w[:, k] *= fr[:, a] if bit else 1 - fr[:, a]
            out.append((idx, w))
        return out


class Mlp:
    def __init__(self, weights_flat: np.ndarray, layers: int):
        self.layers = layers
        self.W = []
        o = 0
        for l in range(layers):
            rows = WIDTH if l + 1 < layers else OUT_PAD
            self.W.append(weights_flat[o:o + rows * IN].reshape(rows, IN).astype(np.float64))
            o += rows * IN


BLOB_BINS = 4
EXTRA = 5 * BLOB_BINS + 3


def one_blob(s: np.ndarray) -> np.ndarray:
    c = (np.arange(BLOB_BINS) + 0.5) / BLOB_BINS
    d = (s[:, None] - c[None, :]) * BLOB_BINS
    return np.exp(-0.5 * d * d)


def spherical(v: np.ndarray):
    theta = np.arccos(np.clip(v[:, 2], -1, 1)) / np.pi
    phi = np.arctan2(v[:, 1], v[:, 0]) / (2 * np.pi) + 0.5
    return theta, phi


def encode_extras(inputs: np.ndarray) -> np.ndarray:
    """Normal and outgoing direction (spherical angles) and 1 - exp(-roughness)
    in one-blob encodings of 4 bins, albedo as is (the neural radiance
    caching input encoding)."""
    q = inputs.astype(np.float64)
    tn, pn = spherical(q[:, 3:6])
    tw, pw = spherical(q[:, 10:13])
    parts = [one_blob(tn), one_blob(pn), one_blob(tw), one_blob(pw), one_blob(1 - np.exp(-q[:, 6])),
             q[:, 7:10]]
    return np.concatenate(parts, axis=1)


def encode(grid: Grid, table: np.ndarray, inputs: np.ndarray, rounding=True):
    """Encoded inputs X0 [n, 64] and the corner data for the backward pass."""
    n = inputs.shape[0]
    tab = table.reshape(-1, 2).astype(np.float64)
    if rounding:
        tab = bf16(tab)
    X = np.zeros((n, IN))
    cs = grid.corners(inputs[:, :3])
    for l, (idx, w) in enumerate(cs):
        X[:, 2 * l] = (w * tab[idx, 0]).sum(1)
        X[:, 2 * l + 1] = (w * tab[idx, 1]).sum(1)
    o = 2 * grid.levels
    X[:, o:o + EXTRA] = encode_extras(inputs)
    if rounding:
        X = bf16(X)
    return X, cs


def forward(mlp: Mlp, X0: np.ndarray, rounding=True):
    acts = [X0]
    x = X0
    for l in range(mlp.layers):
        W = bf16(mlp.W[l]) if rounding else mlp.W[l]
        z = x @ W.T
        if l + 1 < mlp.layers:
            x = np.maximum(z, 0)
            if rounding:
                x = bf16(x)
            acts.append(x)
        else:
            return z[:, :3], acts


def loss_and_grad(y: np.ndarray, t: np.ndarray):
    n = y.shape[0]
    den = y * y + 0.01
    loss = ((y - t) ** 2 / den).sum() / (n * 3)
    g = 2 * (y - t) / den / (n * 3)
    return loss, g


def backward(mlp: Mlp, acts, dy: np.ndarray, rounding=True, loss_scale=128.0):
    """Gradients of the MLP weights (list per layer) and of X0."""
    n = dy.shape[0]
    d = np.zeros((n, OUT_PAD))
    d[:, :3] = dy * loss_scale
    grads = [None] * mlp.layers
    for l in range(mlp.layers - 1, -1, -1):
        dr = bf16(d) if rounding else d
        X = acts[l]
        grads[l] = dr.T @ X / loss_scale
        W = bf16(mlp.W[l]) if rounding else mlp.W[l]
        dX = dr @ W
        if l > 0:
            dX = dX * (X > 0)
        d = dX
    return grads, d / loss_scale


def table_grad(grid: Grid, cs, dX0: np.ndarray, n_entries: int) -> np.ndarray:
    g = np.zeros((n_entries, 2))
    for l, (idx, w) in enumerate(cs):
        for f in range(2):
            np.add.at(g[:, f], idx.reshape(-1), (w * dX0[:, 2 * l + f][:, None]).reshape(-1))
    return g.reshape(-1)
