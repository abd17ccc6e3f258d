"""CPU restatement of the learned empty-space predictor.  TEST INFRASTRUCTURE ONLY.

The reference renderer has no learned skipping (ray.c samples every lattice
point), so there is no reference code to pin this against.  Parity is
anchored instead on:
- the exact per-cell bound, which uses the index rule of the plain grid's
  empty-cell test (the test whose grid renders bitwise equal to the
  unskipped march, itself pinned to the reference);
- the analytic gradient below, checked against central finite differences
  in float64 by the CPU tests.

Network (parameters as one float32 vector of 6337, offsets below):
  h1 = relu(x W1 + b1)   x: 26 features zero-padded to 32, W1 [32][64]
  h2 = relu(h1 W2 + b2)  W2 [64 in][64 out]
  y  = h2 . w3 + b3
Loss per row with bound t: t > 0 -> w (y - t)^2, w = wneg if y < t else 1;
t <= 0 -> max(y + gamma, 0)^2.  Sum / n.

With ``emulate=True`` values are rounded to BF16 where the tensor-core
kernels hold BF16 operands (x, W1, W2, h1, dL/dh2, dL/dh1); everything else
is float64.
"""
from __future__ import annotations

import numpy as np

IN, HID, FEAT, KNOTS = 32, 64, 26, 16
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
NPARAMS = OFF_B3 + 1
GAMMA = 0.5
CELL = 16


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_bits(x) -> np.ndarray:
    return bf16(x).view(np.uint32) >> 16


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(IN, HID), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(HID, HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def _r(a, emulate):
    return bf16(a).astype(np.float64) if emulate else np.asarray(a, dtype=np.float64)


def forward(p, X, emulate=True):
    """y (float64 [n]) and the activations."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = _r(X, emulate)
    W1e, W2e = _r(W1, emulate), _r(W2, emulate)
    h1 = _r(np.maximum(x @ W1e + b1, 0.0), emulate)
    h2 = np.maximum(h1 @ W2e + b2, 0.0)
    y = h2 @ w3 + b3
    return y, (x, W1e, W2e, h1, h2)


def loss_grad(p, X, T, wneg, gamma=GAMMA, emulate=True):
    """(loss, gradient float64 [NPARAMS]) of the mean loss over the rows."""
    W1, b1, W2, b2, w3, b3 = unpack(p)
    T = np.asarray(T, dtype=np.float64)
    n = len(T)
    y, (x, W1e, W2e, h1, h2) = forward(p, X, emulate)
    pos = T > 0
    r = np.where(pos, y - T, np.maximum(y + gamma, 0.0))
    wt = np.where(pos & (r < 0), wneg, 1.0)
    loss = float(np.sum(wt * r * r) / n)
    dy = 2.0 * wt * r / n
    g = np.zeros(NPARAMS)
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    d2 = dy[:, None] * w3[None, :] * (h2 > 0)
    g[OFF_B2:OFF_W3] = d2.sum(axis=0)
    d2e = _r(d2, emulate)
    g[OFF_W2:OFF_B2] = (h1.T @ d2e).ravel()
    d1 = (d2e @ W2e.T) * (h1 > 0)
    g[OFF_B1:OFF_W2] = d1.sum(axis=0)
    d1e = _r(d1, emulate)
    g[OFF_W1:OFF_B1] = (x.T @ d1e).ravel()
    return loss, g


def lut_index(v, scale, off, n):
    """(int)(v*scale) - off clamped to [0, n-1] for float32 v."""
    i = np.trunc(np.float32(v) * np.float32(scale)).astype(np.int64) - off
    return np.clip(i, 0, n - 1)


def bound(lo, hi, lut, off, scale):
    """Exact post-TF bound of a cell with value range [lo, hi]: the largest
    LUT opacity over the indices [(int)(lo*s)-1-off, (int)(hi*s)+1-off]."""
    n = len(lut)
    a = np.clip(np.trunc(np.float32(lo) * np.float32(scale)).astype(np.int64) - 1 - off, 0, n - 1)
    b = np.clip(np.trunc(np.float32(hi) * np.float32(scale)).astype(np.int64) + 1 - off, 0, n - 1)
    return float(lut[a:b + 1, 3].max())


def knots(lut):
    """16-knot encoding over 16 knots evenly spaced on the LUT's entries
    (entry k (n-1)/15): feature k < 15 = the largest opacity between knots k
    and k + 1 (entries floor(k (n-1)/15) .. ceil((k+1) (n-1)/15)), feature 15
    = the largest opacity of the LUT."""
    n = len(lut)
    last = KNOTS - 1
    out = np.zeros(KNOTS, np.float32)
    for k in range(last):
        a, b = k * (n - 1) // last, ((k + 1) * (n - 1) + last - 1) // last
        out[k] = lut[a:b + 1, 3].max()
    out[last] = lut[:, 3].max()
    return out


def cell_grid(nx, ny, nz, cell=CELL):
    """Macrocell grid dims of an nx x ny x nz brick: cells of `cell` voxel
    spacings (16 by default), each with its +1 layer."""
    return (nx - 2) // cell + 1, (ny - 2) // cell + 1, (nz - 2) // cell + 1


def features(vol, lut, off, scale, cell=CELL):
    """Features (float32 holding BF16 values, [n][32]) and bounds ([n]) of
    every macrocell (edge `cell`) of a one-brick volume, cells x fastest."""
    v = np.asarray(vol).astype(np.float32)
    nz, ny, nx = v.shape
    vmin, vmax = np.float32(v.min()), np.float32(v.max())
    mcx, mcy, mcz = cell_grid(nx, ny, nz, cell)
    kn = knots(lut)
    inv = np.float32(1.0) / (vmax - vmin) if vmax > vmin else np.float32(0.0)
    hscale = np.float32(8.0) / (vmax - vmin) if vmax > vmin else np.float32(0.0)
    X = np.zeros((mcx * mcy * mcz, IN), np.float32)
    T = np.zeros(mcx * mcy * mcz, np.float32)
    c = 0
    for cz in range(mcz):
        for cy in range(mcy):
            for cx in range(mcx):
                x0, y0, z0 = cx * cell, cy * cell, cz * cell
                blk = v[z0:min(z0 + cell, nz - 1) + 1, y0:min(y0 + cell, ny - 1) + 1, x0:min(x0 + cell, nx - 1) + 1]
                lo, hi = blk.min(), blk.max()
                bins = np.clip(np.trunc((blk - vmin) * hscale).astype(np.int64), 0, 7)
                hist = np.bincount(bins.ravel(), minlength=8).astype(np.float32) / np.float32(blk.size)
                row = np.zeros(IN, np.float32)
                row[0] = (lo - vmin) * inv
                row[1] = (hi - vmin) * inv
                row[2:10] = hist
                row[10:26] = kn
                X[c] = bf16(row)
                T[c] = bound(lo, hi, lut, off, scale)
                c += 1
    return X, T
