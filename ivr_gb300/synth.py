"""Seeded synthetic volumes and transfer functions for the benchmark workloads.

The reference's datasets (skull.vol, vel_grid_*.bin, vizwoman8.dat) are not
available, so every workload runs on seeded synthetic inputs with the shapes
and value distributions below.  Volumes are x-fastest arrays of shape
(d, h, w), the reference's voxel order (mathutil.h:139-143).

* ``blob_volume``: a sum of isotropic Gaussian blobs (centres uniform in
  [0.2, 0.8]^3, sigma uniform 0.03-0.12 of the largest dimension, amplitude
  uniform 0.3-1.0), optional multi-octave value noise and uniform noise,
  clamped to [0, 1] and scaled to the dtype's range (u8: 0-255, u16:
  0-65535, f32: 0-255 so that LUT indices are the value's integer part).
* ``ramp_tf``: 256-entry RGBA FP32 transfer function, opacity 0 below 0.2 and
  a linear ramp to 0.8 at 1.0, hue ramp blue -> red.
* ``knot_tf``: random piecewise-linear transfer function with 16 knots.

Small volumes are generated with numpy; large ones on the GPU with torch
when it is available (generation only; nothing here is on the render path).
"""
from __future__ import annotations

import numpy as np

DT_MAX = {"u8": 255.0, "u16": 65535.0, "f32": 255.0}
NP_DT = {"u8": np.uint8, "u16": np.uint16, "f32": np.float32}


def _blob_params(rng, n_blobs, sigma_scale=1.0):
    c = rng.uniform(0.2, 0.8, size=(n_blobs, 3))
    s = rng.uniform(0.03, 0.12, size=n_blobs) * sigma_scale
    a = rng.uniform(0.3, 1.0, size=n_blobs)
    return c, s, a


def _axis(n, maxdim):
    # normalised coordinate of voxel centres, scaled by the largest dimension
    return (np.arange(n, dtype=np.float64) + 0.5) / maxdim


def _value_noise_np(rng, shape, octaves):
    d, h, w = shape
    out = np.zeros(shape, dtype=np.float32)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        f = 4 * (2 ** o)
        g = rng.uniform(-1.0, 1.0, size=(f + 1, f + 1, f + 1)).astype(np.float32)
        idx, frac = [], []
        for n in (d, h, w):  # lattice coordinate of each voxel along the axis
            u = np.linspace(0, f, n)
            i0 = np.minimum(np.floor(u).astype(np.int64), f - 1)
            idx.append(i0)
            frac.append((u - i0).astype(np.float32))
        kz, ky, kx = np.ix_(*idx)
        fz, fy, fx = frac[0][:, None, None], frac[1][None, :, None], frac[2][None, None, :]
        acc = np.zeros(shape, dtype=np.float32)
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    wgt = (fz if dz else 1 - fz) * (fy if dy else 1 - fy) * (fx if dx else 1 - fx)
                    acc += wgt * g[kz + dz, ky + dy, kx + dx]
        out += amp * acc
        total += amp
        amp *= 0.5
    return out / total


def blob_volume(shape, n_blobs=8, seed=0, dtype="u8", noise=0.05, value_noise=0.0,
                octaves=3, zero_fraction=0.0, cell=16, device=None, sigma_scale=1.0):
    """Sum of Gaussian blobs, see the module docstring.  ``zero_fraction``
    zeroes every voxel below the threshold that makes that fraction of the
    ``cell``^3 macrocells exactly zero.  ``sigma_scale`` multiplies every
    blob's sigma: (8 / n_blobs)^(1/3) keeps hundreds of blobs from summing
    to a saturated volume (whose cell maxima are all 1, leaving no threshold
    for the zero cells)."""
    d, h, w = shape
    rng = np.random.default_rng(seed)
    c, s, a = _blob_params(rng, n_blobs, sigma_scale)
    maxdim = float(max(shape))
    use_torch = device is not None
    if use_torch:
        import torch
        dev = torch.device(device)
        vol = torch.zeros((d, h, w), dtype=torch.float32, device=dev)
        ax = [torch.from_numpy(_axis(n, maxdim)).to(dev) for n in (w, h, d)]
        for b in range(n_blobs):
            g = [torch.exp(-((ax[i] - c[b, i] * (shape[2 - i] / maxdim)) ** 2) / (2 * s[b] ** 2)).float()
                 for i in range(3)]
            vol += float(a[b]) * g[2][:, None, None] * g[1][None, :, None] * g[0][None, None, :]
        if value_noise > 0:
            import torch.nn.functional as F
            gen = torch.Generator(device="cpu").manual_seed(seed + 1)
            amp, total, vn = 1.0, 0.0, torch.zeros_like(vol)
            for o in range(octaves):
                f = 4 * (2 ** o)
                g = (torch.rand((1, 1, f + 1, f + 1, f + 1), generator=gen) * 2 - 1).to(dev)
                vn += amp * F.interpolate(g, size=(d, h, w), mode="trilinear", align_corners=True)[0, 0]
                total += amp
                amp *= 0.5
            vol += value_noise * vn / total
        if noise > 0:
            gen = torch.Generator(device=dev).manual_seed(seed + 2)
            vol += (torch.rand((d, h, w), generator=gen, device=dev) * 2 - 1) * noise
        vol.clamp_(0.0, 1.0)
        if zero_fraction > 0:
            vol = _zero_cells_torch(vol, zero_fraction, cell)
        vol = vol * DT_MAX[dtype]
        if dtype == "f32":
            return vol.cpu().numpy()
        return vol.round().to(torch.int32).cpu().numpy().astype(NP_DT[dtype])

    vol = np.zeros((d, h, w), dtype=np.float32)
    axes = [_axis(n, maxdim) for n in (w, h, d)]
    for b in range(n_blobs):
        g = [np.exp(-((axes[i] - c[b, i] * (shape[2 - i] / maxdim)) ** 2) / (2 * s[b] ** 2)).astype(np.float32)
             for i in range(3)]
        vol += np.float32(a[b]) * g[2][:, None, None] * g[1][None, :, None] * g[0][None, None, :]
    if value_noise > 0:
        vol += np.float32(value_noise) * _value_noise_np(np.random.default_rng(seed + 1), shape, octaves)
    if noise > 0:
        vol += np.random.default_rng(seed + 2).uniform(-noise, noise, size=shape).astype(np.float32)
    np.clip(vol, 0.0, 1.0, out=vol)
    if zero_fraction > 0:
        vol = _zero_cells_np(vol, zero_fraction, cell)
    vol = vol * np.float32(DT_MAX[dtype])
    if dtype == "f32":
        return vol.astype(np.float32)
    return np.rint(vol).astype(NP_DT[dtype])


def _cell_max_np(vol, cell):
    d, h, w = vol.shape
    pd, ph, pw = (-d) % cell, (-h) % cell, (-w) % cell
    v = np.pad(vol, ((0, pd), (0, ph), (0, pw)))
    D, H, W = v.shape
    return v.reshape(D // cell, cell, H // cell, cell, W // cell, cell).max(axis=(1, 3, 5))


def _zero_cells_np(vol, frac, cell):
    cm = _cell_max_np(vol, cell)
    t = np.float32(np.quantile(cm, frac))
    return np.where(vol <= t, np.float32(0.0), vol).astype(np.float32)


def _zero_cells_torch(vol, frac, cell):
    import torch
    import torch.nn.functional as F
    cm = F.max_pool3d(vol[None, None], kernel_size=cell, stride=cell, ceil_mode=True)[0, 0]
    t = torch.quantile(cm.flatten().float().cpu(), frac).item()
    return torch.where(vol <= t, torch.zeros_like(vol), vol)


def _hue_blue_to_red(x):
    """Hue ramp: blue (x=0) -> cyan -> green -> yellow -> red (x=1)."""
    r = np.clip(np.minimum(4 * x - 1.5, -4 * x + 4.5), 0, 1)
    g = np.clip(np.minimum(4 * x - 0.5, -4 * x + 3.5), 0, 1)
    b = np.clip(np.minimum(4 * x + 0.5, -4 * x + 2.5), 0, 1)
    # map x in [0,1] onto the 1/8..7/8 band of that ramp: blue .. red
    return r, g, b


def ramp_tf(n=256):
    """256-entry RGBA FP32: opacity 0 below 0.2, linear to 0.8 at 1.0,
    hue blue -> red.  Returns float32 array (n, 4)."""
    x = np.arange(n, dtype=np.float64) / (n - 1)
    a = np.where(x < 0.2, 0.0, 0.8 * (x - 0.2) / 0.8)
    hx = 0.125 + 0.75 * x
    r, g, b = _hue_blue_to_red(hx)
    return np.stack([r, g, b, a], axis=1).astype(np.float32)


def knot_tf(seed, n=256, knots=16, zero_frac=0.6, zero_first=False):
    """Random piecewise-linear TF: 16 knots evenly spaced on [0,1], opacity
    knots uniform in [0,1] with ``zero_frac`` of them zeroed, colour from the
    blue -> red hue ramp.  ``zero_first`` zeroes the first two knots: the
    lowest fifteenth of the range, and with it the empty background, is
    transparent.  Returns (lut float32 (n,4), knot opacities (16,))."""
    rng = np.random.default_rng(seed)
    ka = rng.uniform(0.0, 1.0, size=knots)
    ka[rng.uniform(size=knots) < zero_frac] = 0.0
    if zero_first:
        ka[:2] = 0.0
    kx = np.linspace(0.0, 1.0, knots)
    x = np.arange(n, dtype=np.float64) / (n - 1)
    a = np.interp(x, kx, ka)
    r, g, b = _hue_blue_to_red(0.125 + 0.75 * x)
    return np.stack([r, g, b, a], axis=1).astype(np.float32), ka.astype(np.float32)
