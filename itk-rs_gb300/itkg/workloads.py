"""Seeded synthetic inputs with the shapes and value distributions of the
workloads this path is measured and tested on.  The reference publishes no
dataset for its Gaussian path; these generators stand in for one.

  blobs_volume   Image<f32,3>: a sum of seeded Gaussian blobs plus N(0, noise)
                 (the 256^3 sigma 2 forward, the 192^3 multi-scale VJP stack)
  ct_volume      Image<i16,3>: a CT-like volume of seeded constant ellipsoids in
                 [-1000, 1500] plus N(0, 20), rounded and saturated to i16
  uniform_image  U[0, 1) f32 (the 2-D 512^2 sigma 1.5 forward)

Arrays are numpy, axis order (z, y, x): axis 0 of the image (x) is the last,
fastest-varying numpy axis.
"""
from __future__ import annotations

import numpy as np


def blobs_volume(shape, seed, nblobs=32, noise=0.05):
    """Sum of `nblobs` seeded Gaussian blobs (centres uniform in the volume,
    amplitude U[0.5, 2], std U[4, 24] voxels) plus N(0, noise)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z = np.arange(nz, dtype=np.float32)[:, None, None]
    y = np.arange(ny, dtype=np.float32)[None, :, None]
    x = np.arange(nx, dtype=np.float32)[None, None, :]
    vol = np.zeros(shape, np.float32)
    for _ in range(nblobs):
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        amp = rng.uniform(0.5, 2.0)
        sd = rng.uniform(4.0, 24.0)
        k = np.float32(-0.5 / (sd * sd))
        gz = np.exp(k * (z - cz) ** 2)
        gy = np.exp(k * (y - cy) ** 2)
        gx = np.exp(k * (x - cx) ** 2)
        vol += np.float32(amp) * (gz * gy * gx)
    vol += rng.normal(0.0, noise, shape).astype(np.float32)
    return vol


def ct_volume(shape=(384, 512, 512), seed=0, n_ellipsoids=12):
    """CT-like i16 volume: air (-1000) with `n_ellipsoids` seeded ellipsoids of
    constant value U[-1000, 1500], plus N(0, 20), rounded and saturated."""
    rng = np.random.default_rng(seed)
    z = np.arange(shape[0])[:, None, None]
    y = np.arange(shape[1])[None, :, None]
    x = np.arange(shape[2])[None, None, :]
    vol = np.full(shape, -1000.0, np.float32)
    for _ in range(n_ellipsoids):
        c = rng.uniform(0.2, 0.8, 3) * np.array(shape)
        ax = rng.uniform(0.05, 0.35, 3) * np.array(shape)
        val = rng.uniform(-1000, 1500)
        m = ((z - c[0]) / ax[0]) ** 2 + ((y - c[1]) / ax[1]) ** 2 + ((x - c[2]) / ax[2]) ** 2 <= 1
        vol[m] = val
    vol += rng.normal(0, 20, shape).astype(np.float32)
    return np.clip(np.rint(vol), -32768, 32767).astype(np.int16)


def uniform_image(shape, seed=0):
    """i.i.d. U[0, 1) f32 pixels from `seed`."""
    return np.random.default_rng(seed).random(shape, dtype=np.float32)


def registration_pair(shape=(512, 512), seed=0, margin=24, nblobs=40, shift=(1.5, -1.0)):
    """Fixed / moving Image<f32,2> for the demons registrations: `nblobs`
    seeded cones (radius U[6, 14]) and the same cones shifted by `shift`
    pixels, zero within `margin` of the edges (there the field stays zero, so
    no warped index leaves the image, where the reference panics)."""
    rng = np.random.default_rng(seed)
    h, w = shape
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    f = np.zeros(shape)
    m = np.zeros(shape)
    for _ in range(nblobs):
        r = rng.uniform(6, 14)
        cy, cx = rng.uniform(margin + r, h - margin - r), rng.uniform(margin + r, w - margin - r)
        f += np.maximum(0.0, 1.0 - np.hypot(xx - cx, yy - cy) / r)
        m += np.maximum(0.0, 1.0 - np.hypot(xx - cx - shift[0], yy - cy - shift[1]) / r)
    return f.astype(np.float32), m.astype(np.float32)


def biased_image(shape=(512, 512), seed=0):
    """Image<f32,2> for the bias-field correction: a two-level seeded phantom
    (ellipses of 120 on 60) times a smooth multiplicative bias, plus N(0, 2)."""
    rng = np.random.default_rng(seed)
    h, w = shape
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    bias = 1.0 + 0.4 * (xx / w) - 0.2 * (yy / h) + 0.1 * np.sin(xx / 40.0)
    base = np.full(shape, 60.0)
    for _ in range(5):
        cy, cx = rng.uniform(0.2, 0.8) * h, rng.uniform(0.2, 0.8) * w
        ay, ax = rng.uniform(0.05, 0.25) * h, rng.uniform(0.05, 0.25) * w
        base[((yy - cy) / ay) ** 2 + ((xx - cx) / ax) ** 2 < 1.0] = 120.0
    return (base * bias + rng.normal(0, 2, shape)).astype(np.float32)
