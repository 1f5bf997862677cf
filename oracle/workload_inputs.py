"""Seeded host (NumPy/SciPy) inputs of the benchmark workload family, for the
golden solves that the reference's own code runs on NumPy and for the
reference's CPU timing.

Test infrastructure, like the rest of oracle/: `tests/golden/make_golden.py`
feeds these arrays to the reference's `multiscale_correlate_gpu(xp=numpy)`,
the GPU tests regenerate the very same arrays from the seeds and feed them
to this package's solver, and the benchmark's CPU leg times the reference's
operators on them.  Each golden stores a SHA-256 digest of its inputs so a
test can tell whether the regenerated bytes are the ones the reference saw.

Texture: Gaussian-filtered white noise (sigma 2 vx) plus bright randomly
oriented cylinders (radius 3 vx, length 40 vx), normalised to [0, 1].
Deformed image: g(x) = f(x - u(x)) (order-1 interpolation, clamped at the
border) + N(0, sigma_n^2).  Volumes are n*h + 1 voxels per axis.

Fields:
  * plain_small: u = (0.5, -0.3, 0.2) + diag(-0.004, -0.004, 0.01) (x - c):
    1 % uniaxial z strain with 0.4 Poisson contraction and a translation.
  * necking: u_z = 0.02 z plus a Gaussian-profile radial contraction of up
    to 3 vx at mid-height (profile width 64 n / 513 vx).
"""
from __future__ import annotations

import hashlib

import numpy as np


def cylinders(n, shape, radius=3.0, length=40.0, seed=2):
    """(n, 8) float64: centre uniform in the volume, direction uniform on the
    sphere, radius, half length."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)) * (np.array(shape) - 1)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([c, d, np.full((n, 1), radius), np.full((n, 1), length / 2)], axis=1)


def texture(shape, n_cyl, seed=0, cyl_seed=2, sigma=2.0, noise_amp=0.15):
    """float32 volume pix[x, y, z] (C order) in [0, 1]."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    t = gaussian_filter(rng.standard_normal(shape), sigma, mode="nearest", truncate=4.0)
    t = 0.5 + noise_amp * t / t.std()
    for cx, cy, cz, dx, dy, dz, rad, hl in cylinders(n_cyl, shape, seed=cyl_seed):
        ext = [hl * abs(d) + rad + 1.0 for d in (dx, dy, dz)]
        lo = [max(0, int(np.floor(c - e))) for c, e in zip((cx, cy, cz), ext)]
        hi = [min(s - 1, int(np.ceil(c + e))) for c, e, s in zip((cx, cy, cz), ext, shape)]
        if any(h < l for l, h in zip(lo, hi)):
            continue
        X, Y, Z = np.meshgrid(*[np.arange(l, h + 1, dtype=np.float64) for l, h in zip(lo, hi)], indexing="ij")
        px, py, pz = X - cx, Y - cy, Z - cz
        ax = px * dx + py * dy + pz * dz
        rho = np.sqrt(np.maximum(px * px + py * py + pz * pz - ax * ax, 0.0))
        val = np.clip(rad + 0.5 - rho, 0.0, 1.0) * np.clip(hl + 0.5 - np.abs(ax), 0.0, 1.0)
        sl = tuple(slice(l, h + 1) for l, h in zip(lo, hi))
        t[sl] = np.maximum(t[sl], val)
    t = (t - t.min()) / (t.max() - t.min())
    return t.astype(np.float32)


def field_plain_small(X, Y, Z, c=64.0):
    return (0.5 - 0.004 * (X - c), -0.3 - 0.004 * (Y - c), 0.2 + 0.01 * (Z - c))


def field_necking(X, Y, Z, n):
    zc = xc = yc = (n - 1) / 2.0
    s, R = 64.0 * n / 513.0, (n - 1) / 2.0
    gz = 3.0 * np.exp(-(Z - zc) ** 2 / (2 * s * s)) / R
    return (-gz * (X - xc), -gz * (Y - yc), 0.02 * Z)


def warp(f, field, noise=0.01, seed=1):
    """g(x) = f(x - u(x)) + N(0, noise^2), float32, same shape as f."""
    from scipy.ndimage import map_coordinates
    shp = f.shape
    g = np.empty(shp, np.float64)
    rng = np.random.default_rng(seed)
    # slab by slab along z to bound the coordinate arrays' memory
    step = max(1, (1 << 22) // (shp[0] * shp[1]))
    for z0 in range(0, shp[2], step):
        z1 = min(shp[2], z0 + step)
        X, Y, Z = np.meshgrid(np.arange(shp[0], dtype=np.float64), np.arange(shp[1], dtype=np.float64),
                              np.arange(z0, z1, dtype=np.float64), indexing="ij")
        u = field(X, Y, Z)
        coords = np.stack([X - u[0], Y - u[1], Z - u[2]])
        g[:, :, z0:z1] = map_coordinates(f.astype(np.float64), coords, order=1, mode="nearest")
    g += noise * rng.standard_normal(shp)
    return g.astype(np.float32)


def plain_small(n=129):
    """129^3, 200 cylinders, affine field; h = 16 (8^3 elements)."""
    f = texture((n, n, n), 200)
    return f, warp(f, field_plain_small)


def necking(n=129):
    """n^3 replica of the 513^3 tensile-necking workload (cylinder count
    scaled with the volume), h = 8."""
    f = texture((n, n, n), int(round(5000 * (n / 513.0) ** 3)))
    return f, warp(f, lambda X, Y, Z: field_necking(X, Y, Z, n))


CASES = {"plain_small": plain_small, "necking_129": lambda: necking(129), "necking_257": lambda: necking(257),
         "necking_513": lambda: necking(513)}


def digest(f, g):
    return hashlib.sha256(np.ascontiguousarray(f).tobytes() + np.ascontiguousarray(g).tobytes()).hexdigest()
