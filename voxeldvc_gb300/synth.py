"""Seeded synthetic DVC workloads, generated on the GPU (include/vdvc_synth.h).

Textures: Gaussian-filtered white noise (sigma 2 vx) plus bright randomly
oriented cylinders (radius 3 vx, length 40 vx) mimicking a fiber
composite, normalised to [0,1].  Deformed images: g(x) = f(x - u(x)) +
N(0, sigma_n^2) for analytic fields u.  Volumes are snapped to n*h + 1
voxels so the Hex8 mesh covers them exactly.

Seeds: texture noise 0, cylinder placement 2, deformed-image noise 1.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _device as D
from . import _lib

FIELD_AFFINE, FIELD_NECKING, FIELD_AFFINE_SIN, FIELD_BUMPS = 0, 1, 2, 3

def _L():
    return _lib.lib()


def cylinders(n, shape, radius=3.0, length=40.0, seed=2):
    """(n, 8) float32: centre uniform in the volume, direction uniform on
    the sphere, radius, half length."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3)) * (np.array(shape) - 1)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.concatenate([c, d, np.full((n, 1), radius), np.full((n, 1), length / 2)], axis=1)
    return out.astype(np.float32)


def texture(shape, n_cyl, seed=0, sigma=2.0, noise_amp=0.15, cyl_value=1.0, cyl_seed=2):
    """Texture volume in vox layout (float32 CUDA tensor, x fastest)."""
    L = _L()
    nx, ny, nz = shape
    out = D.empty(nx * ny * nz, np.float32)
    cyl = D.to_device(cylinders(n_cyl, shape, seed=cyl_seed)) if n_cyl else None
    nb = L.vdvc_synth_workspace_bytes(nx, ny, nz)
    ws = D.torch().empty(nb, dtype=D.torch().uint8, device=D.device())
    _lib.check(L.vdvc_synth_texture(out.data_ptr(), nx, ny, nz, seed, sigma, noise_amp, D.ptr(cyl), n_cyl,
                                    cyl_value, ws.data_ptr(), nb, D.stream()), "synth_texture")
    return out


def warp(f_vox, shape, field_kind, params, noise_sigma=0.01, seed=1):
    L = _L()
    nx, ny, nz = shape
    g = D.empty(nx * ny * nz, np.float32)
    p = np.ascontiguousarray(params, dtype=np.float64)
    _lib.check(L.vdvc_synth_warp(f_vox.data_ptr(), nx, ny, nz, field_kind, p.ctypes.data_as(_lib.pd), p.size,
                                 noise_sigma, seed, g.data_ptr(), D.stream()), "synth_warp")
    return g


def vox_to_pix(vox, shape):
    """vox layout -> pix[x,y,z] C-order device tensor (a layout copy)."""
    nx, ny, nz = shape
    return vox.view(nz, ny, nx).permute(2, 1, 0).contiguous()


def field_at(kind, params, X):
    """Analytic u at points X (n, 3), float64 host -- the true field."""
    p = np.asarray(params, dtype=np.float64)
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    if kind == FIELD_NECKING:
        ez, a, zc, s, xc, yc, R = p[:7]
        gz = a * np.exp(-(z - zc) ** 2 / (2 * s * s)) / R
        return np.stack([-gz * (x - xc), -gz * (y - yc), ez * z], 1)
    G = p[3:12].reshape(3, 3)
    u = p[:3][None, :] + (X - p[12:15][None, :]) @ G.T
    if kind == FIELD_AFFINE_SIN:
        amp, wl = p[15], p[16]
        for k in range(3):
            u[:, k] += amp * np.sin(2 * np.pi * X[:, (k + 1) % 3] / wl)
    if kind == FIELD_BUMPS:
        for b in range(int(p[15])):
            q = p[16 + 7 * b: 23 + 7 * b]
            e = np.exp(-np.sum((X - q[None, :3]) ** 2, axis=1) / (2 * q[3] ** 2))
            u += e[:, None] * q[None, 4:7]
    return u


def field_grid(kind, params, grid, stride):
    """u at the grid points (i, j, k) * stride on the GPU: float32 CUDA
    tensor (gx*gy*gz, 3), x fastest."""
    gx, gy, gz = grid
    out = D.empty(gx * gy * gz * 3, np.float32)
    p = np.ascontiguousarray(params, dtype=np.float64)
    _lib.check(_L().vdvc_synth_field_grid(kind, p.ctypes.data_as(_lib.pd), p.size, gx, gy, gz, float(stride),
                                          out.data_ptr(), D.stream()), "synth_field_grid")
    return out.view(-1, 3)


@dataclass
class Workload:
    name: str
    shape: tuple
    h: int
    n_cyl: int
    field: int
    params: list
    noise: float = 0.01
    solve: dict = field(default_factory=dict)
    storage: str = "f32"  # "u16": both images quantised to 0..65535

    @property
    def mesh(self):
        return tuple((s - 1) // self.h for s in self.shape)

    def make(self):
        """(f_pix, g_pix) CUDA tensors in pix[x,y,z] layout: float32, or
        uint16 counts (texture and noise scaled by 65535) for "u16"."""
        f = texture(self.shape, self.n_cyl)
        g = warp(f, self.shape, self.field, self.params, self.noise)
        fp, gp = vox_to_pix(f, self.shape), vox_to_pix(g, self.shape)
        if self.storage == "u16":
            fp, gp = _to_u16(fp), _to_u16(gp)
        return fp, gp

    def true_U(self):
        """True nodal displacement (Ndof,) float64 in the correlation's sense:
        g(x + U(x)) = f(x).  With g(y) = f(y - u(y)) that is the fixed point
        U(x) = u(x + U(x)) (a contraction for |grad u| < 1), which differs
        from u(x) by about |grad u| |u|."""
        Nx, Ny, Nz = self.mesh
        nn = np.arange((Nx + 1) * (Ny + 1) * (Nz + 1))
        X = np.stack([nn % (Nx + 1), (nn // (Nx + 1)) % (Ny + 1), nn // ((Nx + 1) * (Ny + 1))], 1) * float(self.h)
        return inverse_field(self.field, self.params, X).reshape(-1)


def _to_u16(t):
    """[0, 1] float32 -> uint16 counts (round to nearest, clamp); int32 where
    this torch has no uint16 casts (the solver reads either)."""
    T = D.torch()
    q = (t * 65535.0).round_().clamp_(0, 65535).to(T.int32)
    try:
        return q.to(T.uint16)
    except (AttributeError, RuntimeError, TypeError):
        return q


def large_1024(seed=5):
    """1025^3 uint16 pair, 40000 cylinders: an affine map (3 degree rotation
    about a seeded random axis, 20 vx translation, 0.5 % shear) composed
    with a sinusoidal field of amplitude 1.5 vx and wavelength 128 vx, noise
    1 % of the range; h = 8 (128^3 elements, 6,440,067 dof), 4-level
    pyramid (scales 3, 2, 1, 0) seeded by the FFT shift and the affine
    prealign, Laplacian regulariser l0 = 4.5 h, precision form."""
    rng = np.random.default_rng(seed)
    axis = rng.standard_normal(3)
    axis /= np.linalg.norm(axis)
    th = np.deg2rad(3.0)
    Kx = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx
    shear = np.zeros((3, 3))
    shear[0, 2] = 0.005
    G = R + shear - np.eye(3)
    t = 20.0 * axis[[1, 2, 0]] / np.linalg.norm(axis)
    c = 512.0
    params = [*t, *G.reshape(-1), c, c, c, 1.5, 128.0]
    return Workload("affine_sin_1025^3_h8_u16", (1025, 1025, 1025), 8, 40000, FIELD_AFFINE_SIN, params, noise=0.01,
                    solve=dict(reg_type='laplacian', l0=4.5 * 8, scales=(3, 2, 1, 0), prealign_affine=True,
                               precision="mixed"), storage="u16")


def plain_small():
    """129^3, 200 cylinders, 1 % z strain with 0.4 Poisson contraction plus a
    (0.5, -0.3, 0.2) vx translation; h = 16, Laplacian with l0 = 2h,
    3-level pyramid."""
    c = 64.0
    G = np.diag([-0.004, -0.004, 0.01]).reshape(-1)
    params = [0.5, -0.3, 0.2, *G, c, c, c]
    return Workload("plain_small_129^3_h16", (129, 129, 129), 16, 200, FIELD_AFFINE, params,
                    solve=dict(reg_type='laplacian', l0=2 * 16, scales=(2, 1, 0)))


def _necking(n, reg):
    params = [0.02, 3.0, (n - 1) / 2, 64.0 * n / 513, (n - 1) / 2, (n - 1) / 2, (n - 1) / 2]
    solve = dict(reg_type=reg, l0=4.5 * 8, scales=(2, 1, 0))
    if reg == 'equilibrium_gap':
        solve.update(reg_exponent=4, nu=0.3)
    tag = "" if reg == 'laplacian' else "_eqgap"
    return Workload(f"necking_{n}^3_h8{tag}", (n, n, n), 8, int(round(5000 * (n / 513) ** 3)), FIELD_NECKING, params,
                    solve=solve)


def necking_512():
    """513^3, 5000 cylinders, tensile necking: u_z = 0.02 z plus a
    Gaussian-profile radial contraction of up to 3 vx at mid-height (profile
    width s = 64 vx); h = 8 (64^3 elements, 823,875 dof), 3-level pyramid,
    Laplacian regularizer with l0 = 4.5 h (the `voxeldvc run` settings)."""
    return _necking(513, 'laplacian')


def necking_512_eqgap():
    """necking_512 with the equilibrium-gap regularizer (nu = 0.3,
    reg_exponent 4).  The reference algorithm does not converge on this
    pyramid (its coarse levels diverge); kept for the parity checks."""
    return _necking(513, 'equilibrium_gap')


def necking_256():
    """necking_512 scaled to 257^3 (h = 8, 32^3 elements): the profiling case."""
    return _necking(257, 'laplacian')


def series_385(n_steps=16, seed=3):
    """A load series against one reference: a 385^3 reference (2000
    cylinders), n_steps deformed images under uniaxial strain
    eps_z = 0.2 % ... 3.2 % (Poisson contraction 0.4 eps in x and y, about the
    volume centre, plus a 0.5 eps x 100 vx rigid drift in z), and one ROI
    per step with edges drawn uniformly in [256, 384] voxels, snapped to
    n h + 1 for h drawn from {8, 12, 16}, placed uniformly inside the
    volume.  Returns (f_pix, [g_pix], problems, true fields (callables))."""
    shape = (385, 385, 385)
    rng = np.random.default_rng(seed)
    f = texture(shape, 2000, seed=seed, cyl_seed=seed + 1)
    gs, problems, fields = [], [], []
    c = (shape[0] - 1) / 2.0
    for k in range(n_steps):
        ez = 0.002 * (k + 1)
        params = [0.0, 0.0, 50.0 * ez, *np.diag([-0.4 * ez, -0.4 * ez, ez]).reshape(-1), c, c, c]
        g = warp(f, shape, FIELD_AFFINE, params, 0.01, seed=seed + 100 + k)
        gs.append(vox_to_pix(g, shape))
        h = int(rng.choice([8, 12, 16]))
        mesh, origin = [], []
        for ax in range(3):
            edge = int(rng.integers(256, 385))
            n_el = max(1, (edge - 1) // h)
            mesh.append(n_el)
            origin.append(int(rng.integers(0, shape[ax] - (n_el * h + 1) + 1)))
        problems.append(dict(origin=tuple(origin), h=h, mesh=tuple(mesh)))
        fields.append((FIELD_AFFINE, params))
    return vox_to_pix(f, shape), gs, problems, fields


def inverse_field(kind, params, X, iters=60, tol=1e-10):
    """U at points X with U = u(X + U): the displacement a correlation of
    f against g(y) = f(y - u(y)) recovers (fixed-point iteration)."""
    U = field_at(kind, params, X)
    for _ in range(iters):
        U_new = field_at(kind, params, X + U)
        done = np.max(np.abs(U_new - U)) < tol
        U = U_new
        if done:
            break
    return U


def true_U_problem(problem, field):
    """True nodal displacement of a series problem (ROI frame)."""
    kind, params = field
    h = problem["h"]
    Nx, Ny, Nz = problem["mesh"]
    o = np.asarray(problem["origin"], np.float64)
    nn = np.arange((Nx + 1) * (Ny + 1) * (Nz + 1))
    X = np.stack([nn % (Nx + 1), (nn // (Nx + 1)) % (Ny + 1), nn // ((Nx + 1) * (Ny + 1))], 1) * float(h) + o
    return inverse_field(kind, params, X).reshape(-1)


WORKLOADS = {"plain_small": plain_small, "necking_512": necking_512, "necking_512_eqgap": necking_512_eqgap,
             "necking_256": necking_256, "large_1024": large_1024}


# ---- known-answer (ground-truth) stand-ins ---------------------------------
# Seeded substitutes for a 65^3 uint16 reference volume and its (66^3, 3)
# float32 displacement sampled at the integer coordinates 0..65: a speckle
# volume with mean 32112, std 6270, clipped to [15192, 58729], and a uniaxial
# z strain eps with lateral contraction nu eps plus a smooth non-affine part.
# "z+0.01" is +1 % tension (u_z 0 -> 0.65 vx), "z-0.05" -5 % compression
# (u_z 0 -> -3.25 vx).  Generated with numpy / scipy on the host so the
# oracle and the GPU pipeline see the same bytes.
GT_KINDS = {"z+0.01": (0.01, 0.3), "z-0.05": (-0.05, 0.26)}


def gt_stand_in(kind="z+0.01", n=65, seed=11):
    """(ref (n, n, n) uint16, U (n+1, n+1, n+1, 3) float32)."""
    from scipy.ndimage import gaussian_filter
    eps, nu = GT_KINDS[kind]
    rng = np.random.default_rng(seed)
    t = gaussian_filter(rng.standard_normal((n, n, n)), 1.2)
    t = (t - t.mean()) / t.std()
    ref = np.clip(np.round(32112.0 + 6270.0 * t), 15192, 58729).astype(np.uint16)
    g = np.arange(n + 1, dtype=np.float64)
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    U = np.empty((n + 1, n + 1, n + 1, 3))
    x0 = 0.15 * n
    U[..., 0] = -nu * eps * (X - x0)
    U[..., 1] = -nu * eps * (Y - x0)
    U[..., 2] = eps * Z
    amp = 2.0 * abs(eps)   # smooth bumps of amplitude 2 |eps| vx, width n/5
    for _ in range(4):
        c = rng.random(3) * n
        a = rng.standard_normal(3) * amp
        w = np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * (n / 5.0) ** 2))
        U += w[..., None] * a
    return ref, U.astype(np.float32)
