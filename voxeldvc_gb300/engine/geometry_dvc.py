"""Hex8 tables of the voxel-centre DVC discretisation (host, float64).

Same API as the reference module engine/geometry_dvc.py.  The element
operators are the exact unit-cube integrals, built here from 1-D factors:
with N_a(x,y,z) = phi_ax(x) phi_ay(y) phi_az(z) on [0,1]^3 and phi_0 = 1-t,
phi_1 = t, every integral of a product of two shape-function derivatives
factorises over the axes into the 1-D matrices

    M[a,b] = int phi_a phi_b      = [[1/3, 1/6], [1/6, 1/3]]
    S[a,b] = int phi_a' phi_b'    = [[1, -1], [-1, 1]]
    G[a,b] = int phi_a' phi_b     = [[-1/2, -1/2], [1/2, 1/2]]

The reference integrates the same polynomials with 2x2x2 Gauss points
(geometry_dvc.py:58-110), which is exact for them, so both agree to
rounding.  Local corner order: 0=(000) 1=(100) 2=(110) 3=(010) 4=(001)
5=(101) 6=(111) 7=(011) (geometry_dvc.py:14-17).
"""
from __future__ import annotations

import numpy as np

# corner a -> (dx, dy, dz)
CORNERS = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                    (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)], dtype=np.int64)

_M1 = np.array([[1.0 / 3.0, 1.0 / 6.0], [1.0 / 6.0, 1.0 / 3.0]])
_S1 = np.array([[1.0, -1.0], [-1.0, 1.0]])
_G1 = np.array([[-0.5, -0.5], [0.5, 0.5]])


def _axis_factor(i, j, d):
    """1-D factor along axis d of int d_i N_a d_j N_b."""
    if d == i and d == j:
        return _S1
    if d == i:
        return _G1
    if d == j:
        return _G1.T
    return _M1


def _grad_gram():
    """I[i, j, a, b] = int_{[0,1]^3} dN_a/dx_i dN_b/dx_j."""
    I = np.zeros((3, 3, 8, 8))
    for i in range(3):
        for j in range(3):
            F = [_axis_factor(i, j, d) for d in range(3)]
            for a in range(8):
                for b in range(8):
                    v = 1.0
                    for d in range(3):
                        v *= F[d][CORNERS[a, d], CORNERS[b, d]]
                    I[i, j, a, b] = v
    return I


def VoxelCenterStencil(h):
    """Voxel-centre quadrature of one element of edge h voxels: points at
    xi = 2k/h - 1, k = 0..h per axis (meshgrid 'ij' order, last axis
    fastest), trapezoid weights 1/2 on the end planes of each axis
    (geometry_dvc.py:26-51)."""
    k = np.arange(h + 1)
    xi = 2 * k / h - 1
    w = np.ones(h + 1)
    w[[0, -1]] = 0.5
    n = h + 1
    xg = np.repeat(xi, n * n)
    yg = np.tile(np.repeat(xi, n), n)
    zg = np.tile(xi, n * n)
    wg = (w[:, None, None] * w[None, :, None] * w[None, None, :]).reshape(-1)
    return xg, yg, zg, wg


def build_K_ref_laplacian() -> np.ndarray:
    """24x24 vector Laplacian of the unit cube: component-diagonal blocks
    K[3a+c, 3b+c] = int grad N_a . grad N_b (geometry_dvc.py:88-110)."""
    I = _grad_gram()
    L8 = I[0, 0] + I[1, 1] + I[2, 2]
    K = np.zeros((24, 24))
    for c in range(3):
        K[c::3, c::3] = L8
    return K


# Voigt strain rows (xx, yy, zz, xy, yz, xz): entries (component p, derivative i)
_STRAIN_TERMS = [((0, 0),), ((1, 1),), ((2, 2),), ((0, 1), (1, 0)), ((1, 2), (2, 1)), ((0, 2), (2, 0))]


def build_K_ref(nu: float) -> np.ndarray:
    """24x24 isotropic elastic stiffness of the unit cube, E = 1, node-major
    dof order (geometry_dvc.py:58-85): K = int B^T D B with engineering shear
    strains and D the isotropic elasticity matrix."""
    c1 = (1.0 - nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))
    c2 = nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    c3 = 1.0 / (2.0 * (1.0 + nu))
    D = np.diag([c1, c1, c1, c3, c3, c3])
    D[0, 1] = D[0, 2] = D[1, 0] = D[1, 2] = D[2, 0] = D[2, 1] = c2
    # selector C[k, p, i]: strain k picks d u_p / d x_i
    C = np.zeros((6, 3, 3))
    for kk, terms in enumerate(_STRAIN_TERMS):
        for p, i in terms:
            C[kk, p, i] = 1.0
    I = _grad_gram()
    # K[a,p,b,q] = sum_{k,l,i,j} D[k,l] C[k,p,i] C[l,q,j] I[i,j,a,b]
    K4 = np.einsum('kl,kpi,lqj,ijab->apbq', D, C, C, I)
    return K4.reshape(24, 24)


def _hex8_N(x, y, z):
    """Hex8 shape functions at natural coordinates in [-1,1]^3, (npts, 8)."""
    hx = np.stack([(1 - x) / 2, (1 + x) / 2])
    hy = np.stack([(1 - y) / 2, (1 + y) / 2])
    hz = np.stack([(1 - z) / 2, (1 + z) / 2])
    cols = [hx[dx] * hy[dy] * hz[dz] for dx, dy, dz in CORNERS]
    return np.stack(cols, axis=-1)


def build_N_stencil(h: int):
    """(N_stencil ((h+1)^3, 8), w_stencil ((h+1)^3,)) at the voxel-centre
    points of VoxelCenterStencil (geometry_dvc.py:171-184)."""
    xg, yg, zg, wg = VoxelCenterStencil(h)
    return _hex8_N(xg, yg, zg), wg


def build_node_index(Nx: int, Ny: int, Nz: int) -> np.ndarray:
    """(Nx+1, Ny+1, Nz+1) array of node ids i + j(Nx+1) + k(Nx+1)(Ny+1).
    Reference: engine/geometry_dvc.py:191-198."""
    i = np.arange(Nx + 1)[:, None, None]
    j = np.arange(Ny + 1)[None, :, None]
    k = np.arange(Nz + 1)[None, None, :]
    return i + j * (Nx + 1) + k * (Nx + 1) * (Ny + 1)


def build_interior_dof_mask(Nx: int, Ny: int, Nz: int) -> np.ndarray:
    """(Ndof,) bool: dofs of nodes off the outer surface of the mesh.
    Reference: engine/geometry_dvc.py:201-217."""
    i = np.arange(Nx + 1)[:, None, None]
    j = np.arange(Ny + 1)[None, :, None]
    k = np.arange(Nz + 1)[None, None, :]
    inner = (i > 0) & (i < Nx) & (j > 0) & (j < Ny) & (k > 0) & (k < Nz)
    node_inner = np.transpose(inner, (2, 1, 0)).reshape(-1)  # node order, x fastest
    return np.repeat(node_inner, 3)


def element_node_ids(node_idx: np.ndarray, Nx: int, Ny: int, Nz: int) -> np.ndarray:
    """(Nx*Ny*Nz, 8) node ids per element, element order x fastest, corner
    order as documented above.
    Reference: engine/geometry_dvc.py:220-239."""
    out = np.empty((Nz, Ny, Nx, 8), dtype=node_idx.dtype)
    for a, (dx, dy, dz) in enumerate(CORNERS):
        out[..., a] = np.transpose(node_idx[dx:dx + Nx, dy:dy + Ny, dz:dz + Nz], (2, 1, 0))
    return out.reshape(-1, 8)


def _shape_grads(xi: float, eta: float, zeta: float) -> np.ndarray:
    """(3, 8) physical gradients of the shape functions at (xi,eta,zeta) in
    [0,1]^3 of the unit cube."""
    p = np.array([xi, eta, zeta], dtype=float)
    val = np.stack([1.0 - p, p])          # val[d_corner, axis]
    der = np.array([[-1.0] * 3, [1.0] * 3])
    g = np.empty((3, 8))
    for a, c in enumerate(CORNERS):
        for ax in range(3):
            f = 1.0
            for d in range(3):
                f *= der[c[d], d] if d == ax else val[c[d], d]
            g[ax, a] = f
    return g


def _B_matrix(xi: float, eta: float, zeta: float):
    """(6, 24) strain-displacement matrix and detJ = 1/8 at Gauss coordinates
    in [-1,1]^3 of the unit cube."""
    dN = _shape_grads(0.5 * (xi + 1.0), 0.5 * (eta + 1.0), 0.5 * (zeta + 1.0))
    B = np.zeros((6, 24))
    for kk, terms in enumerate(_STRAIN_TERMS):
        for p, i in terms:
            B[kk, p::3] = dN[i]
    return B, 0.125
