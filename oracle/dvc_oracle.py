"""CPU oracle of the voxelDVC global Gauss-Newton path -- TEST INFRASTRUCTURE.

A NumPy/SciPy restatement of the reference algorithm (project voxelDVC,
src/voxeldvc/engine/{geometry_dvc,kernels_dvc,correlate_gpu}.py), written
for checking the CUDA implementation: only tests, the smoke check and the
benchmark's CPU-baseline leg may import it.  It is never the product path.

Parity pinning: every function here is checked against golden vectors
produced by running the reference's own NumPy code
(tests/golden/make_golden.py -> tests/golden/*.npz, see
tests/test_oracle_golden.py).

Third-party arithmetic the reference relies on and this oracle also uses
(same published algorithms): scipy.ndimage.map_coordinates (order 1,
mode 'nearest'), scipy.ndimage.minimum_filter, numpy.gradient, numpy.fft.

Conventions (kernels_dvc.py:9-21): node i + j(Nx+1) + k(Nx+1)(Ny+1),
dof 3*node + c, element i + j Nx + k Nx Ny, voxel vx + vy Nvx + vz Nvx Nvy.
"""
from __future__ import annotations

import numpy as np

# ----------------------------------------------------------------------------
# geometry (geometry_dvc.py)
# ----------------------------------------------------------------------------

# local corner order 000,100,110,010,001,101,111,011 (geometry_dvc.py:14-17)
CORNER = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


def voxel_center_stencil(h):
    """geometry_dvc.py:26-51: xi = 2k/h - 1 on a (h+1)^3 'ij' grid, trapezoid
    weights (1/2 on the two end planes per axis)."""
    xi = 2 * np.arange(h + 1) / h - 1
    w1 = np.where((np.arange(h + 1) == 0) | (np.arange(h + 1) == h), 0.5, 1.0)
    g = np.meshgrid(xi, xi, xi, indexing='ij')
    wg = np.meshgrid(w1, w1, w1, indexing='ij')
    return g[0].ravel(), g[1].ravel(), g[2].ravel(), (wg[0] * wg[1] * wg[2]).ravel()


def hex8_shape(x, y, z):
    """geometry_dvc.py:155-168: N_a = 1/8 (1 +- x)(1 +- y)(1 +- z)."""
    sx = 2 * CORNER[:, 0] - 1
    sy = 2 * CORNER[:, 1] - 1
    sz = 2 * CORNER[:, 2] - 1
    return 0.125 * (1 + x[:, None] * sx) * (1 + y[:, None] * sy) * (1 + z[:, None] * sz)


def n_stencil(h):
    """geometry_dvc.py:171-184."""
    x, y, z, w = voxel_center_stencil(h)
    return hex8_shape(x, y, z), w


def _dN_unit(p):
    """geometry_dvc.py:113-125: (3, 8) physical gradients on [0,1]^3."""
    out = np.empty((3, 8))
    for a in range(8):
        f = [p[d] if CORNER[a, d] else 1 - p[d] for d in range(3)]
        s = [1.0 if CORNER[a, d] else -1.0 for d in range(3)]
        out[0, a] = s[0] * f[1] * f[2]
        out[1, a] = f[0] * s[1] * f[2]
        out[2, a] = f[0] * f[1] * s[2]
    return out


_GAUSS = (-1 / np.sqrt(3), 1 / np.sqrt(3))


def k_ref_laplacian():
    """geometry_dvc.py:88-110: 2x2x2 Gauss, detJ = 1/8, per-component blocks."""
    L8 = np.zeros((8, 8))
    for a in _GAUSS:
        for b in _GAUSS:
            for c in _GAUSS:
                dN = _dN_unit(0.5 * (np.array([a, b, c]) + 1))
                L8 += 0.125 * dN.T @ dN
    K = np.zeros((24, 24))
    for c in range(3):
        K[c::3, c::3] = L8
    return K


def k_ref_elastic(nu):
    """geometry_dvc.py:58-85, 128-148: int B^T D B, E = 1, engineering shear."""
    c1 = (1 - nu) / ((1 + nu) * (1 - 2 * nu))
    c2 = nu / ((1 + nu) * (1 - 2 * nu))
    c3 = 1 / (2 * (1 + nu))
    Dm = np.array([[c1, c2, c2, 0, 0, 0], [c2, c1, c2, 0, 0, 0], [c2, c2, c1, 0, 0, 0],
                   [0, 0, 0, c3, 0, 0], [0, 0, 0, 0, c3, 0], [0, 0, 0, 0, 0, c3]])
    K = np.zeros((24, 24))
    for a in _GAUSS:
        for b in _GAUSS:
            for c in _GAUSS:
                dN = _dN_unit(0.5 * (np.array([a, b, c]) + 1))
                B = np.zeros((6, 24))
                B[0, 0::3] = dN[0]
                B[1, 1::3] = dN[1]
                B[2, 2::3] = dN[2]
                B[3, 0::3], B[3, 1::3] = dN[1], dN[0]
                B[4, 1::3], B[4, 2::3] = dN[2], dN[1]
                B[5, 0::3], B[5, 2::3] = dN[2], dN[0]
                K += 0.125 * B.T @ Dm @ B
    return K


def node_index(Nx, Ny, Nz):
    """geometry_dvc.py:191-198: (Nx+1, Ny+1, Nz+1) ids, x fastest."""
    return np.arange((Nx + 1) * (Ny + 1) * (Nz + 1)).reshape(Nz + 1, Ny + 1, Nx + 1).transpose(2, 1, 0)


def interior_dof_mask(Nx, Ny, Nz):
    """geometry_dvc.py:201-217."""
    ni = node_index(Nx, Ny, Nz)
    inner = np.zeros(ni.shape, dtype=bool)
    inner[1:Nx, 1:Ny, 1:Nz] = True
    m = np.zeros(3 * ni.size, dtype=bool)
    for c in range(3):
        m[3 * ni.ravel() + c] = inner.ravel()
    return m


def element_nodes(Nx, Ny, Nz):
    """geometry_dvc.py:220-239: (Ne, 8) node ids."""
    ni = node_index(Nx, Ny, Nz)
    cols = [ni[dx:dx + Nx, dy:dy + Ny, dz:dz + Nz] for dx, dy, dz in CORNER]
    return np.stack(cols, axis=-1).transpose(2, 1, 0, 3).reshape(-1, 8)


# ----------------------------------------------------------------------------
# implicit connectivity (kernels_dvc.py:32-89)
# ----------------------------------------------------------------------------

def elem_dofs(e, Nx, Ny):
    """kernels_dvc.py:32-61."""
    e = np.asarray(e)
    i, j, k = e % Nx, (e // Nx) % Ny, e // (Nx * Ny)
    n0 = i + j * (Nx + 1) + k * (Nx + 1) * (Ny + 1)
    off = CORNER[:, 0] + CORNER[:, 1] * (Nx + 1) + CORNER[:, 2] * (Nx + 1) * (Ny + 1)
    nodes = n0[:, None] + off.astype(e.dtype)[None, :]
    return (3 * nodes[:, :, None] + np.arange(3, dtype=e.dtype)).reshape(-1, 24)


def voxel_offsets(h, Nx, Ny):
    """kernels_dvc.py:64-78."""
    Nvx, Nvy = Nx * h + 1, Ny * h + 1
    q = np.arange(h + 1, dtype=np.int32)
    qx, qy, qz = np.meshgrid(q, q, q, indexing='ij')
    return (qx + qy * Nvx + qz * Nvx * Nvy).ravel()


def elem_voxel_origins(e, h, Nx, Ny):
    """kernels_dvc.py:81-89."""
    e = np.asarray(e)
    Nvx, Nvy = Nx * h + 1, Ny * h + 1
    return h * (e % Nx + ((e // Nx) % Ny) * Nvx + (e // (Nx * Ny)) * Nvx * Nvy)


def _chunks(Ne, size):
    for s in range(0, Ne, size):
        yield np.arange(s, min(s + size, Ne), dtype=np.int32)


def _scatter(f, idx, vals):
    # np.add.at semantics, via bincount (same sums, CPU friendly)
    f += np.bincount(idx.ravel(), weights=vals.ravel(), minlength=f.shape[0]).astype(f.dtype)


# ----------------------------------------------------------------------------
# regularizers (kernels_dvc.py:349-437)
# ----------------------------------------------------------------------------

def matvec_k_ref(v, K, E, Nx, Ny, Nz, chunk=500_000):
    """kernels_dvc.py:349-374: f = sum_e E_e P_e^T K P_e v."""
    Ne = Nx * Ny * Nz
    f = np.zeros(v.shape[0], dtype=v.dtype)
    Kx = np.asarray(K, dtype=v.dtype)
    Ee = np.broadcast_to(np.asarray(E, dtype=v.dtype), (Ne,))
    for e in _chunks(Ne, chunk):
        d = elem_dofs(e, Nx, Ny)
        loc = v[d] @ Kx.T
        loc *= Ee[e][:, None]
        _scatter(f, d, loc)
    return f


def diag_k_ref(K, E, Nx, Ny, Nz, Ndof):
    """kernels_dvc.py:377-392 (float64, from K's diagonal)."""
    dk = np.diag(np.asarray(K))
    Ne = Nx * Ny * Nz
    Ee = np.broadcast_to(np.asarray(E), (Ne,))
    out = np.zeros(Ndof, dtype=dk.dtype)
    e = np.arange(Ne, dtype=np.int32)
    _scatter(out, elem_dofs(e, Nx, Ny), Ee[:, None] * dk[None, :])
    return out


def matvec_eqgap(v, K_el, interior, E, Nx, Ny, Nz):
    """kernels_dvc.py:402-417: K (P_i (K v))."""
    w = interior * matvec_k_ref(v, K_el, E, Nx, Ny, Nz)
    return matvec_k_ref(w, K_el, E, Nx, Ny, Nz)


def diag_eqgap(K_el, interior, E, Nx, Ny, Nz, Ndof, n_probes=32, seed=0):
    """kernels_dvc.py:420-437: Hutchinson with default_rng(seed) Rademacher
    probes, then clip at 1e-12 max|diag|."""
    rng = np.random.default_rng(seed)
    acc = np.zeros(Ndof)
    for _ in range(n_probes):
        z = rng.choice([-1.0, 1.0], size=Ndof)
        acc = acc + z * matvec_eqgap(z, K_el, interior, E, Nx, Ny, Nz)
    d = acc / n_probes
    return np.clip(d, 1e-12 * float(np.abs(d).max()), None)


# ----------------------------------------------------------------------------
# correlation Hessian (kernels_dvc.py:444-543)
# ----------------------------------------------------------------------------

def _hchunk(nq):
    return max(1, 20_000_000 // (nq * 24))  # kernels_dvc.py:444-449


def matvec_h(v, grad, mask, h, Nx, Ny, Nz, chunk=None):
    """kernels_dvc.py:452-506: H v, separable einsum form."""
    N, w = n_stencil(h)
    N = N.astype(v.dtype)
    w = w.astype(v.dtype)
    offs = voxel_offsets(h, Nx, Ny)
    Ne = Nx * Ny * Nz
    f = np.zeros(v.shape[0], dtype=v.dtype)
    for e in _chunks(Ne, chunk or _hchunk(offs.size)):
        d = elem_dofs(e, Nx, Ny)
        vl = v[d].reshape(-1, 8, 3)
        vid = elem_voxel_origins(e, h, Nx, Ny)[:, None] + offs[None, :]
        gq = grad[vid]
        mq = mask[vid]
        u = np.einsum('qa,cak->cqk', N, vl)
        coef = w[None, :] * mq * np.einsum('cqk,cqk->cq', gq, u)
        loc = np.einsum('qa,cqk->cak', N, coef[:, :, None] * gq).reshape(-1, 24)
        _scatter(f, d, loc)
    return f


def _kl(k, l):
    k, l = min(k, l), max(k, l)
    return (0, 1, 2, 3, 4, 5)[[(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)].index((k, l))]


def eh_f16_elements(grad_bf16, mask, h, Nx, Ny, Nz):
    """Element Hessians of the precision form as the tensor-core formation
    computes them: owner-computes point sets (a shared face belongs to the
    element beyond it), trapezoid halves on the domain faces only, operands
    A = w m g_k g_l x 2^(13 - floor(log2 max g^2)) and P = 256 psi psi psi
    rounded to FP16 from their FP32 values, products summed exactly (float64)
    and unscaled.  Returns T (Ne, 27, 6): T[e, 9 sx + 3 sy + sz, kl].  The
    precision form has no counterpart in the reference; T restates the
    Hessian of kernels_dvc.py:452-506 element by element."""
    H = h
    g = np.asarray(grad_bf16, np.float32).reshape(-1, 3)
    gm = np.float32(np.abs(g).max()) if g.size else np.float32(0)
    g2 = np.float32(gm * gm)
    e2 = int(np.floor(np.log2(g2))) if 0 < g2 < 3.0e38 else 0
    e2 = max(-100, min(100, e2))
    scaleA = np.float32(2.0 ** (13 - e2))
    inv_h = np.float32(1) / np.float32(H)
    q1 = np.arange(H + 1)
    f1 = q1.astype(np.float32) * inv_h
    f0 = np.float32(1) - f1
    psi = np.stack([f0 * f0, f0 * f1, f1 * f1])                     # (3, H+1) float32
    P = np.zeros((27, H + 1, H + 1, H + 1), np.float32)
    for sx in range(3):
        for sy in range(3):
            for sz in range(3):
                P[9 * sx + 3 * sy + sz] = ((np.float32(256) * psi[sx][:, None, None]) * psi[sy][None, :, None]) \
                    * psi[sz][None, None, :]
    P16 = P.astype(np.float16).astype(np.float64).reshape(27, -1)     # index (qx, qy, qz), qz fastest
    Nvx, Nvy = Nx * H + 1, Ny * H + 1
    QX, QY, QZ = (a.ravel() for a in np.meshgrid(q1, q1, q1, indexing='ij'))
    Ne = Nx * Ny * Nz
    T = np.zeros((Ne, 27, 6))
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for e in range(Ne):
        i, j, k = e % Nx, (e // Nx) % Ny, e // (Nx * Ny)
        own = ((QX < H) | (i == Nx - 1)) & ((QY < H) | (j == Ny - 1)) & ((QZ < H) | (k == Nz - 1))
        v = i * H + QX + (j * H + QY) * Nvx + (k * H + QZ) * Nvx * Nvy
        w = np.full(QX.shape, scaleA, np.float32)
        w = np.where(((QX == 0) & (i == 0)) | ((QX == H) & (i == Nx - 1)), w * np.float32(0.5), w)
        w = np.where(((QY == 0) & (j == 0)) | ((QY == H) & (j == Ny - 1)), w * np.float32(0.5), w)
        w = np.where(((QZ == 0) & (k == 0)) | ((QZ == H) & (k == Nz - 1)), w * np.float32(0.5), w)
        w = np.where(own & np.asarray(mask, bool)[np.where(own, v, 0)], w, np.float32(0))
        gv = g[np.where(own, v, 0)]
        for c, (kk, ll) in enumerate(pairs):
            A16 = (w * (gv[:, kk] * gv[:, ll])).astype(np.float16).astype(np.float64)
            T[e, :, c] = P16 @ A16
    return T / (256.0 * float(scaleA))


def eh_matvec(T, v, Nx, Ny, Nz):
    """H v from element Hessians T (Ne, 27, 6):
    K_e[(a,k),(b,l)] = T[e, 9 (ax+bx) + 3 (ay+by) + (az+bz), kl(k,l)]; the
    assembly of kernels_dvc.py:452-506 with stored element matrices."""
    out = np.zeros(v.shape[0])
    for e in range(Nx * Ny * Nz):
        d = elem_dofs(np.array([e]), Nx, Ny)[0]
        K = np.empty((24, 24))
        for a in range(8):
            for b in range(8):
                s = 9 * (CORNER[a, 0] + CORNER[b, 0]) + 3 * (CORNER[a, 1] + CORNER[b, 1]) + CORNER[a, 2] + CORNER[b, 2]
                for k in range(3):
                    for l in range(3):
                        K[3 * a + k, 3 * b + l] = T[e, s, _kl(k, l)]
        np.add.at(out, d, K @ v[d])
    return out


def diag_h(grad, mask, h, Nx, Ny, Nz, Ndof, chunk=None):
    """kernels_dvc.py:509-543."""
    N, w = n_stencil(h)
    N2 = N.astype(grad.dtype) ** 2
    w = w.astype(grad.dtype)
    offs = voxel_offsets(h, Nx, Ny)
    Ne = Nx * Ny * Nz
    out = np.zeros(Ndof, dtype=grad.dtype)
    for e in _chunks(Ne, chunk or _hchunk(offs.size)):
        d = elem_dofs(e, Nx, Ny)
        vid = elem_voxel_origins(e, h, Nx, Ny)[:, None] + offs[None, :]
        gq = grad[vid]
        t = (w[None, :] * mask[vid])[:, :, None] * gq ** 2
        _scatter(out, d, np.einsum('qa,cqk->cak', N2, t).reshape(-1, 24))
    return out


def compute_b(res, mask, grad, h, Nx, Ny, Nz, Ndof, chunk=None):
    """correlate_gpu.py:341-378."""
    N, w = n_stencil(h)
    N = N.astype(grad.dtype)
    w = w.astype(grad.dtype)
    offs = voxel_offsets(h, Nx, Ny)
    Ne = Nx * Ny * Nz
    out = np.zeros(Ndof, dtype=grad.dtype)
    for e in _chunks(Ne, chunk or _hchunk(offs.size)):
        d = elem_dofs(e, Nx, Ny)
        vid = elem_voxel_origins(e, h, Nx, Ny)[:, None] + offs[None, :]
        gq = grad[vid]
        coef = w[None, :] * mask[vid] * res[vid]
        _scatter(out, d, np.einsum('qa,cqk->cak', N, coef[:, :, None] * gq).reshape(-1, 24))
    return out


def pcg(matvec, b, M_inv, x0=None, max_iter=1000, tol=1e-8):
    """kernels_dvc.py:550-583 (numpy promotion rules as in the reference)."""
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - matvec(x)
    z = M_inv * r
    p = z.copy()
    rz = np.dot(r, z)
    r0 = np.dot(b, b) + 1e-30
    for _ in range(max_iter):
        Ap = matvec(p)
        alpha = rz / (np.dot(p, Ap) + 1e-30)
        x = x + alpha * p
        r = r - alpha * Ap
        if float(np.sqrt(np.dot(r, r) / r0)) < tol:
            break
        z = M_inv * r
        rz_new = np.dot(r, z)
        p = z + rz_new / (rz + 1e-30) * p
        rz = rz_new
    return x


# ----------------------------------------------------------------------------
# voxel fields (correlate_gpu.py:49-338)
# ----------------------------------------------------------------------------

def image_grad_and_values(pix, dtype=np.float32):
    """correlate_gpu.py:49-72: F-order values and per-axis np.gradient."""
    p = np.asarray(pix, dtype=dtype)
    g = np.empty((p.size, 3), dtype=dtype)
    for c in range(3):
        g[:, c] = np.gradient(p, axis=c).ravel(order='F')
    return p.ravel(order='F'), g


def erode(mask, Nvx, Nvy, Nvz):
    """correlate_gpu.py:75-94: 6-neighbour minimum filter, mode 'nearest'."""
    from scipy.ndimage import minimum_filter
    fp = np.zeros((3, 3, 3), dtype=bool)
    fp[1, 1, :] = fp[1, :, 1] = fp[:, 1, 1] = True
    out = minimum_filter(mask.reshape(Nvx, Nvy, Nvz, order='F'), footprint=fp, mode='nearest')
    return out.ravel(order='F')


def masked_mean_std(field, mask, h, Nx, Ny, Nz):
    """correlate_gpu.py:113-157: multiplicity-weighted masked mean / std
    with float64 sums."""
    offs = voxel_offsets(h, Nx, Ny)
    Ne = Nx * Ny * Nz
    cnt = s1 = s2 = 0.0
    for e in _chunks(Ne, _hchunk(offs.size)):
        vid = elem_voxel_origins(e, h, Nx, Ny)[:, None] + offs[None, :]
        m = mask[vid].astype(np.float64)
        v = field[vid].astype(np.float64) * m
        cnt += m.sum()
        s1 += v.sum()
        s2 += (v * v).sum()
    if cnt < 1:
        return 0.0, 0.0
    mean = s1 / cnt
    var = s2 / cnt - mean * mean
    return mean, (var if var > 0.0 else 0.0) ** 0.5


def interp_field(U, h, Nx, Ny, Nz):
    """correlate_gpu.py:160-198: u at every voxel, later elements win."""
    N, _ = n_stencil(h)
    N = N.astype(U.dtype)
    offs = voxel_offsets(h, Nx, Ny)
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    out = np.zeros((Nvox, 3), dtype=U.dtype)
    e = np.arange(Nx * Ny * Nz, dtype=np.int32)
    ul = U[elem_dofs(e, Nx, Ny)].reshape(-1, 8, 3)
    vid = elem_voxel_origins(e, h, Nx, Ny)[:, None] + offs[None, :]
    out[vid.reshape(-1)] = np.einsum('qa,kac->kqc', N, ul).reshape(-1, 3)
    return out


def push_field_forward(field, U, Nx, Ny, Nz, h, order=1, mode='nearest', cval=0.0):
    """write_output.py:571-608: field(x - u(x)) on the voxel grid, u the
    FE-interpolated displacement, scipy map_coordinates(order, mode, cval)."""
    from scipy.ndimage import map_coordinates
    Nvx, Nvy, Nvz = field.shape
    u = interp_field(np.asarray(U), h, Nx, Ny, Nz)
    vx, vy, vz = (np.ravel(a, order='F').astype(u.dtype) for a in
                  np.meshgrid(np.arange(Nvx), np.arange(Nvy), np.arange(Nvz), indexing='ij'))
    coords = np.stack([vx - u[:, 0], vy - u[:, 1], vz - u[:, 2]])
    return map_coordinates(field, coords, order=order, mode=mode, cval=cval).reshape(Nvx, Nvy, Nvz, order='F')


def zncc(f_flat, g_flat, mask):
    """write_output.py:658-690: zero-normalised cross-correlation over mask."""
    f = np.asarray(f_flat, dtype=np.float64)[mask]
    g = np.asarray(g_flat, dtype=np.float64)[mask]
    if f.size == 0:
        return float('nan')
    f = f - f.mean()
    g = g - g.mean()
    den = np.sqrt(np.sum(f * f) * np.sum(g * g))
    return float(np.sum(f * g) / den) if den > 0 else float('nan')


def warp_onto_ref_grid(A, t, c, Nf, g):
    """preprocess.py:233-285: g at A (x - c) + c + t on f's grid, coordinates
    in float32 as the reference forms them, order-1, 0 outside (the
    reference samples with cupyx's map_coordinates, scipy's semantics)."""
    from scipy.ndimage import map_coordinates
    A32, t32, c32 = (np.asarray(v, np.float32) for v in (A, t, c))
    I, J, K = np.meshgrid(*[np.arange(n, dtype=np.float32) for n in Nf], indexing='ij')
    pts = np.stack([I.ravel(), J.ravel(), K.ravel()])
    pts_g = A32 @ (pts - c32.reshape(3, 1)) + c32.reshape(3, 1) + t32.reshape(3, 1)
    return map_coordinates(np.asarray(g, np.float32), pts_g, order=1, mode='constant',
                           cval=0.0).reshape(Nf).astype(np.float32)


def bin_volume(vol, B):
    """preprocess.py:288-312: float32 sums over the B^3 strided sub-volumes."""
    S0, S1, S2 = vol.shape
    out = np.zeros((S0 // B, S1 // B, S2 // B), dtype=np.float32)
    for i in range(B):
        for j in range(B):
            for k in range(B):
                out += vol[i::B, j::B, k::B]
    out /= B ** 3
    return out


def compute_crop(f, g, h, glt=0.0):
    """preprocess.py:315-367: n h + 1 crop of the valid overlap."""
    valid = (f > glt) & (g > glt)
    idx = [np.where(valid.any(axis=tuple(b for b in range(3) if b != a)))[0] for a in range(3)]
    lo = np.array([i[0] for i in idx])
    hi = np.array([i[-1] for i in idx])
    snapped = ((hi - lo) // h) * h + 1
    lo_out = (lo + hi) // 2 - snapped // 2
    hi_out = lo_out + snapped
    for a in range(3):
        if lo_out[a] < 0:
            hi_out[a] -= lo_out[a]
            lo_out[a] = 0
        if hi_out[a] > f.shape[a]:
            lo_out[a] -= hi_out[a] - f.shape[a]
            hi_out[a] = f.shape[a]
    return lo_out, hi_out


# ----------------------------------------------------------------------------
# per-element output fields (write_output.py:256-491) and diagnostic masks
# (kernels_dvc.py:92-341); element arrays x-fastest unless stated
# ----------------------------------------------------------------------------

def _elem_blocks(h, Nx, Ny, Nz):
    """(Ne, (h+1)^3) flat voxel indices of every element's block."""
    return elem_voxel_origins(np.arange(Nx * Ny * Nz), h, Nx, Ny)[:, None] + voxel_offsets(h, Nx, Ny)[None, :]


def _x_flat(a):
    a = np.asarray(a)
    return a.reshape(-1, order='F') if a.ndim == 3 else a.reshape(-1)


def _to_cells(a, Nx, Ny, Nz):
    return np.asarray(a).reshape(Nx, Ny, Nz, order='F')


def _corner_nodes(Nx, Ny, Nz):
    e = np.arange(Nx * Ny * Nz)
    n0 = e % Nx + ((e // Nx) % Ny) * (Nx + 1) + (e // (Nx * Ny)) * (Nx + 1) * (Ny + 1)
    off = CORNER[:, 0] + CORNER[:, 1] * (Nx + 1) + CORNER[:, 2] * (Nx + 1) * (Ny + 1)
    return n0[:, None] + off[None, :]


def principal_strains_cell(U_grid, h):
    """write_output.py:256-281: eigenvalues (descending) of the symmetric
    displacement gradient at each centroid, corner weights +-1/(4h)."""
    Nx, Ny, Nz = (n - 1 for n in U_grid.shape[:3])
    sgn = 2.0 * CORNER - 1.0                                   # (8, 3)
    g = np.zeros((Nx, Ny, Nz, 3, 3))
    for a, (dx, dy, dz) in enumerate(CORNER):
        ua = U_grid[dx:dx + Nx, dy:dy + Ny, dz:dz + Nz, :]      # (..., 3) component c
        g += ua[..., :, None] * (sgn[a] * 0.25 / h)[None, None, None, None, :]
    eps = 0.5 * (g + np.swapaxes(g, -1, -2))
    return np.linalg.eigvalsh(eps)[..., ::-1]


def equivalent_strain(ps):
    """write_output.py:284-310."""
    e1, e2, e3 = ps[..., 0], ps[..., 1], ps[..., 2]
    return np.sqrt(2.0) / 3.0 * np.sqrt((e1 - e2) ** 2 + (e2 - e3) ** 2 + (e3 - e1) ** 2)


def material_cell_mask(ref, h, Nx, Ny, Nz, glt=0.0):
    """write_output.py:313-338: block mean of ref > glt (float64 mean)."""
    r = _x_flat(ref).astype(np.float64)
    return _to_cells(r[_elem_blocks(h, Nx, Ny, Nz)].mean(axis=1) > glt, Nx, Ny, Nz)


def material_cell_mask_eroded(m):
    """write_output.py:341-355: 26-neighbour erosion, border counts as set."""
    p = np.pad(np.asarray(m, bool), 1, constant_values=True)
    out = np.ones(m.shape, bool)
    for di in range(3):
        for dj in range(3):
            for dk in range(3):
                out &= p[di:di + m.shape[0], dj:dj + m.shape[1], dk:dk + m.shape[2]]
    return out


def safe_cell_mask(unsafe_vox, h, Nx, Ny, Nz):
    """write_output.py:358-381: no unsafe voxel in the block."""
    u = _x_flat(unsafe_vox).astype(bool)
    return _to_cells(~u[_elem_blocks(h, Nx, Ny, Nz)].any(axis=1), Nx, Ny, Nz)


def correlation_quality_cell(res, ref, h, Nx, Ny, Nz, min_active=8):
    """write_output.py:384-452: per-block population std of res and ZNCC of
    ref and ref - res over the active (res != 0) voxels."""
    B = _elem_blocks(h, Nx, Ny, Nz)
    std = np.full(len(B), np.nan)
    zn = np.full(len(B), np.nan)
    r_all = _x_flat(res).astype(np.float64)
    f_all = _x_flat(ref).astype(np.float64)
    for e, vox in enumerate(B):
        r = r_all[vox]
        act = r != 0.0
        n = int(act.sum())
        if n < min_active:
            continue
        r, f = r[act], f_all[vox][act]
        std[e] = np.sqrt(max(np.mean(r * r) - np.mean(r) ** 2, 0.0))
        fc, gc = f - f.mean(), (f - r) - (f - r).mean()
        den = np.sqrt(np.sum(fc * fc) * np.sum(gc * gc))
        if den > 0.0:
            zn[e] = np.sum(fc * gc) / den
    return _to_cells(std, Nx, Ny, Nz), _to_cells(zn, Nx, Ny, Nz)


def gn_convergence_cell(dU, U, Nx, Ny, Nz):
    """write_output.py:455-491: corner-DOF norm ratio, NaN where ||U|| = 0."""
    cn = _corner_nodes(Nx, Ny, Nz)
    d = np.asarray(dU, np.float64).reshape(-1, 3)[cn]
    u = np.asarray(U, np.float64).reshape(-1, 3)[cn]
    num = np.sqrt((d * d).sum(axis=(1, 2)))
    den = np.sqrt((u * u).sum(axis=(1, 2)))
    out = np.full(num.shape, np.nan)
    ok = den > 0.0
    out[ok] = num[ok] / den[ok]
    return _to_cells(out, Nx, Ny, Nz)


def boundary_elements(Nx, Ny, Nz):
    """kernels_dvc.py:92-116: the outer element shell, x-fastest."""
    e = np.arange(Nx * Ny * Nz)
    i, j, k = e % Nx, (e // Nx) % Ny, e // (Nx * Ny)
    return (i == 0) | (j == 0) | (k == 0) | (i == Nx - 1) | (j == Ny - 1) | (k == Nz - 1)


def unsafe_masks(active_vox, h, Nx, Ny, Nz, mask0_vox=None, frac_threshold=0.0, min_material_frac=0.5):
    """kernels_dvc.py:119-341 -> dict of unsafe_vox, unsafe_elem,
    unsafe_node and (with mask0_vox) overlap_lost."""
    act = np.asarray(active_vox, bool)
    B = _elem_blocks(h, Nx, Ny, Nz)
    cn = _corner_nodes(Nx, Ny, Nz)
    Nn = (Nx + 1) * (Ny + 1) * (Nz + 1)
    bnd = boundary_elements(Nx, Ny, Nz)
    node_pre = np.zeros(Nn, bool)
    node_pre[cn[(~act)[B].any(axis=1)].ravel()] = True
    elem = node_pre[cn].any(axis=1) | bnd
    node = node_pre.copy()
    node[cn[bnd].ravel()] = True
    vox = np.zeros(act.shape[0], bool)
    vox[B[elem].ravel()] = True
    out = dict(unsafe_vox=vox, unsafe_elem=elem, unsafe_node=node)
    if mask0_vox is not None:
        m0 = np.asarray(mask0_vox, bool)
        n_mat = m0[B].sum(axis=1)
        n_lost = (m0 & ~act)[B].sum(axis=1)
        lost = np.zeros(len(B), bool)
        has = n_mat > 0
        lost[has] = n_lost[has] / n_mat[has] > frac_threshold
        node_lost = np.zeros(Nn, bool)
        node_lost[cn[lost].ravel()] = True
        out["overlap_lost"] = node_lost[cn].any(axis=1) | (n_mat / B.shape[1] < min_material_frac) | bnd
    return out


# ----------------------------------------------------------------------------
# known-answer harness (ground_truth/prepare_ground_truth.py,
# ground_truth/analyse_ground_truth.py)
# ----------------------------------------------------------------------------

def gt_warp(ref, u):
    """prepare_ground_truth.py:66-89: ref(x - u(x)), trilinear with linear
    extrapolation (RegularGridInterpolator(fill_value=None)): per axis the
    cell i = clip(ceil(p) - 1, 0, n - 2), weights (1 - t, t), t = p - i;
    corner terms summed lo-before-hi with the last axis fastest."""
    ref = np.asarray(ref, np.float64)
    dims = ref.shape
    grids = np.meshgrid(*(np.arange(n, dtype=np.float64) for n in dims), indexing='ij')
    lo, w = [], []
    for a in range(3):
        p = grids[a] - u[..., a]
        i = np.clip(np.ceil(p) - 1.0, 0, dims[a] - 2).astype(np.int64)
        t = p - i
        lo.append(i)
        w.append((1.0 - t, t))
    acc = np.zeros(dims)
    for b0 in (0, 1):
        for b1 in (0, 1):
            for b2 in (0, 1):
                wt = (w[0][b0] * w[1][b1]) * w[2][b2]
                acc = acc + ref[lo[0] + b0, lo[1] + b1, lo[2] + b2] * wt
    return acc


def gt_uniaxial(n, strain):
    """prepare_ground_truth.py:92-107: u_x = strain x on the (n,)*3 grid."""
    u = np.zeros((n, n, n, 3))
    u[..., 0] = strain * np.arange(n, dtype=np.float64)[:, None, None]
    return u


def gt_voxel_in_bounds(u, g_shape):
    """analyse_ground_truth.py:113-136: x + u(x) inside [0, g - 1]."""
    ok = np.ones(u.shape[:3], bool)
    for a in range(3):
        c = np.arange(u.shape[a], dtype=np.float64).reshape([-1 if b == a else 1 for b in range(3)]) + u[..., a]
        ok &= (c >= 0) & (c <= g_shape[a] - 1)
    return ok


def gt_node_oob_fraction(u, h, nb, g_shape, crop_lo):
    """analyse_ground_truth.py:139-174 via a summed-volume table of the
    in-bounds mask: 1 - (in-bounds count / voxel count) over each node's
    clamped support box [v - h, v + h]."""
    inb = gt_voxel_in_bounds(u, g_shape).astype(np.int64)
    S = np.zeros(tuple(n + 1 for n in inb.shape), np.int64)
    S[1:, 1:, 1:] = inb.cumsum(0).cumsum(1).cumsum(2)
    ax = []
    for a in range(3):
        v = crop_lo[a] + np.arange(nb[a]) * h
        ax.append((np.maximum(v - h, 0), np.minimum(v + h, inb.shape[a] - 1) + 1))
    A0, A1, A2 = np.meshgrid(ax[0][0], ax[1][0], ax[2][0], indexing='ij')
    B0, B1, B2 = np.meshgrid(ax[0][1], ax[1][1], ax[2][1], indexing='ij')
    cnt = (S[B0, B1, B2] - S[A0, B1, B2] - S[B0, A1, B2] - S[B0, B1, A2]
           + S[A0, A1, B2] + S[A0, B1, A2] + S[B0, A1, A2] - S[A0, A1, A2])
    tot = (B0 - A0) * (B1 - A1) * (B2 - A2)
    return 1.0 - cnt / tot


def sample_deformed(U, g_pix, h, Nx, Ny, Nz, g_origin=(0, 0, 0), mask0=None, glt=0.0):
    """correlate_gpu.py:201-281: g at (u + x) - g_origin, clipped, order-1
    map_coordinates; mask in_bounds & mask0 & g > glt."""
    from scipy.ndimage import map_coordinates
    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    Nvox = Nvx * Nvy * Nvz
    if mask0 is None:
        mask0 = np.ones(Nvox, dtype=bool)
    dt = U.dtype
    u = interp_field(U, h, Nx, Ny, Nz)
    v = np.arange(Nvox)
    c = [u[:, 0] + (v % Nvx).astype(dt) - g_origin[0],
         u[:, 1] + ((v // Nvx) % Nvy).astype(dt) - g_origin[1],
         u[:, 2] + (v // (Nvx * Nvy)).astype(dt) - g_origin[2]]
    n = g_pix.shape
    inb = np.ones(Nvox, dtype=bool)
    for a in range(3):
        inb &= (c[a] >= 0) & (c[a] <= n[a] - 1)
        c[a] = np.clip(c[a], 0, n[a] - 1)
    gv = map_coordinates(g_pix, np.stack(c), order=1, mode='nearest')  # g_pix dtype
    return gv.astype(dt), inb & mask0 & (gv > glt)


# ----------------------------------------------------------------------------
# FFT pre-alignment (correlate_gpu.py:381-414)
# ----------------------------------------------------------------------------

def fft_rigid_shift(f_pix, g_pix):
    """Integer rigid shift from the phase correlation of the common crop
    (correlate_gpu.py:381-414)."""
    f = np.asarray(f_pix)
    g = np.asarray(g_pix)
    shp = tuple(min(a, b) for a, b in zip(f.shape, g.shape))
    sl = tuple(slice(0, s) for s in shp)
    X = np.fft.fftn(f[sl]) * np.conj(np.fft.fftn(g[sl]))
    r = np.fft.ifftn(X / (np.abs(X) + 1e-12)).real
    peak = np.unravel_index(np.argmax(r), r.shape)
    d = []
    for p, s in zip(peak, shp):
        p = int(p)
        d.append(-float(p - s if p > s // 2 else p))
    return np.array(d)


# ----------------------------------------------------------------------------
# Gauss-Newton driver (correlate_gpu.py:828-1140) and pyramid (:1143-1305)
# ----------------------------------------------------------------------------

def correlate(f_pix, g_pix, Nx, Ny, Nz, h, g_origin=(0, 0, 0), glt=0.0, l0=None, K_lap=None, reg_exponent=2,
              c_reg=1.0, reg_type='laplacian', K_el=None, eps_reg=1e-3, dynamic_mask=False, freeze_mask_after=None,
              U0=None, maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000, dtype=np.float32, log=None):
    """The Gauss-Newton driver of correlate_gpu.py:828-1140 on NumPy.
    Returns (U, res, dU); `log` (a list) receives one dict per GN iteration."""
    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    Nvox = Nvx * Nvy * Nvz
    g_pix = np.asarray(g_pix, dtype=dtype)
    f_vox, grad = image_grad_and_values(f_pix, dtype)
    mask0 = f_vox > glt
    grad[~erode(mask0, Nvx, Nvy, Nvz)] = 0
    mean0, std0 = masked_mean_std(f_vox, mask0, h, Nx, Ny, Nz)
    f_vox -= mean0
    interior = interior_dof_mask(Nx, Ny, Nz).astype(dtype) if reg_type == 'equilibrium_gap' else None

    def reg(v):
        if reg_type == 'laplacian':
            return matvec_k_ref(v, K_lap, h, Nx, Ny, Nz)
        return matvec_eqgap(v, K_el, interior, h, Nx, Ny, Nz) + eps_reg * matvec_k_ref(v, K_lap, h, Nx, Ny, Nz)

    def reg_diag():
        if reg_type == 'laplacian':
            return diag_k_ref(K_lap, h, Nx, Ny, Nz, Ndof)
        return diag_eqgap(K_el, interior, h, Nx, Ny, Nz, Ndof) + eps_reg * diag_k_ref(K_lap, h, Nx, Ny, Nz, Ndof)

    ll = 0.0
    if l0 is not None:
        T = 10 * h
        if reg_type == 'equilibrium_gap':
            H0 = float(diag_h(grad, mask0, h, Nx, Ny, Nz, Ndof).sum())
            L0 = float(reg_diag().sum())
        else:
            jj = (np.arange((Nx + 1) * (Ny + 1) * (Nz + 1)) // (Nx + 1)) % (Ny + 1)
            V = np.zeros(Ndof, dtype=dtype)
            V[0::3] = np.cos(jj.astype(dtype) * h / T * 2 * np.pi)
            H0 = float(np.dot(V, matvec_h(V, grad, mask0, h, Nx, Ny, Nz)))
            L0 = float(np.dot(V, reg(V)))
        ll = c_reg * (l0 / T) ** reg_exponent * H0 / L0

    U = np.zeros(Ndof, dtype=dtype) if U0 is None else np.asarray(U0, dtype=dtype).copy()
    res = np.zeros(Nvox, dtype=dtype)
    dU = np.zeros(Ndof, dtype=dtype)
    if not dynamic_mask:
        dg = diag_h(grad, mask0, h, Nx, Ny, Nz, Ndof)
        if l0 is not None:
            dg = dg + ll * reg_diag()
        M_inv = 1.0 / (dg + 1e-5 * float(dg.min()))
        H_mask = mask0
    frozen = None
    for ik in range(maxiter):
        gv, live = sample_deformed(U, g_pix, h, Nx, Ny, Nz, g_origin, mask0, glt)
        if freeze_mask_after is not None and frozen is None and ik >= freeze_mask_after:
            frozen = live.copy()
        bm = frozen if frozen is not None else live
        gmean, std1 = masked_mean_std(gv, bm, h, Nx, Ny, Nz)
        gv = gv - gmean
        gv = gv * -(std0 / std1)
        res = gv + f_vox
        res[~bm] = 0.0
        b = compute_b(res, bm, grad, h, Nx, Ny, Nz, Ndof)
        if l0 is not None:
            b = b - ll * reg(U)
        if dynamic_mask:
            dg = diag_h(grad, bm, h, Nx, Ny, Nz, Ndof)
            if l0 is not None:
                dg = dg + ll * reg_diag()
            M_inv = 1.0 / (dg + 1e-5 * float(dg.min()))
            H_mask = bm

        def A(v, _m=H_mask):
            out = matvec_h(v, grad, _m, h, Nx, Ny, Nz)
            return out + ll * reg(v) if l0 is not None else out

        dU = pcg(A, b, M_inv, max_iter=pcg_max_iter, tol=pcg_tol)
        U = U + dU
        err = float(np.linalg.norm(dU) / np.linalg.norm(U))
        if log is not None:
            _, stdr = masked_mean_std(res, live, h, Nx, Ny, Nz)
            log.append({"err": err, "stdr": stdr, "n_active": int(live.sum()), "ll": ll})
        if err < eps:
            break
    return U, res, dU


def multiscale(f_pix, g_pix, Nx, Ny, Nz, h, scales=(2, 1, 0), g_origin=(0, 0, 0), l0=None, fft_prealign=True,
               ext_affine=None, **kw):
    """correlate_gpu.py:1143-1305 (without the Powell affine pre-alignment)."""
    dtype = kw.get('dtype', np.float32)
    U = None
    prev = None
    res = dU = None
    for i in sorted(set(scales), reverse=True):
        s = 2 ** i
        if h % s != 0:
            raise ValueError("h=%d not divisible by 2**%d=%d" % (h, i, s))
        if any(o % s for o in g_origin):
            raise ValueError("g_origin=%r not divisible by 2**%d=%d" % (g_origin, i, s))
        hi = h // s
        fi = np.asarray(f_pix)[::s, ::s, ::s]
        gi = np.asarray(g_pix)[::s, ::s, ::s]
        if U is not None:
            U = U * (prev / s)
        elif ext_affine is not None:
            A, t, c = (np.asarray(q, dtype=np.float64) for q in ext_affine)
            nn = np.arange((Nx + 1) * (Ny + 1) * (Nz + 1))
            X = np.stack([nn % (Nx + 1), (nn // (Nx + 1)) % (Ny + 1), nn // ((Nx + 1) * (Ny + 1))], 1) * float(hi)
            u = (X - c / s) @ A.T + c / s + t / s - X
            U = u.reshape(-1).astype(dtype)
        elif fft_prealign:
            d = fft_rigid_shift(fi, gi)
            U = np.tile(d, (Nx + 1) * (Ny + 1) * (Nz + 1)).astype(dtype)
        U, res, dU = correlate(fi, gi, Nx, Ny, Nz, hi, g_origin=tuple(o // s for o in g_origin),
                               l0=None if l0 is None else l0 / s, U0=U, **kw)
        prev = s
    return U, res, dU


# ----------------------------------------------------------------------------
# affine pre-alignment (correlate_gpu.py:417-825)
# ----------------------------------------------------------------------------

def affine_matrix(p):
    """correlate_gpu.py:436-448: R = Rz Ry Rx, A = R diag(s)."""
    rx, ry, rz, sx, sy, sz = p[:6]
    cx, sxr, cy, syr, cz, szr = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sxr], [0, sxr, cx]])
    Ry = np.array([[cy, 0, syr], [0, 1, 0], [-syr, 0, cy]])
    Rz = np.array([[cz, -szr, 0], [szr, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx @ np.diag([sx, sy, sz])


def zncc_cost(f_flat, g_samp, valid):
    """correlate_gpu.py:417-433: 1 - ZNCC over `valid`, 2.0 when degenerate."""
    if int(valid.sum()) < 1000:
        return 2.0
    fv = f_flat[valid] - f_flat[valid].mean()
    gv = g_samp[valid] - g_samp[valid].mean()
    den = np.sqrt((fv * fv).sum() * (gv * gv).sum())
    if float(den) < 1e-8:
        return 2.0
    return 1.0 - float((fv * gv).sum() / den)


def affine_cost(f_d, g_d, p):
    """warp_and_cost of affine_prealign (correlate_gpu.py:523-536)."""
    from scipy.ndimage import map_coordinates
    c = np.array([(n - 1) / 2.0 for n in f_d.shape])
    X = np.stack([a.ravel() for a in np.meshgrid(*[np.arange(n) for n in f_d.shape], indexing='ij')]).astype(float)
    Xp = affine_matrix(p) @ (X - c[:, None]) + c[:, None] + np.asarray(p[6:9])[:, None]
    n = g_d.shape
    inb = np.all([(Xp[a] >= 0) & (Xp[a] <= n[a] - 1) for a in range(3)], axis=0)
    gs = map_coordinates(g_d, Xp, order=1, mode='nearest')
    return zncc_cost(f_d.ravel(), gs, inb)


def affine_normal_equations(f_s, grads, g_s, g, M, tr, c, cval=0.0):
    """The 12x12 float64 system of one affine_refine_gn iteration
    (correlate_gpu.py:757-791), whole volume at once."""
    from scipy.ndimage import map_coordinates
    Mf, trf, cf = M.astype(np.float32), tr.astype(np.float32), np.asarray(c, np.float32)
    shp = f_s.shape
    Xc = [(np.arange(shp[a], dtype=np.float32) - cf[a]).reshape([-1 if b == a else 1 for b in range(3)])
          for a in range(3)]
    Xc = [np.broadcast_to(x, shp) for x in Xc]
    base = [np.broadcast_to(np.arange(shp[a], dtype=np.float32).reshape([-1 if b == a else 1 for b in range(3)]), shp)
            for a in range(3)]
    coords = np.stack([base[i] - (Mf[i, 0] * Xc[0] + Mf[i, 1] * Xc[1] + Mf[i, 2] * Xc[2]) - trf[i] for i in range(3)])
    warped = map_coordinates(f_s, coords, order=1, mode='constant', cval=cval)
    inb = np.all([(coords[a] >= 0) & (coords[a] <= shp[a] - 1) for a in range(3)], axis=0)
    mask = (inb & (g != cval)).astype(np.float32)
    e = (g_s - warped) * mask
    gs = [map_coordinates(grads[i], coords, order=1, mode='nearest') for i in range(3)]
    J = [-gs[i] * Xc[j] * mask for i in range(3) for j in range(3)] + [-gs[i] * mask for i in range(3)]
    Jf = np.stack([j.ravel() for j in J]).astype(np.float64)
    return Jf @ Jf.T, Jf @ e.ravel().astype(np.float64)


def affine_refine(f, g, A0, t0, c, sigmas=(4.0, 2.0, 1.0, 0.0), max_iter=50, tol=1e-6, patience=3, cval=0.0):
    """correlate_gpu.py:600-825 (whole-volume assembly instead of slabs)."""
    from scipy.ndimage import gaussian_filter
    f = np.asarray(f, np.float32)
    g = np.asarray(g, np.float32)
    Ai = np.linalg.inv(np.asarray(A0, float))
    M, tr = np.eye(3) - Ai, Ai @ np.asarray(t0, float)
    valid = (g != cval).astype(np.float32)
    for sigma in sigmas:
        if sigma > 0:
            fs = gaussian_filter(f, sigma, mode='nearest')
            num = gaussian_filter(g * valid, sigma, mode='constant', cval=0.0)
            den = gaussian_filter(valid, sigma, mode='constant', cval=0.0)
            gs = g.copy()
            ok = den > 1e-6
            gs[ok] = num[ok] / den[ok]
        else:
            fs, gs = f, g
        grads = [np.ascontiguousarray(q) for q in np.gradient(fs)]
        best, stall = np.inf, 0
        for _ in range(max_iter):
            H, b = affine_normal_equations(fs, grads, gs, g, M, tr, c, cval)
            H += np.eye(12) * (1e-9 * np.trace(H) / 12.0 + 1e-30)
            dp = np.linalg.solve(H, b)
            M, tr = M + dp[:9].reshape(3, 3), tr + dp[9:]
            step = float(np.linalg.norm(dp))
            if step < tol:
                break
            if step < best - 1e-12:
                best, stall = step, 0
            else:
                stall += 1
                if stall >= patience:
                    break
    A = np.linalg.inv(np.eye(3) - M)
    return A, A @ tr
