"""Matrix-free operators and PCG of the DVC Hessian and regularizers.

Drop-in counterpart of the reference module engine/kernels_dvc.py: same
function names and positional layout.  Every operator runs on the GPU
through libvdvc.so; `xp` selects the type of the returned arrays (numpy ->
host numpy arrays, anything else -> torch CUDA tensors), inputs may be
numpy arrays or torch tensors.  `chunk_size` is accepted and ignored: the
kernels work on whole meshes.

Dtype behaviour follows the reference: an operator computes in the
promoted type of its floating inputs and returns the dtype the reference
returns (v.dtype for matvecs, grad dtype for diag H).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _device as D
from .. import _lib
from .geometry_dvc import build_N_stencil

# ---------------------------------------------------------------------------
# Implicit connectivity (kernels_dvc.py:32-89) -- index tables for callers;
# the kernels compute the same indices in registers.
# ---------------------------------------------------------------------------

_CORNER_NODE_OFFSETS = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))


def _host_index(x):
    return x.detach().cpu().numpy() if D.is_tensor(x) else np.asarray(x)


def _index_out(a, xp, like=None):
    if D.wants_host(xp) and not D.is_tensor(like):
        return a
    return D.to_device(a)


def get_elem_dofs(elem_ids, Nx, Ny, xp):
    """(chunk, 24) dof ids, node-major with the Hex8 corner order.
    Reference: engine/kernels_dvc.py:32-61."""
    e = _host_index(elem_ids)
    i, j, k = e % Nx, (e // Nx) % Ny, e // (Nx * Ny)
    base = i + j * (Nx + 1) + k * (Nx + 1) * (Ny + 1)
    offs = np.array([dx + dy * (Nx + 1) + dz * (Nx + 1) * (Ny + 1) for dx, dy, dz in _CORNER_NODE_OFFSETS],
                    dtype=e.dtype)
    nodes = base[:, None] + offs[None, :]
    dofs = (3 * nodes[:, :, None] + np.arange(3, dtype=e.dtype)[None, None, :]).reshape(-1, 24)
    return _index_out(dofs, xp, elem_ids)


def get_voxel_offsets(h, Nx, Ny, xp):
    """((h+1)^3,) flat voxel offsets of the stencil points (meshgrid 'ij').
    Reference: engine/kernels_dvc.py:64-78."""
    Nvx, Nvy = Nx * h + 1, Ny * h + 1
    q = np.arange(h + 1, dtype=np.int32)
    offs = (q[:, None, None] + q[None, :, None] * Nvx + q[None, None, :] * (Nvx * Nvy)).reshape(-1)
    return _index_out(offs.astype(np.int32), xp)


def get_elem_voxel_origins(elem_ids, h, Nx, Ny, xp):
    """Flat voxel index of each element's q = (0,0,0) voxel.
    Reference: engine/kernels_dvc.py:81-89."""
    e = _host_index(elem_ids)
    Nvx, Nvy = Nx * h + 1, Ny * h + 1
    i, j, k = e % Nx, (e // Nx) % Ny, e // (Nx * Ny)
    return _index_out(h * (i + j * Nvx + k * Nvx * Nvy), xp, elem_ids)


# ---------------------------------------------------------------------------
# Post-solve diagnostic masks (kernels_dvc.py:92-341), one GPU pass chain
# (`vdvc_unsafe_masks`): element block flags -> node flags -> element flags
# -> voxel flags.  Inputs are flat x-fastest voxel masks; outputs are host
# bool arrays as in the reference (which runs these on the CPU).
# ---------------------------------------------------------------------------

def boundary_element_mask(Nx, Ny, Nz):
    """(Nx*Ny*Nz,) bool, x-fastest element order: the outer element shell.
    Reference: engine/kernels_dvc.py:92-115."""
    i = np.arange(Nx)[None, None, :]
    j = np.arange(Ny)[None, :, None]
    k = np.arange(Nz)[:, None, None]
    m = (i == 0) | (i == Nx - 1) | (j == 0) | (j == Ny - 1) | (k == 0) | (k == Nz - 1)
    return np.broadcast_to(m, (Nz, Ny, Nx)).reshape(-1).copy()


def _unsafe_masks(active_vox, h, Nx, Ny, Nz, mask0_vox=None, frac_threshold=0.0, min_material_frac=0.5,
                  vox=False, elem=False, node=False, lost=False):
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    Ne, Nn = Nx * Ny * Nz, (Nx + 1) * (Ny + 1) * (Nz + 1)
    a = D.mask_u8(active_vox).reshape(-1)
    m0 = D.mask_u8(mask0_vox).reshape(-1) if mask0_vox is not None else None
    if a.numel() != Nvox or (m0 is not None and m0.numel() != Nvox):
        raise ValueError(f"voxel masks must have {Nvox} entries")
    outs = [D.empty(n, np.uint8) if want else None for want, n in ((vox, Nvox), (elem, Ne), (node, Nn), (lost, Ne))]
    nbytes = int(_lib.lib().vdvc_unsafe_masks_workspace_bytes(Nx, Ny, Nz))
    ws = D.scratch.get(nbytes)
    _lib.check(_lib.lib().vdvc_unsafe_masks(a.data_ptr(), D.ptr(m0), int(h), Nx, Ny, Nz, float(frac_threshold),
                                            float(min_material_frac), *(D.ptr(o) for o in outs), ws.data_ptr(),
                                            ws.numel(), D.stream()), "unsafe masks")
    return [D.out(o.view(D.torch().bool), np) if o is not None else None for o in outs]


def compute_unsafe_voxel_mask(active_vox, h, Nx, Ny, Nz):
    """(Nvox,) bool: voxels of every element touching an unsafe node (a node
    of an element holding an inactive voxel), plus the outer element shell.
    Reference: engine/kernels_dvc.py:166-193."""
    return _unsafe_masks(active_vox, h, Nx, Ny, Nz, vox=True)[0]


def compute_unsafe_element_mask(active_vox, h, Nx, Ny, Nz):
    """(Nx*Ny*Nz,) bool, x-fastest: elements touching an unsafe node, plus
    the outer element shell.
    Reference: engine/kernels_dvc.py:196-213."""
    return _unsafe_masks(active_vox, h, Nx, Ny, Nz, elem=True)[1]


def compute_unsafe_node_mask(active_vox, h, Nx, Ny, Nz):
    """((Nx+1)*(Ny+1)*(Nz+1),) bool: nodes of elements holding an inactive
    voxel, plus the nodes of the outer element shell.
    Reference: engine/kernels_dvc.py:216-233."""
    return _unsafe_masks(active_vox, h, Nx, Ny, Nz, node=True)[2]


def compute_overlap_lost_element_mask(active_vox, mask0_vox, h, Nx, Ny, Nz, frac_threshold=0.0,
                                      min_material_frac=0.5):
    """(Nx*Ny*Nz,) bool, x-fastest: elements sharing a node with an element
    whose lost material fraction exceeds frac_threshold, elements whose
    material count fraction is below min_material_frac, and the outer
    element shell.
    Reference: engine/kernels_dvc.py:236-341."""
    return _unsafe_masks(active_vox, h, Nx, Ny, Nz, mask0_vox, frac_threshold, min_material_frac, lost=True)[3]


def auto_chunk_size(nq, max_tensor_elems=20_000_000):
    """Element-chunk size of the reference's chunked loops (kept for API
    compatibility; the kernels here do not chunk).
    Reference: engine/kernels_dvc.py:444-449."""
    return max(1, max_tensor_elems // (nq * 24))


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def _float_dtype(*arrays):
    dt = np.result_type(*[D.np_dtype_of(a) for a in arrays])
    if dt not in (np.float32, np.float64):
        dt = np.dtype(np.float64) if dt.kind == 'f' and dt.itemsize > 4 else np.dtype(np.float32)
    return np.dtype(dt)


def _check_stencil(N_stencil, w_stencil, h):
    """The kernels evaluate the standard voxel-centre Hex8 stencil in
    registers; refuse any other table instead of silently ignoring it."""
    N = _host_index(N_stencil)
    w = _host_index(w_stencil)
    nq = (h + 1) ** 3
    if N.shape != (nq, 8) or w.shape != (nq,):
        raise ValueError(f"N_stencil/w_stencil must have shapes ({nq}, 8)/({nq},) for h={h}")
    Nr, wr = build_N_stencil(h)
    tol = 1e-6 if N.dtype == np.float32 else 1e-12
    if not (np.allclose(N, Nr, rtol=0, atol=tol) and np.allclose(w, wr, rtol=0, atol=tol)):
        raise ValueError("only the voxel-centre Hex8 stencil of build_N_stencil(h) is supported")


def _mesh_sizes(h, Nx, Ny, Nz):
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    return Nvox, Ndof


def _ws(dtype, h, Nx, Ny, Nz):
    n = _lib.lib().vdvc_workspace_bytes(D.code_of(dtype), h, Nx, Ny, Nz)
    if n == 0:
        _lib.check(_lib.ERR_ARG, "workspace size query")
    return D.scratch.get(n), n


def _kmat(K):
    K = np.ascontiguousarray(_host_index(K), dtype=np.float64)
    if K.shape != (24, 24):
        raise ValueError("K_ref must be 24x24")
    return K, K.ctypes.data_as(_lib.pd)


def _E_args(E_elem, Ne, dtype):
    """(device array or None, scalar) for a per-element modulus argument."""
    if D.is_tensor(E_elem) or (np.ndim(E_elem) > 0 and np.size(E_elem) > 1):
        a = D.to_device(E_elem, dtype).reshape(-1)
        if a.numel() != Ne:
            raise ValueError(f"E_elem has {a.numel()} entries, expected {Ne}")
        return a, 0.0
    return None, float(np.asarray(_host_index(E_elem)).reshape(-1)[0])


# ---------------------------------------------------------------------------
# Regularizer operators (kernels_dvc.py:349-437)
# ---------------------------------------------------------------------------

def matvec_K_ref(v, K_ref, E_elem, Nx, Ny, Nz, xp, chunk_size=500_000):
    """f = sum_e E_e P_e^T K_ref P_e v (node-centric stencil, no scatter).
    Reference: engine/kernels_dvc.py:349-374."""
    out_dt = D.np_dtype_of(v)
    dt = _float_dtype(v)
    vd = D.to_device(v, dt).reshape(-1)
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    if vd.numel() != Ndof:
        raise ValueError(f"v has {vd.numel()} entries, expected Ndof={Ndof}")
    Kh, Kp = _kmat(K_ref)
    Ed, Es = _E_args(E_elem, Nx * Ny * Nz, dt)
    out = D.empty(Ndof, dt)
    L = _lib.lib()
    _lib.check(L.vdvc_matvec_K_ref(vd.data_ptr(), D.code_of(dt), Kp, D.ptr(Ed), Es, Nx, Ny, Nz, out.data_ptr(),
                                   D.stream()), "matvec_K_ref")
    if out_dt != dt and out_dt.kind == 'f':
        out = out.to(D.torch_dtype(out_dt))
    return D.out(out, xp)


def build_diagonal_K_ref(K_ref, E_elem, Nx, Ny, Nz, Ndof, xp):
    """Diagonal of the K_ref operator (float64, like the reference's
    np.diag of the float64 K_ref).
    Reference: engine/kernels_dvc.py:377-392."""
    Kh, Kp = _kmat(K_ref)
    dt = np.dtype(np.float64)
    Ed, Es = _E_args(E_elem, Nx * Ny * Nz, dt)
    out = D.empty(Ndof, dt)
    _lib.check(_lib.lib().vdvc_diag_K_ref(D.code_of(dt), Kp, D.ptr(Ed), Es, Nx, Ny, Nz, out.data_ptr(),
                                          D.stream()), "build_diagonal_K_ref")
    return D.out(out, xp)


def matvec_equilibrium_gap(v, K_ref_elastic, interior_mask, E_elem, Nx, Ny, Nz, xp, chunk_size=500_000):
    """f = K (P_i (K v)), K = sum_e E_e P_e^T K_el P_e.
    Reference: engine/kernels_dvc.py:402-417."""
    out_dt = D.np_dtype_of(v)
    dt = _float_dtype(v, interior_mask) if D.np_dtype_of(interior_mask).kind == 'f' else _float_dtype(v)
    vd = D.to_device(v, dt).reshape(-1)
    Pi = D.to_device(interior_mask, dt).reshape(-1)
    Kh, Kp = _kmat(K_ref_elastic)
    Ed, Es = _E_args(E_elem, Nx * Ny * Nz, dt)
    Ndof = vd.numel()
    out = D.empty(Ndof, dt)
    ws, n = _ws(dt, 1, Nx, Ny, Nz)
    _lib.check(_lib.lib().vdvc_matvec_equilibrium_gap(vd.data_ptr(), D.code_of(dt), Kp, Pi.data_ptr(), D.ptr(Ed),
                                                      Es, Nx, Ny, Nz, out.data_ptr(), ws.data_ptr(), n,
                                                      D.stream()), "matvec_equilibrium_gap")
    res_dt = np.result_type(out_dt, dt)
    if res_dt != dt:
        out = out.to(D.torch_dtype(res_dt))
    return D.out(out, xp)


def rademacher_probes(Ndof, n_probes=32, seed=0):
    """The reference's probe sequence: n_probes draws of
    np.random.default_rng(seed).choice([-1., 1.], size=Ndof), as int8."""
    rng = np.random.default_rng(seed)
    z = np.empty((n_probes, Ndof), dtype=np.int8)
    for p in range(n_probes):
        z[p] = rng.choice([-1.0, 1.0], size=Ndof).astype(np.int8)
    return z


def build_diagonal_equilibrium_gap(K_ref_elastic, interior_mask, E_elem, Nx, Ny, Nz, Ndof, xp, n_probes=32,
                                   seed=0):
    """Hutchinson estimate of diag(K P_i K) with the reference's Rademacher
    probes (generated on the host with numpy's default_rng(seed), as in
    kernels_dvc.py:430-433), clipped at 1e-12 max|diag|; float64."""
    probes = D.to_device(rademacher_probes(Ndof, n_probes, seed))
    Pi = D.to_device(interior_mask, np.float64).reshape(-1)
    Kh, Kp = _kmat(K_ref_elastic)
    Ed, Es = _E_args(E_elem, Nx * Ny * Nz, np.float64)
    out = D.empty(Ndof, np.float64)
    ws, n = _ws(np.float64, 1, Nx, Ny, Nz)
    _lib.check(_lib.lib().vdvc_diag_equilibrium_gap(probes.data_ptr(), n_probes, Kp, Pi.data_ptr(), D.ptr(Ed), Es,
                                                    Nx, Ny, Nz, out.data_ptr(), ws.data_ptr(), n, D.stream()),
               "build_diagonal_equilibrium_gap")
    return D.out(out, xp)


# ---------------------------------------------------------------------------
# Correlation Hessian (kernels_dvc.py:452-543)
# ---------------------------------------------------------------------------

def _grad_mask(grad_f_vox, mask0_vox, dt, Nvox):
    g = D.to_device(grad_f_vox, dt).reshape(-1)
    if g.numel() != 3 * Nvox:
        raise ValueError(f"grad_f_vox must have shape ({Nvox}, 3)")
    m = D.mask_u8(mask0_vox).reshape(-1)
    if m.numel() != Nvox:
        raise ValueError(f"mask must have {Nvox} entries")
    return g, m


def matvec_H(v, grad_f_vox, mask0_vox, N_stencil, w_stencil, h, Nx, Ny, Nz, xp, chunk_size=None):
    """f = H v = sum_e sum_q w_q m_q (v_eq . v_loc) v_eq, matrix-free.
    Reference: engine/kernels_dvc.py:452-506."""
    _check_stencil(N_stencil, w_stencil, h)
    Nvox, Ndof = _mesh_sizes(h, Nx, Ny, Nz)
    out_dt = D.np_dtype_of(v)
    dt = _float_dtype(v, grad_f_vox)
    vd = D.to_device(v, dt).reshape(-1)
    if vd.numel() != Ndof:
        raise ValueError(f"v has {vd.numel()} entries, expected Ndof={Ndof}")
    g, m = _grad_mask(grad_f_vox, mask0_vox, dt, Nvox)
    out = D.empty(Ndof, dt)
    ws, n = _ws(dt, h, Nx, Ny, Nz)
    _lib.check(_lib.lib().vdvc_matvec_H(vd.data_ptr(), g.data_ptr(), m.data_ptr(), D.code_of(dt), h, Nx, Ny, Nz,
                                        out.data_ptr(), ws.data_ptr(), n, D.stream()), "matvec_H")
    if out_dt != dt and out_dt.kind == 'f':
        out = out.to(D.torch_dtype(out_dt))
    return D.out(out, xp)


def matvec_H_mixed(v, grad_f_vox, mask0_vox, N_stencil, w_stencil, h, Nx, Ny, Nz, xp, chunk_size=None):
    """H v in the precision form: BF16 gradient, element Hessians formed with
    FP32 accumulation, FP32 application.  Always computes in float32."""
    _check_stencil(N_stencil, w_stencil, h)
    Nvox, Ndof = _mesh_sizes(h, Nx, Ny, Nz)
    dt = np.dtype(np.float32)
    vd = D.to_device(v, dt).reshape(-1)
    if vd.numel() != Ndof:
        raise ValueError(f"v has {vd.numel()} entries, expected Ndof={Ndof}")
    g, m = _grad_mask(grad_f_vox, mask0_vox, dt, Nvox)
    out = D.empty(Ndof, dt)
    n = _lib.lib().vdvc_eh_workspace_bytes(h, Nx, Ny, Nz)
    if n == 0:
        _lib.check(_lib.ERR_ARG, "element-Hessian workspace size query")
    ws = D.scratch.get(n)
    _lib.check(_lib.lib().vdvc_matvec_H_mixed(vd.data_ptr(), g.data_ptr(), m.data_ptr(), h, Nx, Ny, Nz,
                                              out.data_ptr(), ws.data_ptr(), n, D.stream()), "matvec_H_mixed")
    return D.out(out, xp)


class ElementHessians:
    """The operator of matvec_H held as element Hessians (the 162 distinct
    entries of each element's 24x24 block, FP32 accumulation): formed once
    from the float32 gradient -- or from its BF16 rounding with bf16=True --
    and applied many times, as the GN solver's PCG does at element edges
    >= 6.  The reference applies H matrix-free on every call
    (engine/kernels_dvc.py:452-506); the float32 form sums the same float32
    products in another order."""

    def __init__(self, grad_f_vox, mask0_vox, h, Nx, Ny, Nz, bf16=False):
        torch = D.torch()
        Nvox, self.Ndof = _mesh_sizes(h, Nx, Ny, Nz)
        self.mesh = (h, Nx, Ny, Nz)
        L = _lib.lib()
        nT = L.vdvc_eh_bytes(h, Nx, Ny, Nz)
        nw = L.vdvc_eh_op_workspace_bytes(h, Nx, Ny, Nz)
        if nT == 0 or nw == 0:
            _lib.check(_lib.ERR_ARG, "element-Hessian size query")
        g, m = _grad_mask(grad_f_vox, mask0_vox, np.dtype(np.float32), Nvox)
        if bf16:
            g = g.to(torch.bfloat16)
        self.T = torch.empty(nT // 4, dtype=torch.float32, device=D.device())
        self.ws = torch.zeros(nw, dtype=torch.uint8, device=D.device())
        _lib.check(L.vdvc_eh_form(g.data_ptr(), int(bool(bf16)), m.data_ptr(), h, Nx, Ny, Nz, self.T.data_ptr(),
                                  self.ws.data_ptr(), nw, D.stream()), "ElementHessians")
        self._keep = g

    def matvec_into(self, v, out):
        """out = H v for float32 CUDA tensors of Ndof entries (no checks,
        no allocation: the timing path)."""
        h, Nx, Ny, Nz = self.mesh
        _lib.check(_lib.lib().vdvc_eh_apply(self.T.data_ptr(), v.data_ptr(), h, Nx, Ny, Nz, out.data_ptr(),
                                            self.ws.data_ptr(), self.ws.numel(), D.stream()), "ElementHessians")

    def matvec(self, v, xp):
        vd = D.to_device(v, np.dtype(np.float32)).reshape(-1).contiguous()
        if vd.numel() != self.Ndof:
            raise ValueError(f"v has {vd.numel()} entries, expected Ndof={self.Ndof}")
        out = D.empty(self.Ndof, np.dtype(np.float32))
        self.matvec_into(vd, out)
        self.status()
        return D.out(out, xp)

    def status(self):
        """Raises VdvcTimeout if a bulk-copy wait of an apply timed out."""
        h, Nx, Ny, Nz = self.mesh
        _lib.check(_lib.lib().vdvc_eh_status(self.ws.data_ptr(), self.ws.numel(), h, Nx, Ny, Nz, D.stream()),
                   "ElementHessians")


def build_diagonal_H(grad_f_vox, mask0_vox, N_stencil, w_stencil, h, Nx, Ny, Nz, Ndof, xp, chunk_size=None):
    """diag(H)[i] = sum over (e,q) touching dof i of w_q m_q v_eq[i]^2.
    Reference: engine/kernels_dvc.py:509-543."""
    _check_stencil(N_stencil, w_stencil, h)
    Nvox, nd = _mesh_sizes(h, Nx, Ny, Nz)
    if nd != Ndof:
        raise ValueError(f"Ndof={Ndof} does not match the mesh ({nd})")
    dt = _float_dtype(grad_f_vox)
    g, m = _grad_mask(grad_f_vox, mask0_vox, dt, Nvox)
    out = D.empty(Ndof, dt)
    ws, n = _ws(dt, h, Nx, Ny, Nz)
    _lib.check(_lib.lib().vdvc_diag_H(g.data_ptr(), m.data_ptr(), D.code_of(dt), h, Nx, Ny, Nz, out.data_ptr(),
                                      ws.data_ptr(), n, D.stream()), "build_diagonal_H")
    return D.out(out, xp)


# ---------------------------------------------------------------------------
# Preconditioned conjugate gradient (kernels_dvc.py:550-583)
# ---------------------------------------------------------------------------

def pcg(matvec, b, M_inv, xp, x0=None, max_iter=1000, tol=1e-8, verbose=False):
    """Jacobi PCG for an arbitrary callable matvec (v -> A v) on device
    vectors.  The vector updates and the float64 dot products are libvdvc
    kernels; `matvec` is called with CUDA tensors and may return a CUDA
    tensor or anything convertible to one.  Solver objects of this package
    bypass this loop with their fused, graph-replayed PCG.
    Reference: engine/kernels_dvc.py:550-583."""
    dt = _float_dtype(b, M_inv)
    bd = D.to_device(b, dt).reshape(-1)
    Md = D.to_device(M_inv, dt).reshape(-1)
    n = bd.numel()
    x = D.zeros(n, dt) if x0 is None else D.to_device(x0, dt).reshape(-1).clone()
    r, z, p = D.empty(n, dt), D.empty(n, dt), D.empty(n, dt)
    L = _lib.lib()
    ws = D.torch().empty(L.vdvc_pcg_workspace_bytes(), dtype=D.torch().uint8, device=D.device())
    wsn = ws.numel()
    code = D.code_of(dt)

    def _apply(v):
        out = matvec(v)
        return D.to_device(out, dt).reshape(-1)

    Ax = _apply(x)
    _lib.check(L.vdvc_pcg_begin(bd.data_ptr(), Ax.data_ptr(), Md.data_ptr(), code, n, r.data_ptr(), z.data_ptr(),
                                p.data_ptr(), int(max_iter), float(tol), ws.data_ptr(), wsn, D.stream()), "pcg")
    res = C.c_double(0.0)
    done = C.c_int(0)
    for it in range(max_iter):
        Ap = _apply(p)
        _lib.check(L.vdvc_pcg_step(Ap.data_ptr(), Md.data_ptr(), code, n, x.data_ptr(), r.data_ptr(),
                                   z.data_ptr(), p.data_ptr(), ws.data_ptr(), wsn, C.byref(res), C.byref(done),
                                   D.stream()), "pcg")
        rv = res.value
        if verbose and (it % 10 == 0 or it < 5):
            print(f"  PCG iter {it:4d}  rel.residual = {rv:.3e}")
        if rv < tol:
            if verbose:
                print(f"  Converged at iter {it}, residual = {rv:.3e}")
            break
        _lib.check(L.vdvc_pcg_direction(z.data_ptr(), p.data_ptr(), code, n, ws.data_ptr(), wsn, D.stream()), "pcg")
    return D.out(x, xp)
