"""CUDA operators (through the C ABI, via the drop-in Python API and raw
ctypes) against the reference's golden vectors and the CPU oracle."""
import ctypes as C

import numpy as np
import pytest

from conftest import OPS_CASES, load_golden
from oracle import dvc_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def api(cuda):
    from voxeldvc_gb300.engine import kernels_dvc as K, correlate_gpu as CG, geometry_dvc as G
    return K, CG, G


@pytest.mark.parametrize("case", OPS_CASES)
def test_hessian_rhs_diag(api, case):
    K, CG, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    Ndof = c["v"].size
    N, w = G.build_N_stencil(h)
    # float32: owner-computes quadrature, different rounding than the einsum chain
    Hv = K.matvec_H(c["v"], c["grad"], c["mask"], N, w, h, Nx, Ny, Nz, np)
    assert Hv.dtype == np.float32 and rel(Hv, c["out_matvec_H"]) < 5e-6
    Hv64 = K.matvec_H(c["v"].astype(np.float64), c["grad"].astype(np.float64), c["mask"], N, w, h, Nx, Ny, Nz, np)
    assert rel(Hv64, c["out_matvec_H_f64"]) < 1e-12
    d = K.build_diagonal_H(c["grad"], c["mask"], N, w, h, Nx, Ny, Nz, Ndof, np)
    assert rel(d, c["out_diag_H"]) < 5e-6
    b = CG.compute_b_gpu(c["res"], c["mask"], c["grad"], N, w, h, Nx, Ny, Nz, Ndof, np)
    assert rel(b, c["out_compute_b"]) < 5e-6
    # symmetry of H (a size-independent property): u.Hv == v.Hu
    u = np.random.default_rng(0).standard_normal(Ndof)
    Hu = K.matvec_H(u, c["grad"].astype(np.float64), c["mask"], N, w, h, Nx, Ny, Nz, np)
    assert abs(np.dot(u, Hv64) - np.dot(c["v"], Hu)) <= 1e-10 * np.abs(u).sum() * np.abs(Hv64).max()


@pytest.mark.parametrize("case", OPS_CASES)
def test_regularizers(api, case):
    K, CG, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    Ndof = c["v"].size
    K_lap, K_el = G.build_K_ref_laplacian(), G.build_K_ref(0.3)
    assert rel(K.matvec_K_ref(c["v"], K_lap, h, Nx, Ny, Nz, np), c["out_matvec_K_lap"]) < 2e-6
    assert rel(K.build_diagonal_K_ref(K_lap, h, Nx, Ny, Nz, Ndof, np), c["out_diag_K_lap"]) < 1e-14
    Rv = K.matvec_equilibrium_gap(c["v"].astype(np.float64), K_el, c["interior"], h, Nx, Ny, Nz, np)
    assert rel(Rv, c["out_matvec_eqgap"]) < 1e-12
    dR = K.build_diagonal_equilibrium_gap(K_el, c["interior"], h, Nx, Ny, Nz, Ndof, np)
    assert rel(dR, c["out_diag_eqgap"]) < 1e-12
    # per-element modulus array equal to the scalar gives the same operator
    Ee = np.full(Nx * Ny * Nz, float(h), dtype=np.float32)
    assert rel(K.matvec_K_ref(c["v"], K_lap, Ee, Nx, Ny, Nz, np), c["out_matvec_K_lap"]) < 2e-6


@pytest.mark.parametrize("case", OPS_CASES)
def test_voxel_fields(api, case):
    K, CG, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    N, _ = G.build_N_stencil(h)
    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    # gradient and erosion: bit-exact
    f_vox, grad = CG.image_grad_and_values(c["f_pix"], np)
    assert np.array_equal(f_vox, c["out_f_vox"]) and np.array_equal(grad, c["out_grad_f"])
    assert np.array_equal(CG.erode_mask0_vox(f_vox > 0, Nvx, Nvy, Nvz, np), c["out_eroded"])
    # statistics (float64 sums of float32 partials)
    assert np.allclose(CG.masked_quadpoint_mean_std(c["res"], c["mask"], h, Nx, Ny, Nz, np), c["out_stats"],
                       rtol=1e-6, atol=1e-7)
    # interpolation: separable trilinear vs N.U
    ui = CG.interp_field_vox(c["U"], N, h, Nx, Ny, Nz, np)
    assert np.abs(ui - c["out_interp"]).max() <= 2e-6 * max(1.0, np.abs(c["U"]).max())
    ucf = CG.interp_field_vox(c["U"], N, h, Nx, Ny, Nz, np, channels_first=True)
    assert np.array_equal(ucf, ui.T)
    # sampling: masks bit-exact away from the bounds, values to float32 rounding
    go = tuple(int(o) for o in c["g_origin"])
    gv, gm = CG.sample_deformed_field(c["U"], c["g_pix"], N, h, Nx, Ny, Nz, np, g_origin=go, mask0_vox=c["mask"])
    ref_g, ref_m = c["out_sample_g"], c["out_sample_mask"]
    u = O.interp_field(c["U"].astype(np.float64), h, Nx, Ny, Nz)
    v = np.arange(u.shape[0])
    pos = np.stack([v % Nvx, (v // Nvx) % Nvy, v // (Nvx * Nvy)], 1) + u - np.array(go)
    gshape = np.array(c["g_pix"].shape) - 1
    near = (np.abs(pos).min(1) < 1e-4) | (np.abs(pos - gshape).min(1) < 1e-4)
    assert np.array_equal(gm[~near], ref_m[~near])
    assert np.abs(gv - ref_g).max() < 1e-5
    am = CG.compute_active_mask(c["U"], c["g_pix"], Nx, Ny, Nz, h, np, g_origin=go, mask0_vox=c["mask"])
    assert np.array_equal(am, gm)


@pytest.mark.parametrize("case", OPS_CASES)
def test_image_grad_stats_fused(api, case):
    """The level set-up's fused pass: gradient and mask0 bit-identical to
    vdvc_image_grad, the sums of f over mask0 those of vdvc_masked_stats
    (float64 sums of float32 partials in another order)."""
    import torch
    from voxeldvc_gb300 import _lib
    K, CG, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    f_vox, fs = CG.pix_to_vox(c["f_pix"], np.float32)
    glt = float(np.quantile(c["f_pix"], 0.2))  # a threshold that leaves mask0 partial
    grad_ref, m_ref = CG._grad_vox(f_vox, fs, np.float32, glt)
    ref3 = CG._stats_sums(f_vox, m_ref, h, Nx, Ny, Nz)
    n = Nvx * Nvy * Nvz
    grad = torch.empty(3 * n, dtype=torch.float32, device="cuda")
    m0 = torch.empty(n, dtype=torch.uint8, device="cuda")
    out3 = torch.zeros(3, dtype=torch.float64, device="cuda")
    ws = torch.empty(1 << 18, dtype=torch.uint8, device="cuda")
    L = _lib.lib()
    s = torch.cuda.current_stream().cuda_stream
    _lib.check(L.vdvc_image_grad_stats(f_vox.data_ptr(), Nvx, Nvy, Nvz, glt, grad.data_ptr(), m0.data_ptr(), h, Nx,
                                       Ny, Nz, out3.data_ptr(), ws.data_ptr(), ws.numel(), s))
    assert torch.equal(grad, grad_ref) and torch.equal(m0, m_ref)
    assert 0 < m0.sum().item() < n
    assert np.allclose(out3.cpu().numpy(), ref3, rtol=1e-6)
    with pytest.raises(Exception):  # an image that is not the mesh's voxel grid
        _lib.check(L.vdvc_image_grad_stats(f_vox.data_ptr(), Nvx, Nvy, Nvz, glt, grad.data_ptr(), m0.data_ptr(), h,
                                           Nx + 1, Ny, Nz, out3.data_ptr(), ws.data_ptr(), ws.numel(), s))


@pytest.mark.parametrize("case", ["A", "B", "C"])
def test_generic_pcg(api, case):
    K, CG, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    Ndof = c["v"].size
    N, w = G.build_N_stencil(h)
    K_lap = G.build_K_ref_laplacian()
    ll = float(c["out_pcg_ll"])
    import torch
    dg = K.build_diagonal_H(c["grad"], c["mask"], N, w, h, Nx, Ny, Nz, Ndof, np) + \
        ll * K.build_diagonal_K_ref(K_lap, h, Nx, Ny, Nz, Ndof, np)
    Minv = 1.0 / (dg + 1e-5 * float(dg.min()))

    def A(x):
        return K.matvec_H(x, c["grad"], c["mask"], N, w, h, Nx, Ny, Nz, torch) + \
            ll * K.matvec_K_ref(x, K_lap, h, Nx, Ny, Nz, torch)

    x = K.pcg(A, c["b_pcg"], Minv, np, max_iter=300, tol=1e-7)
    assert rel(x, c["out_pcg_x"]) < 1e-5


def test_raw_c_abi_matvec(cuda):
    """vdvc_matvec_H called directly through ctypes with device pointers."""
    torch = cuda
    from voxeldvc_gb300 import _lib
    L = _lib.lib()
    c = load_golden("ops_A.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    v = torch.from_numpy(c["v"]).cuda()
    g = torch.from_numpy(c["grad"]).cuda()
    m = torch.from_numpy(c["mask"]).cuda()
    out = torch.empty_like(v)
    nws = L.vdvc_workspace_bytes(_lib.F32, h, Nx, Ny, Nz)
    ws = torch.empty(nws, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    st = L.vdvc_matvec_H(v.data_ptr(), g.data_ptr(), m.data_ptr(), _lib.F32, h, Nx, Ny, Nz, out.data_ptr(),
                         ws.data_ptr(), nws, s)
    assert st == 0
    assert rel(out.cpu().numpy(), c["out_matvec_H"]) < 5e-6
    # a too-small workspace is refused, not overrun
    st = L.vdvc_matvec_H(v.data_ptr(), g.data_ptr(), m.data_ptr(), _lib.F32, h, Nx, Ny, Nz, out.data_ptr(),
                         ws.data_ptr(), 16, s)
    assert st == _lib.ERR_WORKSPACE
    # bad dtype / sizes map to VDVC_ERR_ARG
    assert L.vdvc_matvec_H(v.data_ptr(), g.data_ptr(), m.data_ptr(), 7, h, Nx, Ny, Nz, out.data_ptr(), ws.data_ptr(),
                           nws, s) == _lib.ERR_ARG
    assert L.vdvc_matvec_H(v.data_ptr(), g.data_ptr(), m.data_ptr(), _lib.F32, 0, Nx, Ny, Nz, out.data_ptr(),
                           ws.data_ptr(), nws, s) == _lib.ERR_ARG
    torch.cuda.synchronize()


def test_fft_rigid_shift(api):
    K, CG, G = api
    c = load_golden("fft.npz")
    assert np.array_equal(CG.fft_rigid_shift(c["f1"], c["g1"], np), c["d1"])
    assert np.array_equal(CG.fft_rigid_shift(c["f2"], c["g2"], np), c["d2"])
    # float32 volumes transform in single precision (complex64, as the
    # reference's fftn does for float32 arrays under CuPy): the same shifts
    for a, b, d in ((c["f1"], c["g1"], c["d1"]), (c["f2"], c["g2"], c["d2"])):
        fv, fs = CG.pix_to_vox(a, np.float32)
        gv, gs = CG.pix_to_vox(b, np.float32)
        assert np.array_equal(CG._fft_shift_vox(fv, fs, gv, gs, np.float32), d)


def test_pix_to_vox_dtypes(api):
    K, CG, G = api
    rng = np.random.default_rng(3)
    for dt in (np.float32, np.float64, np.uint16, np.uint8, np.int16, np.int32):
        a = (rng.random((5, 7, 3)) * 200).astype(dt)
        t, shape = CG.pix_to_vox(a, np.float32)
        assert shape == (5, 7, 3)
        assert np.array_equal(t.cpu().numpy(), a.astype(np.float32).ravel(order='F'))
