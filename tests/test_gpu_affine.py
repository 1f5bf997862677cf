"""Affine pre-alignment on the GPU (cost kernel, normal equations, Gaussian
smoothing, end-to-end prealign/refine) against the oracle and the
reference's golden results."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import dvc_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def CG(cuda):
    from voxeldvc_gb300.engine import correlate_gpu
    return correlate_gpu


def test_zncc_cost_matches_reference(CG):
    import ctypes as C
    from voxeldvc_gb300 import _lib, _device as D
    c = load_golden("affine.npz")
    f_d, g_d = c["f"][::2, ::2, ::2], c["g"][::2, ::2, ::2]
    fv, fs = CG.pix_to_vox(f_d, np.float32)
    gv, gs = CG.pix_to_vox(g_d, np.float32)
    L = _lib.lib()
    import torch
    ws = torch.empty(L.vdvc_affine_workspace_bytes(), dtype=torch.uint8, device="cuda")
    cc = np.array([(n - 1) / 2.0 for n in f_d.shape])
    out = (C.c_double * 6)()
    for p, cost in zip(c["ps"], c["costs"]):
        A = CG._build_affine_matrix(p)
        _lib.check(L.vdvc_affine_zncc_sums(fv.data_ptr(), *fs, gv.data_ptr(), *gs, *(CG._ptr3(x)[1] for x in
                                           (A, p[6:9], cc)), C.cast(out, _lib.pd), ws.data_ptr(), ws.numel(),
                                           D.stream()))
        assert abs(CG._zncc_cost(list(out)) - cost) < 1e-6


def test_gaussian_filters_match_scipy(CG, cuda):
    import torch
    from scipy.ndimage import gaussian_filter
    from voxeldvc_gb300 import _lib, _device as D
    L = _lib.lib()
    rng = np.random.default_rng(1)
    img = rng.random((23, 17, 12)).astype(np.float32)
    img[rng.random(img.shape) < 0.1] = 0.0
    v, shp = CG.pix_to_vox(img, np.float32)
    out, tmp = torch.empty_like(v), torch.empty_like(v)
    t1, t2, t3 = (torch.empty_like(v) for _ in range(3))
    for sigma in (1.0, 2.0, 0.7):
        _lib.check(L.vdvc_gaussian_filter(v.data_ptr(), out.data_ptr(), *shp, sigma, 0, 0.0, None, tmp.data_ptr(),
                                          D.stream()))
        ref = gaussian_filter(img, sigma, mode='nearest').ravel(order='F')
        assert np.abs(out.cpu().numpy() - ref).max() < 1e-5
        _lib.check(L.vdvc_smooth_masked(v.data_ptr(), *shp, sigma, 0.0, out.data_ptr(), t1.data_ptr(), t2.data_ptr(),
                                        t3.data_ptr(), D.stream()))
        valid = (img != 0).astype(np.float32)
        num = gaussian_filter(img * valid, sigma, mode='constant', cval=0.0)
        den = gaussian_filter(valid, sigma, mode='constant', cval=0.0)
        exp = img.copy()
        ok = den > 1e-6
        exp[ok] = num[ok] / den[ok]
        assert np.abs(out.cpu().numpy() - exp.ravel(order='F')).max() < 1e-4


def test_normal_equations_match_oracle(CG):
    import ctypes as C
    import torch
    from voxeldvc_gb300 import _lib, _device as D
    c = load_golden("affine.npz")
    f, g = c["f"], c["g"]
    Ai = np.linalg.inv(c["A_pre"])
    M, tr, cc = np.eye(3) - Ai, Ai @ c["t_pre"], c["c_pre"]
    H0, b0 = O.affine_normal_equations(f, [np.ascontiguousarray(q) for q in np.gradient(f)], g, g, M, tr, cc)
    fv, shp = CG.pix_to_vox(f, np.float32)
    gv, _ = CG.pix_to_vox(g, np.float32)
    grad, _ = CG._grad_vox(fv, shp, np.float32)
    L = _lib.lib()
    ws = torch.empty(L.vdvc_affine_workspace_bytes(), dtype=torch.uint8, device="cuda")
    H, b = np.empty(144), np.empty(12)
    _lib.check(L.vdvc_affine_normal_equations(fv.data_ptr(), grad.data_ptr(), gv.data_ptr(), gv.data_ptr(), *shp,
                                              CG._ptr3(M)[1], CG._ptr3(tr)[1], CG._ptr3(cc)[1], 0.0,
                                              H.ctypes.data_as(_lib.pd), b.ctypes.data_as(_lib.pd), ws.data_ptr(),
                                              ws.numel(), D.stream()))
    assert np.linalg.norm(H.reshape(12, 12) - H0) / np.linalg.norm(H0) < 1e-5
    assert np.linalg.norm(b - b0) / np.linalg.norm(b0) < 1e-4
    # the Gauss-Newton steps agree
    dp = np.linalg.solve(H.reshape(12, 12), b)
    dp0 = np.linalg.solve(H0, b0)
    assert np.linalg.norm(dp - dp0) <= 1e-4 * max(1.0, np.linalg.norm(dp0))


def test_affine_refine_matches_reference(CG):
    c = load_golden("affine.npz")
    A, t, info = CG.affine_refine_gn(c["f"], c["g"], np, c["A_pre"], c["t_pre"], c["c_pre"], sigmas=(2.0, 0.0),
                                     max_iter=20)
    assert np.abs(A - c["A_ref"]).max() < 1e-4
    assert np.abs(t - c["t_ref"]).max() < 1e-3
    assert abs(info["rms_initial"] - float(c["rms_initial"])) < 1e-3
    assert info["rms_final"] < 1e-3


def test_affine_prealign_reaches_reference_cost(CG):
    c = load_golden("affine.npz")
    A, t, cc, info = CG.affine_prealign(c["f"], c["g"], np, decimate=2, maxiter=60)
    assert np.allclose(cc, c["c_pre"])
    assert info["cost_final"] <= float(c["cost_final"]) + 1e-3
    # the refine from this start lands on the same affine
    Ar, tr, _ = CG.affine_refine_gn(c["f"], c["g"], np, A, t, cc, sigmas=(2.0, 0.0), max_iter=20)
    assert np.abs(Ar - c["A_ref"]).max() < 1e-3
    assert np.abs(tr - c["t_ref"]).max() < 1e-2


def test_multiscale_with_affine_seed(CG):
    """prealign_affine=True seeds the coarsest level with the affine field."""
    from voxeldvc_gb300.engine import geometry_dvc as G
    c = load_golden("solve_multiscale.npz")
    U, res, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, scales=(2, 1, 0),
                                            K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=20,
                                            eps=1e-3, disp=False, dynamic_mask=True, freeze_mask_after=4,
                                            prealign_affine=True)
    assert np.all(np.isfinite(U))
    assert float(np.sqrt(np.mean((U - c["U"]) ** 2))) < 0.05
