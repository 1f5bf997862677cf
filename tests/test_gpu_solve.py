"""End-to-end GN solves on the GPU against the reference's golden solves
(displacement tolerance: 1e-3 voxel RMS at FP32, per the parity bar) and
the reference's own multiscale tests, replayed on the drop-in API."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-3  # voxel RMS of nodal displacements, FP32 solve vs reference


def rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


@pytest.fixture(scope="module")
def api(cuda):
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    return CG, G


def test_correlate_sinusoid(api):
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False)
    U, res, dU = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, **kw)
    assert rms(U, c["U"]) < RMS_TOL
    assert np.abs(res - c["res"]).max() < 1e-2
    assert U.shape == c["U"].shape and res.shape == c["res"].shape and dU.shape == c["dU"].shape


def test_multiscale_single_scale_matches_direct(api):
    # reference tests/test_dvc_gpu_multiscale.py:43-57 on this API
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False)
    Ud, rd, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, **kw)
    Um, rm, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, scales=(0,), fft_prealign=False, **kw)
    assert np.allclose(Ud, Um, atol=1e-12)
    assert np.allclose(rd, rm, atol=1e-12)


def test_multiscale_pyramid(api):
    # reference tests/test_dvc_gpu_multiscale.py:60-72, plus the golden pyramid
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=30, eps=1e-3, disp=False)
    Ud, _, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, **kw)
    Um, _, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, scales=(2, 1, 0), **kw)
    assert np.all(np.isfinite(Um))
    assert np.allclose(Ud, Um, atol=1e-2)
    assert rms(Um, c["U_ms"]) < RMS_TOL


def test_dynamic_mask_freeze(api):
    CG, G = api
    c = load_golden("solve_dynamic.npz")
    U, res, _ = CG.correlate_gpu(c["f"], c["g"], 4, 4, 4, 4, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(),
                                 l0=8.0, maxiter=12, eps=1e-4, disp=False, dynamic_mask=True, freeze_mask_after=2,
                                 glt=0.0)
    assert rms(U, c["U"]) < RMS_TOL


def test_equilibrium_gap(api):
    CG, G = api
    c = load_golden("solve_eqgap.npz")
    U, res, _ = CG.correlate_gpu(c["f"], c["g"], 3, 3, 3, 4, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(),
                                 K_ref_elastic=G.build_K_ref(0.3), reg_type='equilibrium_gap', reg_exponent=4,
                                 l0=18.0, maxiter=10, eps=1e-4, disp=False, dynamic_mask=True, freeze_mask_after=4)
    assert rms(U, c["U"]) < RMS_TOL


def test_multiscale_fft_dynamic(api):
    CG, G = api
    c = load_golden("solve_multiscale.npz")
    U, res, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, scales=(2, 1, 0),
                                            K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=20,
                                            eps=1e-3, disp=False, dynamic_mask=True, freeze_mask_after=4,
                                            fft_prealign=True)
    assert rms(U, c["U"]) < RMS_TOL


def test_float64_solve_tighter(api):
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False,
              dtype=np.float64)
    U, _, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, **kw)
    assert rms(U, c["U"]) < 1e-4


def test_device_arrays_in_and_out(api, cuda):
    torch = cuda
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False)
    U, res, dU = CG.correlate_gpu(torch.from_numpy(c["f"]).cuda(), torch.from_numpy(c["g"]).cuda(), 2, 2, 2, 8,
                                  xp=torch, **kw)
    assert U.is_cuda and res.is_cuda
    assert rms(U.cpu().numpy(), c["U"]) < RMS_TOL


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.uint16, np.uint8])
def test_host_array_layout(api, cuda, dtype):
    """pix_to_vox of a host array large enough for the in-place read (where
    the device reads pageable host memory) against the same array staged as
    a device tensor: identical vox layout and values."""
    torch = cuda
    CG, G = api
    rng = np.random.default_rng(5)
    a = (rng.random((97, 83, 71)) * 200).astype(dtype)
    assert a.nbytes >= CG._DIRECT_MIN_BYTES or dtype == np.uint8
    v_host, s_host = CG.pix_to_vox(a, np.float32)
    v_dev, s_dev = CG.pix_to_vox(torch.from_numpy(a.astype(np.float64)).cuda(), np.float32)
    assert s_host == s_dev == a.shape
    assert torch.equal(v_host, v_dev)
    assert np.array_equal(v_host.cpu().numpy(), a.transpose(2, 1, 0).reshape(-1).astype(np.float32))


@pytest.mark.parametrize("dtype", [np.float32, np.uint16])
def test_strided_layout(api, cuda, dtype):
    """vdvc_pix_to_vox_strided = pix_to_vox then the strided decimation, bit
    for bit, from host memory (where the device reads it in place) and from
    device tensors, for steps 1-4 and extents that are not multiples of the
    step."""
    torch = cuda
    CG, G = api
    from voxeldvc_gb300 import _lib, _device as D
    rng = np.random.default_rng(8)
    a = (rng.random((97, 83, 71)) * 200).astype(dtype)
    full, fs = CG.pix_to_vox(a, np.float32)
    t = torch.from_numpy(a.astype(np.float64)).cuda()
    for s in (1, 2, 3, 4):
        ref, o = CG._decimate(full, fs, s, np.float32)
        if CG._host_readable(a):
            got, og = CG._pix_to_vox_strided_host(a, s, np.float32)
            torch.cuda.synchronize()
            assert og == o and torch.equal(got, ref)
        out = D.empty(ref.numel(), np.float32)
        for mb in (0, 7):  # one block per tile, and a bounded grid walking the tiles
            out.zero_()
            _lib.check(_lib.lib().vdvc_pix_to_vox_strided(t.data_ptr(), _lib.F64, *a.shape, s, mb, out.data_ptr(),
                                                          _lib.F32, D.stream()))
            assert torch.equal(out, ref), (s, mb)


def test_multiscale_host_arrays_overlap(api, cuda):
    """A multiscale solve from host arrays (coarsest level read in place at
    its step, the full-resolution layout on a side stream under it) equals
    the same solve from device tensors bit for bit."""
    torch = cuda
    CG, G = api
    from voxeldvc_gb300 import synth
    f = synth.texture((129, 129, 129), 200, seed=3, cyl_seed=4)
    fh = f.view(129, 129, 129).permute(2, 1, 0).contiguous().cpu().numpy()
    g = np.roll(fh, (2, -1, 1), axis=(0, 1, 2)).copy()
    kw = dict(scales=(2, 1, 0), K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=4, disp=False,
              fft_prealign=True, dynamic_mask=True, freeze_mask_after=2)
    assert CG._host_readable(fh) or not CG._host_direct()
    Uh, rh, dh = CG.multiscale_correlate_gpu(fh, g, 16, 16, 16, 8, xp=np, **kw)
    Ud, rd, dd = CG.multiscale_correlate_gpu(torch.from_numpy(fh).cuda(), torch.from_numpy(g).cuda(), 16, 16, 16, 8,
                                             xp=np, **kw)
    assert np.array_equal(Uh, Ud) and np.array_equal(rh, rd) and np.array_equal(dh, dd)


def test_error_paths(api):
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    K_lap = G.build_K_ref_laplacian()
    with pytest.raises(ValueError):
        CG.multiscale_correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, scales=(4, 0), K_ref_laplacian=K_lap,
                                    l0=36.0, disp=False)
    with pytest.raises(ValueError):
        CG.multiscale_correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, scales=(1, 0), g_origin=(1, 0, 0),
                                    K_ref_laplacian=K_lap, l0=36.0, disp=False)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, reg_type='tv', disp=False)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, l0=36.0, disp=False)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, reg_type='equilibrium_gap', l0=36.0,
                         K_ref_laplacian=K_lap, disp=False)


def test_zero_std_raises(api):
    CG, G = api
    f = np.random.default_rng(0).random((9, 9, 9)).astype(np.float32) + 0.1
    g = np.zeros((9, 9, 9), dtype=np.float32)  # no voxel survives g > glt
    with pytest.raises(ZeroDivisionError):
        CG.correlate_gpu(f, g, 2, 2, 2, 4, xp=np, maxiter=2, disp=False)


@pytest.mark.parametrize("h", [1, 2, 3, 4])
@pytest.mark.parametrize("dynamic", [False, True])
def test_small_h_gn_iterations(api, h, dynamic):
    """Two GN iterations at element edges of 1-4 voxels, where the residual /
    b / diag pass runs one thread per element, against the oracle: U, the
    last residual field and the last step (FP32 vs the oracle's FP32 run)."""
    CG, G = api
    from scipy import ndimage
    from oracle import dvc_oracle as O
    n = 6 * h + 1
    rng = np.random.default_rng(40 + h)
    f = ndimage.gaussian_filter(rng.random((n, n, n)), 1.2).astype(np.float32)
    f = (f - f.min()) / (f.max() - f.min()) + np.float32(0.05)
    g = ndimage.shift(f, (0.4, -0.3, 0.25), order=1, mode='nearest').astype(np.float32)
    kw = dict(l0=4.5 * h, maxiter=2, eps=1e-6, dynamic_mask=dynamic, freeze_mask_after=1 if dynamic else None)
    U, res, dU = CG.correlate_gpu(f, g, 6, 6, 6, h, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(), disp=False,
                                  **kw)
    Uo, reso, dUo = O.correlate(f, g, 6, 6, 6, h, K_lap=O.k_ref_laplacian(), **kw)
    assert rms(U, Uo) < 1e-4
    assert rms(dU, dUo) < 1e-4
    assert np.abs(res - reso).max() < 1e-3


def test_eager_pcg_matches_graph(api, monkeypatch):
    """VDVC_PCG=eager launches the graph body's kernels from the host: the
    same kernels in the same order, so the same solve."""
    CG, G = api
    c = load_golden("solve_multiscale.npz")
    kw = dict(scales=(2, 1, 0), K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=20, eps=1e-3,
              disp=False, dynamic_mask=True, freeze_mask_after=4, fft_prealign=True)
    Ug, _, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, **kw)
    monkeypatch.setenv("VDVC_PCG", "eager")
    Ue, _, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, **kw)
    assert np.array_equal(Ue, Ug)
