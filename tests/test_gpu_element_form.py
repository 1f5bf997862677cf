"""Element-Hessian form of the float32 solve (hessian='element'): the element
Hessians are formed from the float32 gradient once per GN iteration and the
PCG applies H from them -- the matrix-free pass's float32 products summed in
another order.  Held to the same parity bar as the matrix-free solve
(1e-3 voxel RMS against the reference's golden solves), to the matrix-free
solve itself, and to the oracle at element edges 1-4."""
import numpy as np
import pytest

from conftest import OPS_CASES, load_golden

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-3  # voxel RMS of nodal displacements, FP32 solve vs reference
SAME_TOL = 1e-4  # the two float32 Hessian forms against each other


def rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


@pytest.fixture(scope="module")
def api(cuda):
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    return CG, G


def _cases(G):
    lap = G.build_K_ref_laplacian()
    return {
        "sinusoid": ("solve_sinusoid.npz", "U", False,
                     dict(dims=(2, 2, 2), h=8, K_ref_laplacian=lap, l0=4.5 * 8, maxiter=20, eps=1e-3)),
        "dynamic": ("solve_dynamic.npz", "U", False,
                    dict(dims=(4, 4, 4), h=4, K_ref_laplacian=lap, l0=8.0, maxiter=12, eps=1e-4, dynamic_mask=True,
                         freeze_mask_after=2, glt=0.0)),
        "eqgap": ("solve_eqgap.npz", "U", False,
                  dict(dims=(3, 3, 3), h=4, K_ref_laplacian=lap, K_ref_elastic=G.build_K_ref(0.3),
                       reg_type='equilibrium_gap', reg_exponent=4, l0=18.0, maxiter=10, eps=1e-4, dynamic_mask=True,
                       freeze_mask_after=4)),
        "multiscale": ("solve_multiscale.npz", "U", True,
                       dict(dims=(4, 3, 2), h=8, scales=(2, 1, 0), K_ref_laplacian=lap, l0=36.0, maxiter=20,
                            eps=1e-3, dynamic_mask=True, freeze_mask_after=4, fft_prealign=True)),
    }


def _solve(CG, c, multiscale, kw, **extra):
    kw = dict(kw)
    Nx, Ny, Nz = kw.pop("dims")
    h = kw.pop("h")
    stats = []
    fn = CG.multiscale_correlate_gpu if multiscale else CG.correlate_gpu
    U, res, dU = fn(c["f"], c["g"], Nx, Ny, Nz, h, xp=np, disp=False, stats=stats, **kw, **extra)
    return U, res, stats


@pytest.mark.parametrize("name", ["sinusoid", "dynamic", "eqgap", "multiscale"])
def test_element_form_against_golden_and_matrix_free(api, name):
    CG, G = api
    golden, key, ms, kw = _cases(G)[name]
    c = load_golden(golden)
    Ue, rese, se = _solve(CG, c, ms, kw, hessian="element")
    Um, resm, sm = _solve(CG, c, ms, kw, hessian="matrix_free")
    assert all(s["hessian"] == "element" for s in se)
    assert all(s["hessian"] == "matrix_free" for s in sm)
    assert rms(Ue, c[key]) < RMS_TOL
    assert rms(Ue, Um) < SAME_TOL
    # the same GN path: iteration counts per level, PCG counts within one
    # (within 5 % on the equilibrium-gap system, whose PCG runs hundreds of
    # iterations on a stiff operator and moves with the last bits of alpha)
    assert [s["gn_iters"] for s in se] == [s["gn_iters"] for s in sm]
    for a, b in zip(se, sm):
        assert all(abs(x - y) <= max(1, 0.05 * y) for x, y in zip(a["pcg_iters"], b["pcg_iters"])), \
            (a["pcg_iters"], b["pcg_iters"])


@pytest.mark.parametrize("h", [1, 2, 3, 4])
def test_element_form_small_h_against_oracle(api, h):
    """Two GN iterations at element edges 1-4 (dynamic mask, frozen after
    one) against the oracle's float32 run."""
    CG, G = api
    from scipy import ndimage
    from oracle import dvc_oracle as O
    n = 6 * h + 1
    rng = np.random.default_rng(40 + h)
    f = ndimage.gaussian_filter(rng.random((n, n, n)), 1.2).astype(np.float32)
    f = (f - f.min()) / (f.max() - f.min()) + np.float32(0.05)
    g = ndimage.shift(f, (0.4, -0.3, 0.25), order=1, mode='nearest').astype(np.float32)
    kw = dict(l0=4.5 * h, maxiter=2, eps=1e-6, dynamic_mask=True, freeze_mask_after=1)
    U, res, dU = CG.correlate_gpu(f, g, 6, 6, 6, h, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(), disp=False,
                                  hessian="element", **kw)
    Uo, reso, dUo = O.correlate(f, g, 6, 6, 6, h, K_lap=O.k_ref_laplacian(), **kw)
    assert rms(U, Uo) < 1e-4
    assert rms(dU, dUo) < 1e-4
    assert np.abs(res - reso).max() < 1e-3


def test_element_form_level_policy(api):
    # 'auto' takes element Hessians at h >= 4 of a float32 plain solve only
    CG, G = api
    c = load_golden("solve_multiscale.npz")
    kw = dict(scales=(2, 1, 0), K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=3, disp=False,
              fft_prealign=False)
    stats = []
    CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, stats=stats, **kw)
    assert [(s["h"], s["hessian"]) for s in stats] == [(2, "matrix_free"), (4, "element"), (8, "element")]
    stats = []
    CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, stats=stats, dtype=np.float64, **kw)
    assert all(s["hessian"] == "matrix_free" for s in stats)


def test_element_form_argument_errors(api):
    CG, G = api
    c = load_golden("solve_sinusoid.npz")
    lap = G.build_K_ref_laplacian()
    kw = dict(l0=36.0, maxiter=2, disp=False)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, K_ref_laplacian=lap, hessian="dense", **kw)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, K_ref_laplacian=lap, hessian="element",
                         dtype=np.float64, **kw)
    # a Laplacian that couples displacement components: no element form
    K = lap.copy()
    K[0, 1] = K[1, 0] = 1e-3
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, K_ref_laplacian=K, hessian="element", **kw)
    stats = []
    CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, K_ref_laplacian=K, stats=stats, **kw)
    assert stats[-1]["hessian"] == "matrix_free"


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("case", OPS_CASES)
def test_element_hessians_operator(api, case):
    """Form once, apply twice: against the reference's FP64 operator, the
    matrix-free float32 pass and (BF16 form) the oracle on the same BF16
    gradient."""
    from voxeldvc_gb300.engine import kernels_dvc as K
    from oracle import dvc_oracle as O
    CG, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    N, w = G.build_N_stencil(h)
    eh = K.ElementHessians(c["grad"], c["mask"], h, Nx, Ny, Nz)
    Hv = eh.matvec(c["v"], np)
    assert Hv.dtype == np.float32
    assert _rel(Hv, c["out_matvec_H_f64"]) < 2e-6
    mf = K.matvec_H(c["v"].astype(np.float32), c["grad"].astype(np.float32), c["mask"], N, w, h, Nx, Ny, Nz, np)
    assert _rel(Hv, mf) < 2e-6
    v2 = np.random.default_rng(3).standard_normal(c["v"].shape)
    ref2 = O.matvec_h(v2.astype(np.float32).astype(np.float64), c["grad"].astype(np.float32).astype(np.float64),
                      c["mask"], h, Nx, Ny, Nz)
    assert _rel(eh.matvec(v2, np), ref2) < 2e-6
    eb = K.ElementHessians(c["grad"], c["mask"], h, Nx, Ny, Nz, bf16=True)
    import torch
    g16 = torch.from_numpy(np.ascontiguousarray(c["grad"], np.float32)).to(torch.bfloat16).float().numpy()
    ref16 = O.matvec_h(c["v"].astype(np.float32).astype(np.float64), g16.astype(np.float64), c["mask"], h, Nx, Ny,
                       Nz)
    assert _rel(eb.matvec(c["v"], np), ref16) < 2e-6
