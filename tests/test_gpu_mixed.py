"""Precision form of the Hessian (BF16 gradient, element Hessians with FP32
accumulation) against the CPU oracle on the same BF16-rounded gradient, and
against the reference's FP64 golden within the BF16 rounding budget."""
import numpy as np
import pytest

from conftest import OPS_CASES, load_golden
from oracle import dvc_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def bf16_round(x):
    """float32 -> nearest BF16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def test_bf16_round_helper():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 0.0], np.float32)
    # ties go to even: 1+2^-8 -> 1, 1+3*2^-8 -> 1+2^-6
    assert np.array_equal(bf16_round(x), np.array([1.0, 1.0, 1.0 + 2.0 ** -6, -2.5, 0.0], np.float32))


@pytest.fixture(scope="module")
def api(cuda):
    from voxeldvc_gb300.engine import kernels_dvc as K, geometry_dvc as G
    return K, G


@pytest.mark.parametrize("case", OPS_CASES)
def test_mixed_matvec(api, case):
    K, G = api
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    N, w = G.build_N_stencil(h)
    Hv = K.matvec_H_mixed(c["v"], c["grad"], c["mask"], N, w, h, Nx, Ny, Nz, np)
    assert Hv.dtype == np.float32
    # same BF16 gradient, FP64 oracle: only FP32 accumulation differs
    g16 = bf16_round(c["grad"]).astype(np.float64)
    ref16 = O.matvec_h(c["v"].astype(np.float64), g16, c["mask"], h, Nx, Ny, Nz)
    assert rel(Hv, ref16) < 2e-6
    # against the reference operator: BF16 rounding of the gradient (<= 2^-8 relative)
    assert rel(Hv, c["out_matvec_H_f64"]) < 1e-2


@pytest.mark.parametrize("h,dims", [(8, (5, 3, 4)), (6, (23, 2, 3)), (8, (1, 1, 1)), (8, (4, 3, 2))])
def test_tensor_core_formation(api, h, dims, monkeypatch):
    """tcgen05 formation (VDVC_EH_FORM=tc) against the FP16-operand oracle
    (ragged 21-element tiles, rows crossing mesh rows) and against the
    CUDA-core formation."""
    K, G = api
    monkeypatch.setenv("VDVC_EH_FORM", "tc")
    rng = np.random.default_rng(h + dims[0])
    Nx, Ny, Nz = dims
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    grad = (rng.standard_normal((Nvox, 3)) * 300.0).astype(np.float32)  # an intensity scale far from 1
    mask = rng.random(Nvox) < 0.9
    v = rng.standard_normal(Ndof).astype(np.float32)
    N, w = G.build_N_stencil(h)
    Hv = K.matvec_H_mixed(v, grad, mask, N, w, h, Nx, Ny, Nz, np)
    T = O.eh_f16_elements(bf16_round(grad), mask, h, Nx, Ny, Nz)
    assert rel(Hv, O.eh_matvec(T, v.astype(np.float64), Nx, Ny, Nz)) < 1e-5
    monkeypatch.setenv("VDVC_EH_FORM", "cuda")
    Hc = K.matvec_H_mixed(v, grad, mask, N, w, h, Nx, Ny, Nz, np)
    ref16 = O.matvec_h(v.astype(np.float64), bf16_round(grad).astype(np.float64), mask, h, Nx, Ny, Nz)
    assert rel(Hc, ref16) < 2e-6
    assert rel(Hv, Hc) < 5e-4


def test_mixed_matvec_random_mesh(api):
    """A mesh with several strips per row and ragged last strip (h = 4, Nx = 37)."""
    K, G = api
    rng = np.random.default_rng(5)
    h, Nx, Ny, Nz = 4, 37, 3, 2
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    grad = rng.standard_normal((Nvox, 3)).astype(np.float32)
    mask = rng.random(Nvox) < 0.85
    v = rng.standard_normal(Ndof).astype(np.float32)
    N, w = G.build_N_stencil(h)
    Hv = K.matvec_H_mixed(v, grad, mask, N, w, h, Nx, Ny, Nz, np)
    ref16 = O.matvec_h(v.astype(np.float64), bf16_round(grad).astype(np.float64), mask, h, Nx, Ny, Nz)
    assert rel(Hv, ref16) < 2e-6


# ---- Gauss-Newton solves in the precision form ------------------------------
# Only H (the Newton matrix) is approximated; b = J^T r - lambda R U keeps the
# FP32 gradient, so the GN fixed point is the plain solve's.

def rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


MIXED_REL_TOL = 2e-3  # RMS error / RMS of the reference's FP32 golden solve, GN stopped at dU/U < eps


def rel_rms(U, ref):
    return rms(U, ref) / rms(ref, np.zeros_like(ref))


@pytest.fixture(scope="module")
def solve_api(cuda):
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    return CG, G


def test_mixed_solve_sinusoid(solve_api):
    CG, G = solve_api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False)
    stats = []
    U, res, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, precision="mixed", stats=stats, **kw)
    assert stats[0]["precision"] == "mixed"
    assert rel_rms(U, c["U"]) < MIXED_REL_TOL


@pytest.mark.parametrize("form", ["cuda", "tc"])
def test_mixed_solve_formations(solve_api, form, monkeypatch):
    """The precision-form solve with either element-Hessian formation (CUDA
    cores, or tcgen05 with FP16 operands) reaches the plain solve's result."""
    CG, G = solve_api
    monkeypatch.setenv("VDVC_EH_FORM", form)
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False)
    U, _, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, precision="mixed", **kw)
    assert rel_rms(U, c["U"]) < MIXED_REL_TOL


def test_mixed_same_fixed_point(solve_api):
    CG, G = solve_api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=4.5 * 8, maxiter=60, eps=1e-6, pcg_tol=1e-8,
              disp=False)
    Up, _, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, **kw)
    Um, _, _ = CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, precision="mixed", **kw)
    # both stop on the FP32 residual's noise floor (~1e-4 voxel)
    assert rms(Up, Um) < 3e-4


def test_mixed_dynamic_mask_freeze(solve_api):
    # H follows the b mask until the freeze, then is formed no more
    CG, G = solve_api
    c = load_golden("solve_dynamic.npz")
    U, _, _ = CG.correlate_gpu(c["f"], c["g"], 4, 4, 4, 4, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(),
                               l0=8.0, maxiter=12, eps=1e-4, disp=False, dynamic_mask=True, freeze_mask_after=2,
                               glt=0.0, precision="mixed", mixed_min_h=1)
    assert rel_rms(U, c["U"]) < MIXED_REL_TOL


def test_mixed_equilibrium_gap(solve_api):
    CG, G = solve_api
    c = load_golden("solve_eqgap.npz")
    U, _, _ = CG.correlate_gpu(c["f"], c["g"], 3, 3, 3, 4, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(),
                               K_ref_elastic=G.build_K_ref(0.3), reg_type='equilibrium_gap', reg_exponent=4,
                               l0=18.0, maxiter=10, eps=1e-4, disp=False, dynamic_mask=True, freeze_mask_after=4,
                               precision="mixed", mixed_min_h=1)
    assert rel_rms(U, c["U"]) < MIXED_REL_TOL


def test_mixed_multiscale(solve_api):
    CG, G = solve_api
    c = load_golden("solve_multiscale.npz")
    U, _, _ = CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, scales=(2, 1, 0),
                                          K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=20,
                                          eps=1e-3, disp=False, dynamic_mask=True, freeze_mask_after=4,
                                          fft_prealign=True, precision="mixed", mixed_min_h=1)
    assert rel_rms(U, c["U"]) < MIXED_REL_TOL


def test_mixed_level_policy(solve_api):
    # element Hessians at h >= mixed_min_h only; the coarser levels stay plain
    CG, G = solve_api
    c = load_golden("solve_multiscale.npz")
    stats = []
    CG.multiscale_correlate_gpu(c["f"], c["g"], 4, 3, 2, 8, xp=np, scales=(2, 1, 0),
                                K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=3, disp=False,
                                fft_prealign=False, precision="mixed", stats=stats)
    assert [(s["h"], s["precision"]) for s in stats] == [(2, "plain"), (4, "mixed"), (8, "mixed")]


def test_mixed_argument_errors(solve_api):
    CG, G = solve_api
    c = load_golden("solve_sinusoid.npz")
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, maxiter=2, disp=False)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, precision="mixed", dtype=np.float64, **kw)
    with pytest.raises(ValueError):
        CG.correlate_gpu(c["f"], c["g"], 2, 2, 2, 8, xp=np, precision="half", **kw)
