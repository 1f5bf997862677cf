"""Size-independent properties of the operators at the benchmark size
(513^3 voxels, h = 8, 64^3 elements, 823,875 dof), where the CPU oracle is
too slow to compare entry by entry: symmetry, linearity and semi-definiteness
of H, FP32 against the FP64 mode, the precision form within its BF16
budget, the Jacobi diagonal against unit-vector probes, the Laplacian's
null space, and the identity sampling at u = 0."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big(cuda):
    import torch
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G, kernels_dvc as K
    wl = synth.WORKLOADS["necking_512"]()
    Nx, Ny, Nz = wl.mesh
    f_pix, g_pix = wl.make()
    f_vox, shape = CG.pix_to_vox(f_pix, np.float32)
    grad, mask0 = CG._grad_vox(f_vox, shape, np.float32, 0.0)
    N, w = G.build_N_stencil(wl.h)
    gen = torch.Generator("cuda").manual_seed(3)
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    v = torch.randn(Ndof, device="cuda", generator=gen)
    u = torch.randn(Ndof, device="cuda", generator=gen)

    def H(x, dtype=torch.float32):
        return K.matvec_H(x.to(dtype), grad.view(-1, 3).to(dtype), mask0, N, w, wl.h, Nx, Ny, Nz, torch)

    return dict(torch=torch, K=K, G=G, CG=CG, wl=wl, mesh=(Nx, Ny, Nz), H=H, v=v, u=u, grad=grad, mask0=mask0,
                N=N, w=w, g_pix=g_pix, f_pix=f_pix, Ndof=Ndof)


def _dot(a, b):
    return float((a.double() * b.double()).sum())


def test_hessian_symmetric_linear_semidefinite(big):
    H, v, u = big["H"], big["v"], big["u"]
    Hv, Hu = H(v), H(u)
    scale = float(Hv.double().norm() * u.double().norm())
    assert abs(_dot(u, Hv) - _dot(v, Hu)) < 1e-5 * scale
    lin = H(2.0 * v + 3.0 * u)
    ref = 2.0 * Hv.double() + 3.0 * Hu.double()
    assert float((lin.double() - ref).norm() / ref.norm()) < 1e-5
    assert _dot(v, Hv) > 0 and _dot(u, Hu) > 0


def test_hessian_fp32_against_fp64_mode(big):
    torch = big["torch"]
    H, v = big["H"], big["v"]
    h32 = H(v).double()
    h64 = H(v.double(), torch.float64)
    assert float((h32 - h64).norm() / h64.norm()) < 2e-6


def test_precision_form_within_bf16_budget(big):
    torch, K = big["torch"], big["K"]
    Nx, Ny, Nz = big["mesh"]
    hm = K.matvec_H_mixed(big["v"], big["grad"].view(-1, 3), big["mask0"], big["N"], big["w"], big["wl"].h,
                          Nx, Ny, Nz, torch).double()
    h64 = big["H"](big["v"].double(), torch.float64)
    assert float((hm - h64).norm() / h64.norm()) < 1e-2


def test_jacobi_diagonal_matches_unit_probes(big):
    torch, K = big["torch"], big["K"]
    Nx, Ny, Nz = big["mesh"]
    d = K.build_diagonal_H(big["grad"].view(-1, 3), big["mask0"], big["N"], big["w"], big["wl"].h, Nx, Ny, Nz,
                           big["Ndof"], torch)
    rng = np.random.default_rng(0)
    for i in rng.integers(0, big["Ndof"], 6):
        e = torch.zeros(big["Ndof"], device="cuda")
        e[int(i)] = 1.0
        hii = float(big["H"](e)[int(i)])
        assert abs(hii - float(d[int(i)])) <= 1e-5 * max(abs(hii), 1e-30)


def test_laplacian_null_space_and_symmetry(big):
    torch, K, G = big["torch"], big["K"], big["G"]
    Nx, Ny, Nz = big["mesh"]
    Kl = G.build_K_ref_laplacian()
    ones = torch.ones(big["Ndof"], device="cuda", dtype=torch.float64)
    r = K.matvec_K_ref(ones, Kl, float(big["wl"].h), Nx, Ny, Nz, torch)
    assert float(r.abs().max()) < 1e-9
    v, u = big["v"].double(), big["u"].double()
    Kv = K.matvec_K_ref(v, Kl, float(big["wl"].h), Nx, Ny, Nz, torch)
    Ku = K.matvec_K_ref(u, Kl, float(big["wl"].h), Nx, Ny, Nz, torch)
    assert abs(_dot(u, Kv) - _dot(v, Ku)) < 1e-10 * float(Kv.norm() * u.norm())


def test_identity_sampling_at_zero_displacement(big):
    torch, CG = big["torch"], big["CG"]
    Nx, Ny, Nz = big["mesh"]
    h = big["wl"].h
    U0 = torch.zeros(big["Ndof"], device="cuda")
    gv, mk = CG.sample_deformed_field(U0, big["g_pix"], big["N"], h, Nx, Ny, Nz, torch)
    g_vox, _ = CG.pix_to_vox(big["g_pix"], np.float32)
    assert torch.equal(gv, g_vox)
    assert torch.equal(mk, g_vox > 0)
