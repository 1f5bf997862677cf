"""Per-element output fields and diagnostic masks on the GPU against the
reference's own outputs (tests/golden/cells.npz), against the oracle on a
larger mesh, and on known answers (a uniform strain field)."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import dvc_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W(cuda):
    from voxeldvc_gb300.engine import write_output
    return write_output


@pytest.fixture(scope="module")
def KD(cuda):
    from voxeldvc_gb300.engine import kernels_dvc
    return kernels_dvc


def _close_nan(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(np.isnan(a), np.isnan(b)) and \
        np.allclose(np.nan_to_num(a), np.nan_to_num(b), rtol=tol, atol=tol)


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_cell_fields_match_reference(W, KD, tag):
    c = load_golden("cells.npz")
    Nx, Ny, Nz, h = (int(x) for x in c[f"{tag}_dims"])
    g = lambda k: c[f"{tag}_{k}"]  # noqa: E731
    ps = W.compute_principal_strains_cell(g("U_grid"), h)
    scale = np.abs(g("principal")).max()
    # Jacobi rotations vs LAPACK: eigenvalues agree to a few ulp of ||eps||
    assert ps.shape == g("principal").shape and np.abs(ps - g("principal")).max() <= 1e-13 * scale
    eq = W.compute_equivalent_strain(ps)
    assert np.abs(eq - g("equivalent")).max() <= 1e-13 * scale
    assert np.allclose(W.compute_equivalent_strain(c["ps3"]), c["eq3"], rtol=1e-14, atol=0)
    for key, glt in (("material", float(g("glt"))), ("material70", 70.0)):
        m = W.compute_material_cell_mask(g("ref"), h, Nx, Ny, Nz, glt=glt)
        assert m.dtype == bool and np.array_equal(m, g(key)), key
    assert np.array_equal(W.compute_material_cell_mask_eroded(g("material")), g("material_eroded"))
    assert np.array_equal(W.compute_material_cell_mask_eroded(g("holes")), g("holes_eroded"))
    assert np.array_equal(W.compute_safe_cell_mask(g("unsafe_vox"), h, Nx, Ny, Nz), g("safe"))
    # the (Nvx, Nvy, Nvz) grid form of the unsafe mask gives the same cells
    grid = g("unsafe_vox").reshape(Nx * h + 1, Ny * h + 1, Nz * h + 1, order="F")
    assert np.array_equal(W.compute_safe_cell_mask(grid, h, Nx, Ny, Nz), g("safe"))
    std, zn = W.compute_correlation_quality_cell(g("res"), g("ref"), h, Nx, Ny, Nz)
    assert _close_nan(std, g("residual_std"), 1e-12) and _close_nan(zn, g("zncc"), 1e-12)
    assert _close_nan(W.compute_gn_convergence_cell(g("dU"), g("U0"), Nx, Ny, Nz), g("gn"), 1e-13)
    active = g("res") != 0
    assert np.array_equal(KD.compute_unsafe_voxel_mask(active, h, Nx, Ny, Nz), g("unsafe_vox"))
    assert np.array_equal(KD.compute_unsafe_element_mask(active, h, Nx, Ny, Nz), g("unsafe_elem"))
    assert np.array_equal(KD.compute_unsafe_node_mask(active, h, Nx, Ny, Nz), g("unsafe_node"))
    assert np.array_equal(KD.compute_overlap_lost_element_mask(active, g("mask0"), h, Nx, Ny, Nz), g("overlap_lost"))
    assert np.array_equal(KD.compute_overlap_lost_element_mask(active, g("mask0"), h, Nx, Ny, Nz, frac_threshold=0.2,
                                                               min_material_frac=0.3), g("overlap_lost_t"))
    assert np.array_equal(KD.boundary_element_mask(Nx, Ny, Nz), g("boundary"))


def test_cell_fields_match_oracle_large(W, KD):
    """A 40 x 36 x 30 mesh at h = 2 (43,200 elements) against the oracle."""
    rng = np.random.default_rng(7)
    Nx, Ny, Nz, h = 40, 36, 30, 2
    shape = (Nx * h + 1, Ny * h + 1, Nz * h + 1)
    Nn = (Nx + 1) * (Ny + 1) * (Nz + 1)
    U = rng.standard_normal(3 * Nn)
    U_grid = np.stack([U[c::3].reshape(Nx + 1, Ny + 1, Nz + 1, order="F") for c in range(3)], axis=-1)
    ps = W.compute_principal_strains_cell(U_grid, h)
    ps_o = O.principal_strains_cell(U_grid, h)
    assert np.abs(ps - ps_o).max() <= 1e-13 * np.abs(ps_o).max()
    ref = rng.random(shape).astype(np.float32) * 100
    ref[:20, :20] = 0
    res = np.where(rng.random(shape) < 0.9, rng.standard_normal(shape), 0.0).reshape(-1, order="F")
    std, zn = W.compute_correlation_quality_cell(res, ref, h, Nx, Ny, Nz)
    std_o, zn_o = O.correlation_quality_cell(res, ref, h, Nx, Ny, Nz)
    assert _close_nan(std, std_o, 1e-12) and _close_nan(zn, zn_o, 1e-12)
    assert np.array_equal(W.compute_material_cell_mask(ref, h, Nx, Ny, Nz, glt=40.0),
                          O.material_cell_mask(ref, h, Nx, Ny, Nz, glt=40.0))
    active = res != 0
    active[: len(active) // 3] = True
    mask0 = ref.reshape(-1, order="F") > 10
    m = O.unsafe_masks(active, h, Nx, Ny, Nz, mask0)
    assert np.array_equal(KD.compute_unsafe_voxel_mask(active, h, Nx, Ny, Nz), m["unsafe_vox"])
    assert np.array_equal(KD.compute_overlap_lost_element_mask(active, mask0, h, Nx, Ny, Nz), m["overlap_lost"])
    dU = rng.standard_normal(3 * Nn)
    assert _close_nan(W.compute_gn_convergence_cell(dU, U, Nx, Ny, Nz), O.gn_convergence_cell(dU, U, Nx, Ny, Nz),
                      1e-13)


def test_uniform_strain_known_answer(W):
    """U = G x on the nodes: every cell carries the eigenvalues of sym(G)."""
    Nx, Ny, Nz, h = 6, 5, 4, 3
    G = np.array([[0.01, 0.002, -0.003], [0.004, -0.02, 0.001], [0.0, 0.005, 0.007]])
    x = np.stack(np.meshgrid(*(np.arange(n + 1) * h for n in (Nx, Ny, Nz)), indexing="ij"), axis=-1).astype(float)
    U_grid = x @ G.T
    ps = W.compute_principal_strains_cell(U_grid, h)
    ev = np.sort(np.linalg.eigvalsh(0.5 * (G + G.T)))[::-1]
    assert np.abs(ps - ev).max() < 1e-15
    eq = W.compute_equivalent_strain(ps)
    assert np.allclose(eq, np.sqrt(2) / 3 * np.sqrt(((ev - np.roll(ev, -1)) ** 2).sum()), rtol=1e-13)
