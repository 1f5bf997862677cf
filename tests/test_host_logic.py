"""Host-side logic of the drop-in API that runs without a GPU: geometry
tables, index helpers, argument validation and the reference's probe
sequence."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import dvc_oracle as O
from voxeldvc_gb300.engine import geometry_dvc as G
from voxeldvc_gb300.engine import kernels_dvc as K


def test_product_geometry_equals_reference_tables():
    g = load_golden("geometry.npz")
    for h in (1, 2, 3, 4, 5, 8):
        N, w = G.build_N_stencil(h)
        assert np.array_equal(N, g[f"N_h{h}"]) and np.array_equal(w, g[f"w_h{h}"])
        for i, a in enumerate(G.VoxelCenterStencil(h)):
            assert np.array_equal(a, g[f"vcs{i}_h{h}"])
    assert np.allclose(G.build_K_ref_laplacian(), g["K_lap"], rtol=0, atol=1e-15)
    for nu in (0.0, 0.3, 0.45):
        assert np.allclose(G.build_K_ref(nu), g[f"K_el_{nu}"], rtol=0, atol=1e-15)
    assert np.allclose(G._shape_grads(0.2, 0.7, 0.4), g["shape_grads"], rtol=0, atol=1e-15)
    assert np.allclose(G._B_matrix(-0.3, 0.5, 0.9)[0], g["B_matrix"], rtol=0, atol=1e-15)
    for (Nx, Ny, Nz) in ((3, 2, 2), (1, 1, 1), (2, 4, 3)):
        tag = f"{Nx}_{Ny}_{Nz}"
        ni = G.build_node_index(Nx, Ny, Nz)
        assert np.array_equal(ni, g[f"node_index_{tag}"])
        assert np.array_equal(G.build_interior_dof_mask(Nx, Ny, Nz), g[f"interior_{tag}"])
        assert np.array_equal(G.element_node_ids(ni, Nx, Ny, Nz), g[f"elem_nodes_{tag}"])


def test_index_helpers_bit_exact():
    g = load_golden("geometry.npz")
    for (Nx, Ny, Nz) in ((3, 2, 2), (1, 1, 1), (2, 4, 3)):
        tag = f"{Nx}_{Ny}_{Nz}"
        e = np.arange(Nx * Ny * Nz, dtype=np.int32)
        d = K.get_elem_dofs(e, Nx, Ny, np)
        assert d.dtype == np.int32 and np.array_equal(d, g[f"elem_dofs_{tag}"])
        for h in (1, 3, 4):
            off = K.get_voxel_offsets(h, Nx, Ny, np)
            assert off.dtype == np.int32 and np.array_equal(off, g[f"vox_offsets_{tag}_h{h}"])
            org = K.get_elem_voxel_origins(e, h, Nx, Ny, np)
            assert np.array_equal(org, g[f"vox_origins_{tag}_h{h}"])
    assert K.auto_chunk_size(729) == 20_000_000 // (729 * 24)


def test_rademacher_probes_match_reference_rng():
    z = K.rademacher_probes(1000, n_probes=4, seed=0)
    rng = np.random.default_rng(0)
    for p in range(4):
        assert np.array_equal(z[p], rng.choice([-1.0, 1.0], size=1000).astype(np.int8))


def test_stencil_validation():
    N, w = G.build_N_stencil(4)
    K._check_stencil(N, w, 4)
    K._check_stencil(N.astype(np.float32), w.astype(np.float32), 4)
    with pytest.raises(ValueError):
        K._check_stencil(N[:-1], w[:-1], 4)
    with pytest.raises(ValueError):
        K._check_stencil(N * 1.5, w, 4)


def test_plane_wave_matches_reference_formula():
    from voxeldvc_gb300.engine.correlate_gpu import _plane_wave
    Nx, Ny, Nz, h = 3, 5, 2, 8
    V = _plane_wave(Nx, Ny, Nz, h, np.float32)
    jj = (np.arange((Nx + 1) * (Ny + 1) * (Nz + 1)) // (Nx + 1)) % (Ny + 1)
    ref = np.zeros(V.size, dtype=np.float32)
    ref[0::3] = np.cos(jj.astype(np.float32) * h / (10 * h) * 2 * np.pi)
    assert np.array_equal(V, ref)


def test_affine_seed_matches_oracle():
    from voxeldvc_gb300.engine.correlate_gpu import _affine_U0
    rng = np.random.default_rng(1)
    A = np.eye(3) + 0.01 * rng.standard_normal((3, 3))
    t, c = rng.standard_normal(3) * 5, np.array([20.0, 16.0, 12.0])
    Nx, Ny, Nz, h, s = 4, 3, 2, 8, 2
    u = _affine_U0(A, t, c, s, h // s, Nx, Ny, Nz)
    nn = np.arange((Nx + 1) * (Ny + 1) * (Nz + 1))
    X = np.stack([nn % (Nx + 1), (nn // (Nx + 1)) % (Ny + 1), nn // ((Nx + 1) * (Ny + 1))], 1) * float(h // s)
    ref = ((X - c / s) @ A.T + c / s + t / s - X).reshape(-1)
    assert np.allclose(u, ref, rtol=0, atol=1e-12)


@pytest.mark.parametrize("scales,origin", [((4, 0), (0, 0, 0)), ((1, 0), (1, 0, 0))])
def test_multiscale_rejects_bad_levels_before_device_work(scales, origin):
    # reference tests/test_dvc_gpu_multiscale.py:88-114: the checks fire before
    # any image reaches the device, so they hold on a machine without a GPU
    from voxeldvc_gb300.engine.correlate_gpu import multiscale_correlate_gpu
    f = np.zeros((17, 17, 17), dtype=np.float32)
    with pytest.raises(ValueError):
        multiscale_correlate_gpu(f, f, 2, 2, 2, 8, xp=np, scales=scales, g_origin=origin,
                                 K_ref_laplacian=G.build_K_ref_laplacian(), l0=36.0, disp=False)


def _owner_walk(h, Nx, Ny, Nz):
    """The voxel walk of the thread-per-element kernels (elem_fast.cu,
    k_elem_rhs, k_elem_sample): element (i,j,k) visits qx,qy,qz in [0, h),
    plus q = h on the mesh's last element of an axis; weight 1/2 per axis on
    the mesh's outer voxel planes; multiplicity 2 per axis on a voxel plane
    shared with the lower neighbour.  Yields (element, (qx,qy,qz), voxel,
    weight, multiplicity)."""
    Nvx, Nvy = Nx * h + 1, Ny * h + 1
    for k in range(Nz):
        for j in range(Ny):
            for i in range(Nx):
                e = i + j * Nx + k * Nx * Ny
                for qz in range(h + (k == Nz - 1)):
                    for qy in range(h + (j == Ny - 1)):
                        for qx in range(h + (i == Nx - 1)):
                            w, mult = 1.0, 1
                            for q, n, idx in ((qx, Nx, i), (qy, Ny, j), (qz, Nz, k)):
                                if (q == 0 and idx == 0) or q == h:
                                    w *= 0.5
                                if q == 0 and idx > 0:
                                    mult *= 2
                            v = (i * h + qx) + (j * h + qy) * Nvx + (k * h + qz) * Nvx * Nvy
                            yield e, (qx, qy, qz), v, w, mult


@pytest.mark.parametrize("h", [1, 2, 3, 4])
def test_owner_walk_equals_reference_quadrature(h):
    """Visiting each voxel once, by its highest-index element, with the walk's
    weights gives the same voxel -> node weights as the reference's
    (element, stencil point) quadrature, which visits shared voxels once per
    element (kernels_dvc.py:452-506, geometry_dvc.py:26-51); the walk's
    multiplicities are the reference's visit counts (correlate_gpu.py:97-157)."""
    Nx, Ny, Nz = 3, 2, 2
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    Nn = (Nx + 1) * (Ny + 1) * (Nz + 1)
    N, w = G.build_N_stencil(h)
    offs = K.get_voxel_offsets(h, Nx, Ny, np)
    nodes = G.element_node_ids(G.build_node_index(Nx, Ny, Nz), Nx, Ny, Nz)
    W_ref = np.zeros((Nvox, Nn))
    visits = np.zeros(Nvox, np.int64)
    for e in range(Nx * Ny * Nz):
        v0 = K.get_elem_voxel_origins(np.array([e], np.int32), h, Nx, Ny, np)[0]
        vox = v0 + offs
        np.add.at(visits, vox, 1)
        for a in range(8):
            np.add.at(W_ref[:, nodes[e, a]], vox, w * N[:, a])
    W_own = np.zeros((Nvox, Nn))
    seen = np.zeros(Nvox, np.int64)
    mults = np.zeros(Nvox, np.int64)
    for e, (qx, qy, qz), v, wt, mult in _owner_walk(h, Nx, Ny, Nz):
        seen[v] += 1
        mults[v] = mult
        fx, fy, fz = qx / h, qy / h, qz / h
        for a in range(8):
            dx, dy, dz = ((a + 1) >> 1) & 1, (a >> 1) & 1, (a >> 2) & 1
            Na = (fx if dx else 1 - fx) * (fy if dy else 1 - fy) * (fz if dz else 1 - fz)
            W_own[v, nodes[e, a]] += wt * Na
    assert np.all(seen == 1)
    assert np.array_equal(mults, visits)
    assert np.allclose(W_own, W_ref, rtol=0, atol=1e-14)


def test_laplacian_block_structure_check():
    """The element-Hessian forms take the vector Laplacian as one 8x8 block
    per displacement component; anything else keeps the matrix-free pass."""
    from voxeldvc_gb300.engine import correlate_gpu as CG
    lap = G.build_K_ref_laplacian()
    assert CG._lap_blockdiag(lap)
    K2 = lap.copy()
    K2[0, 1] = K2[1, 0] = 1e-3
    assert not CG._lap_blockdiag(K2)
    assert not CG._lap_blockdiag(G.build_K_ref(0.3))


def test_seed_mirror_sets():
    """Mirrored network passes only along axes where the pooled input, the
    stride-8 output and the mesh are symmetric under the mirror."""
    from voxeldvc_gb300.learned.seednet import SeedNet

    class _N:
        MIRRORS = SeedNet.MIRRORS

    m = SeedNet.mirrors_for
    assert m(_N(), (513, 513, 513), 8, 64, 64, 64, 2) == (0, 1)
    assert m(_N(), (513, 513, 513), 8, 64, 64, 64, 4) == (0, 1, 2, 3)
    assert m(_N(), (513, 513, 513), 8, 64, 64, 64, 1) == (0,)
    # x not symmetric (mesh short of the volume): only the y mirror is left
    assert m(_N(), (513, 513, 513), 8, 63, 64, 64, 4) == (0, 2)
    # an odd edge that the stride-8 grid does not reach
    assert m(_N(), (515, 513, 513), 2, 257, 256, 256, 2) == (0,)
