"""The CPU oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py).  This pins the oracle before it is used to
check the CUDA path."""
import numpy as np
import pytest

from conftest import OPS_CASES, load_golden
from oracle import dvc_oracle as O


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_geometry_tables_bit_exact():
    g = load_golden("geometry.npz")
    for h in (1, 2, 3, 4, 5, 8):
        N, w = O.n_stencil(h)
        assert np.array_equal(N, g[f"N_h{h}"])
        assert np.array_equal(w, g[f"w_h{h}"])
        for i, a in enumerate(O.voxel_center_stencil(h)):
            assert np.array_equal(a, g[f"vcs{i}_h{h}"])
    assert np.allclose(O.k_ref_laplacian(), g["K_lap"], rtol=0, atol=1e-15)
    for nu in (0.0, 0.3, 0.45):
        assert np.allclose(O.k_ref_elastic(nu), g[f"K_el_{nu}"], rtol=0, atol=1e-15)
    for (Nx, Ny, Nz) in ((3, 2, 2), (1, 1, 1), (2, 4, 3)):
        tag = f"{Nx}_{Ny}_{Nz}"
        assert np.array_equal(O.node_index(Nx, Ny, Nz), g[f"node_index_{tag}"])
        assert np.array_equal(O.interior_dof_mask(Nx, Ny, Nz), g[f"interior_{tag}"])
        assert np.array_equal(O.element_nodes(Nx, Ny, Nz), g[f"elem_nodes_{tag}"])
        e = np.arange(Nx * Ny * Nz, dtype=np.int32)
        d = O.elem_dofs(e, Nx, Ny)
        assert d.dtype == np.int32 and np.array_equal(d, g[f"elem_dofs_{tag}"])
        for h in (1, 3, 4):
            assert np.array_equal(O.voxel_offsets(h, Nx, Ny), g[f"vox_offsets_{tag}_h{h}"])
            assert np.array_equal(O.elem_voxel_origins(e, h, Nx, Ny), g[f"vox_origins_{tag}_h{h}"])


@pytest.mark.parametrize("case", OPS_CASES)
def test_operators_match_reference(case):
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    Ndof = c["v"].size
    K_lap, K_el = O.k_ref_laplacian(), O.k_ref_elastic(0.3)
    assert rel(O.matvec_h(c["v"], c["grad"], c["mask"], h, Nx, Ny, Nz), c["out_matvec_H"]) < 1e-6
    assert rel(O.matvec_h(c["v"].astype(np.float64), c["grad"].astype(np.float64), c["mask"], h, Nx, Ny, Nz),
               c["out_matvec_H_f64"]) < 1e-13
    assert rel(O.diag_h(c["grad"], c["mask"], h, Nx, Ny, Nz, Ndof), c["out_diag_H"]) < 1e-6
    assert rel(O.compute_b(c["res"], c["mask"], c["grad"], h, Nx, Ny, Nz, Ndof), c["out_compute_b"]) < 1e-6
    assert rel(O.matvec_k_ref(c["v"], K_lap, h, Nx, Ny, Nz), c["out_matvec_K_lap"]) < 1e-6
    assert rel(O.diag_k_ref(K_lap, h, Nx, Ny, Nz, Ndof), c["out_diag_K_lap"]) < 1e-14
    assert rel(O.matvec_eqgap(c["v"].astype(np.float64), K_el, c["interior"], h, Nx, Ny, Nz),
               c["out_matvec_eqgap"]) < 1e-13
    assert rel(O.diag_eqgap(K_el, c["interior"], h, Nx, Ny, Nz, Ndof), c["out_diag_eqgap"]) < 1e-13
    assert np.allclose(O.masked_mean_std(c["res"], c["mask"], h, Nx, Ny, Nz), c["out_stats"], rtol=1e-12)
    assert np.array_equal(O.interp_field(c["U"], h, Nx, Ny, Nz), c["out_interp"])
    gv, gm = O.sample_deformed(c["U"], c["g_pix"], h, Nx, Ny, Nz, tuple(int(o) for o in c["g_origin"]), c["mask"])
    assert np.array_equal(gm, c["out_sample_mask"])
    assert np.array_equal(gv, c["out_sample_g"])
    f_vox, grad = O.image_grad_and_values(c["f_pix"])
    assert np.array_equal(f_vox, c["out_f_vox"]) and np.array_equal(grad, c["out_grad_f"])
    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    assert np.array_equal(O.erode(f_vox > 0, Nvx, Nvy, Nvz), c["out_eroded"])


@pytest.mark.parametrize("case", ["A", "B", "C"])
def test_pcg_matches_reference(case):
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    Ndof = c["v"].size
    K_lap = O.k_ref_laplacian()
    ll = float(c["out_pcg_ll"])
    dg = O.diag_h(c["grad"], c["mask"], h, Nx, Ny, Nz, Ndof) + ll * O.diag_k_ref(K_lap, h, Nx, Ny, Nz, Ndof)
    Minv = 1.0 / (dg + 1e-5 * float(dg.min()))

    def A(x):
        return O.matvec_h(x, c["grad"], c["mask"], h, Nx, Ny, Nz) + ll * O.matvec_k_ref(x, K_lap, h, Nx, Ny, Nz)

    x = O.pcg(A, c["b_pcg"], Minv, max_iter=300, tol=1e-7)
    assert rel(x, c["out_pcg_x"]) < 1e-6


def test_affine_matches_reference():
    c = load_golden("affine.npz")
    f_d, g_d = c["f"][::2, ::2, ::2], c["g"][::2, ::2, ::2]
    for p, cost in zip(c["ps"], c["costs"]):
        assert abs(O.affine_cost(f_d, g_d, p) - cost) < 1e-6
    A, t = O.affine_refine(c["f"], c["g"], c["A_pre"], c["t_pre"], c["c_pre"], sigmas=(2.0, 0.0), max_iter=20)
    assert np.abs(A - c["A_ref"]).max() < 1e-6
    assert np.abs(t - c["t_ref"]).max() < 1e-5


def test_fft_shift_matches_reference():
    c = load_golden("fft.npz")
    assert np.array_equal(O.fft_rigid_shift(c["f1"], c["g1"]), c["d1"])
    assert np.array_equal(O.fft_rigid_shift(c["f2"], c["g2"]), c["d2"])
    assert np.array_equal(c["d1"], [3.0, -2.0, 1.0])


def test_correlate_matches_reference():
    c = load_golden("solve_sinusoid.npz")
    K_lap = O.k_ref_laplacian()
    U, res, dU = O.correlate(c["f"], c["g"], 2, 2, 2, 8, K_lap=K_lap, l0=4.5 * 8, maxiter=20, eps=1e-3)
    assert np.abs(U - c["U"]).max() < 1e-4
    assert np.abs(res - c["res"]).max() < 1e-4
    Um, _, _ = O.multiscale(c["f"], c["g"], 2, 2, 2, 8, scales=(2, 1, 0), K_lap=K_lap, l0=4.5 * 8, maxiter=30,
                            eps=1e-3)
    assert np.abs(Um - c["U_ms"]).max() < 1e-5


def test_correlate_dynamic_and_eqgap_match_reference():
    K_lap, K_el = O.k_ref_laplacian(), O.k_ref_elastic(0.3)
    c = load_golden("solve_dynamic.npz")
    U, res, _ = O.correlate(c["f"], c["g"], 4, 4, 4, 4, K_lap=K_lap, l0=8.0, maxiter=12, eps=1e-4,
                            dynamic_mask=True, freeze_mask_after=2)
    assert np.abs(U - c["U"]).max() < 1e-4
    c = load_golden("solve_eqgap.npz")
    U, res, _ = O.correlate(c["f"], c["g"], 3, 3, 3, 4, K_lap=K_lap, K_el=K_el, reg_type='equilibrium_gap',
                            reg_exponent=4, l0=18.0, maxiter=10, eps=1e-4, dynamic_mask=True, freeze_mask_after=4)
    assert np.abs(U - c["U"]).max() < 1e-4
    c = load_golden("solve_multiscale.npz")
    U, res, _ = O.multiscale(c["f"], c["g"], 4, 3, 2, 8, scales=(2, 1, 0), K_lap=K_lap, l0=36.0, maxiter=20,
                             eps=1e-3, dynamic_mask=True, freeze_mask_after=4, fft_prealign=True)
    assert np.abs(U - c["U"]).max() < 1e-4


def test_post_stages_oracle():
    """push_field_forward / compute_zncc restatements against the reference's
    own outputs (tests/golden/post.npz)."""
    c = load_golden("post.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    for name in ("f32", "f64"):
        for key, kw in (("o1_nearest", dict(order=1, mode="nearest")),
                        ("o1_constant", dict(order=1, mode="constant", cval=-1.0)),
                        ("o0_constant", dict(order=0, mode="constant", cval=7.0))):
            out = O.push_field_forward(c[name], c["U"], Nx, Ny, Nz, h, **kw)
            ref = c[f"{name}_{key}"]
            assert out.dtype == ref.dtype and np.array_equal(out, ref), (name, key)
    for key, kw in (("o0_nearest", dict(order=0, mode="nearest")), ("o0_constant", dict(order=0, mode="constant", cval=5))):
        assert np.array_equal(O.push_field_forward(c["lab"], c["U"], Nx, Ny, Nz, h, **kw), c[f"lab_{key}"])
    assert np.array_equal(O.push_field_forward(c["u16"], c["U"], Nx, Ny, Nz, h), c["u16_o1_nearest"])
    assert np.array_equal(O.push_field_forward(c["lab"] * 40, c["U"], Nx, Ny, Nz, h), c["lab_o1_nearest"])
    assert O.zncc(c["zf"], c["zg"], c["zm"]) == pytest.approx(float(c["zncc"]), abs=1e-15)
    assert np.isnan(O.zncc(c["zf"], c["zg"], np.zeros_like(c["zm"])))


def test_preprocess_oracle():
    """bin_volume / compute_crop restatements against the reference's own
    outputs (tests/golden/prep.npz); the warp restatement against known
    answers (the reference's warp needs CuPy, absent here)."""
    c = load_golden("prep.npz")
    assert np.array_equal(O.bin_volume(c["vol8"], 2), c["bin8_2"])
    assert np.array_equal(O.bin_volume(c["vol8"], 4), c["bin8_4"])
    assert np.array_equal(O.bin_volume(c["volf"], 3), c["binf_3"])
    lo, hi = O.compute_crop(c["f"], c["g"], 4)
    assert np.array_equal(lo, c["lo"]) and np.array_equal(hi, c["hi"])
    lo, hi = O.compute_crop(c["f"], c["g"], 8, glt=0.3)
    assert np.array_equal(lo, c["lo2"]) and np.array_equal(hi, c["hi2"])
    g = c["f"]
    assert np.array_equal(O.warp_onto_ref_grid(np.eye(3), np.zeros(3), np.full(3, 7.0), g.shape, g), g)
    w = O.warp_onto_ref_grid(np.eye(3), np.array([2.0, 0.0, -1.0]), np.zeros(3), g.shape, g)
    assert np.array_equal(w[:-2, :, 1:], g[2:, :, :-1]) and np.all(w[-2:] == 0) and np.all(w[:, :, 0] == 0)


def _close_nan(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(np.isnan(a), np.isnan(b)) and \
        np.allclose(np.nan_to_num(a), np.nan_to_num(b), rtol=tol, atol=tol)


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_cell_fields_oracle(tag):
    """Per-element strain / quality fields and the diagnostic masks against
    the reference's own outputs (tests/golden/cells.npz)."""
    c = load_golden("cells.npz")
    Nx, Ny, Nz, h = (int(x) for x in c[f"{tag}_dims"])
    g = lambda k: c[f"{tag}_{k}"]  # noqa: E731
    ps = O.principal_strains_cell(g("U_grid"), h)
    assert _close_nan(ps, g("principal"), 1e-13)
    assert _close_nan(O.equivalent_strain(ps), g("equivalent"), 1e-13)
    assert np.array_equal(O.material_cell_mask(g("ref"), h, Nx, Ny, Nz, glt=float(g("glt"))), g("material"))
    assert np.array_equal(O.material_cell_mask(g("ref"), h, Nx, Ny, Nz, glt=70.0), g("material70"))
    assert np.array_equal(O.material_cell_mask_eroded(g("material")), g("material_eroded"))
    assert np.array_equal(O.material_cell_mask_eroded(g("holes")), g("holes_eroded"))
    assert np.array_equal(O.safe_cell_mask(g("unsafe_vox"), h, Nx, Ny, Nz), g("safe"))
    std, zn = O.correlation_quality_cell(g("res"), g("ref"), h, Nx, Ny, Nz)
    assert _close_nan(std, g("residual_std"), 1e-12) and _close_nan(zn, g("zncc"), 1e-12)
    assert _close_nan(O.gn_convergence_cell(g("dU"), g("U0"), Nx, Ny, Nz), g("gn"), 1e-13)
    active = g("res") != 0
    m = O.unsafe_masks(active, h, Nx, Ny, Nz, g("mask0"))
    for k in ("unsafe_vox", "unsafe_elem", "unsafe_node", "overlap_lost"):
        assert np.array_equal(m[k], g(k)), k
    m = O.unsafe_masks(active, h, Nx, Ny, Nz, g("mask0"), frac_threshold=0.2, min_material_frac=0.3)
    assert np.array_equal(m["overlap_lost"], g("overlap_lost_t"))
    assert np.array_equal(O.boundary_elements(Nx, Ny, Nz), g("boundary"))
    assert np.allclose(O.equivalent_strain(c["ps3"]), c["eq3"], rtol=1e-14, atol=0)


def test_ground_truth_harness_oracle():
    """Known-answer harness restatements against the reference's own
    outputs (tests/golden/gt.npz)."""
    c = load_golden("gt.npz")
    assert np.array_equal(O.gt_warp(c["ref"], c["u"]), c["deformed"])
    assert np.array_equal(O.gt_uniaxial(9, 0.02), c["uni"])
    gs = tuple(int(x) for x in c["g_shape"])
    assert np.array_equal(O.gt_voxel_in_bounds(c["u"], gs), c["inb"])
    oob = O.gt_node_oob_fraction(c["u"], int(c["h"]), tuple(int(x) for x in c["nb"]), gs, c["crop_lo"])
    assert np.allclose(oob, c["oob"], rtol=0, atol=1e-15)
