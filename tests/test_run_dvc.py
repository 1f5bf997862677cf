"""`voxeldvc run` on the GB300 engine: the work-directory contract of the
reference's run_dvc.main (affine_prealign.json + preprocessed volumes)."""
import json

import numpy as np
import pytest

from conftest import load_golden


def _work_dir(tmp_path, shift=(0, 0, 0)):
    c = load_golden("solve_multiscale.npz")
    f, g = c["f"], c["g"]
    np.save(tmp_path / "ref_preprocessed.npy", f)
    np.save(tmp_path / "def_preprocessed.npy", g)
    np.save(tmp_path / "def_ref_aligned.npy", g)
    meta = {"h": 8, "glt": 0.0, "affine_A": np.eye(3).tolist(), "affine_t": [0.0, 0.0, 0.0],
            "affine_c": [(s - 1) / 2 for s in f.shape], "crop_lo": [0, 0, 0], "crop_hi": list(f.shape),
            "def_lo": list(shift), "def_hi": list(g.shape)}
    (tmp_path / "affine_prealign.json").write_text(json.dumps(meta))
    return f, g


def test_cli_help_and_parse():
    from voxeldvc_gb300 import cli, run_dvc
    assert cli.main([]) == 0
    a = run_dvc.parse_args(["/x", "--l0-factor", "2.25"])
    assert a.work_dir == "/x" and a.l0_factor == 2.25
    assert run_dvc.mesh_dims((33, 25, 17), 8) == (4, 3, 2)


@pytest.mark.gpu
def test_run_writes_the_solve(tmp_path, cuda):
    from voxeldvc_gb300 import run_dvc
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    f, g = _work_dir(tmp_path, shift=(0, 0, 0))
    assert run_dvc.main([str(tmp_path)]) == 0
    U_rec = np.load(tmp_path / "U_recovered.npy")
    assert U_rec.shape == (5, 4, 3, 3)
    U, res, dU = CG.multiscale_correlate_gpu(f, g, 4, 3, 2, 8, xp=np, scales=(2, 1, 0), l0=36.0, glt=0.0,
                                             K_ref_laplacian=G.build_K_ref_laplacian(), dynamic_mask=True,
                                             fft_prealign=False, ext_affine=(np.eye(3), np.zeros(3),
                                                                             np.array([16.0, 12.0, 8.0])),
                                             disp=False, freeze_mask_after=4)
    grid = np.stack([U[c::3].reshape(5, 4, 3, order='F') for c in range(3)], axis=-1)
    assert np.allclose(U_rec, grid, atol=1e-12)
    assert np.load(tmp_path / "residual.npy").shape == f.shape
    log = (tmp_path / "run_log.txt").read_text()
    assert "dU/U=" in log
    # post-solve stages: the pushed reference matches the oracle's push of
    # the same displacement; the ZNCC line is logged
    from oracle import dvc_oracle as O
    pushed = np.load(tmp_path / "ref_forward_pushed.npy")
    assert np.allclose(pushed, O.push_field_forward(f.astype(np.float64), U, 4, 3, 2, 8), atol=1e-9)
    assert "ZNCC (active voxels):" in log
    # element-scale fields: strains against the oracle, masks of the right shape
    ps = np.load(tmp_path / "principal_strains_cell.npy")
    assert np.allclose(ps, O.principal_strains_cell(grid, 8), rtol=0, atol=1e-14)
    assert np.allclose(np.load(tmp_path / "equivalent_strain_cell.npy"), O.equivalent_strain(ps), rtol=1e-13)
    res = np.load(tmp_path / "residual.npy").reshape(-1, order='F')
    std, zn = O.correlation_quality_cell(res, f, 8, 4, 3, 2)
    assert np.allclose(np.load(tmp_path / "zncc_cell.npy"), zn, rtol=1e-12, equal_nan=True)
    assert np.allclose(np.load(tmp_path / "residual_std_cell.npy"), std, rtol=1e-12, equal_nan=True)
    for name in ("material_cell_mask", "material_cell_mask_eroded", "overlap_lost_element_mask"):
        m = np.load(tmp_path / f"{name}.npy")
        assert m.shape == (4, 3, 2) and m.dtype == bool, name
    uv = np.load(tmp_path / "unsafe_voxel_mask.npy")
    assert uv.shape == f.shape
    up = np.load(tmp_path / "unsafe_voxel_mask_forward_pushed.npy")
    assert up.dtype == bool and up.shape == f.shape
    ref_up = O.push_field_forward(uv.astype(np.float64), U, 4, 3, 2, 8, order=0, mode='constant', cval=1.0)
    assert np.array_equal(up, ref_up.astype(bool))
    assert "cell eq. strain:" in log and "Material cells" in log
