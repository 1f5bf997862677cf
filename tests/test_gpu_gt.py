"""Known-answer (ground-truth) harness on the GPU: the harness kernels against
the reference's own outputs (tests/golden/gt.npz), and the whole
prepare -> preprocess -> run -> analyse pipeline on the seeded 65^3 stand-in
for the reference's tension dataset."""
import json
import os

import numpy as np
import pytest

from conftest import load_golden
from oracle import dvc_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def GT(cuda):
    from voxeldvc_gb300.ground_truth import analyse_ground_truth as A
    from voxeldvc_gb300.ground_truth import prepare_ground_truth as P
    return P, A


def test_harness_kernels_match_reference(GT):
    P, A = GT
    c = load_golden("gt.npz")
    # bit-identical to RegularGridInterpolator, extrapolation included
    assert np.array_equal(P.make_deformed_image(c["ref"], c["u"]), c["deformed"])
    assert np.array_equal(P.make_uniaxial_gt(9, 0.02), c["uni"])
    gs = tuple(int(x) for x in c["g_shape"])
    assert np.array_equal(A.voxel_in_bounds(c["u"], gs), c["inb"])
    oob = A.node_oob_fraction(c["u"], int(c["h"]), *(int(x) for x in c["nb"]), gs, c["crop_lo"])
    assert np.array_equal(oob, c["oob"])
    assert np.array_equal(A.grid_to_dofs(c["U_grid"]), c["dofs"])


def test_harness_kernels_match_oracle_large(GT):
    P, A = GT
    rng = np.random.default_rng(5)
    n = 70
    ref = rng.random((n, n + 3, n - 4)) * 100
    u = rng.standard_normal((n, n + 3, n - 4, 3)) * 2.0
    assert np.array_equal(P.make_deformed_image(ref, u), O.gt_warp(ref, u))
    gs = (n - 5, n + 1, n - 2)
    assert np.array_equal(A.voxel_in_bounds(u, gs), O.gt_voxel_in_bounds(u, gs))
    oob = A.node_oob_fraction(u, 8, 8, 9, 7, gs, np.array([3, 2, 4]))
    assert np.array_equal(oob, O.gt_node_oob_fraction(u, 8, (8, 9, 7), gs, np.array([3, 2, 4])))


def test_node_oob_fraction_rejects_nodes_off_the_image(GT):
    _, A = GT
    u = np.zeros((10, 10, 10, 3))
    with pytest.raises(ValueError, match="nodes outside the image"):
        A.node_oob_fraction(u, 4, 4, 2, 2, (10, 10, 10), np.array([0, 0, 0]))


@pytest.mark.parametrize("kind", ["z+0.01", "z-0.05"])
def test_pipeline_matches_reference_run(GT, tmp_path, kind):
    """prepare -> preprocess -> run -> analyse on the seeded 65^3 stand-ins
    (+1 % tension, -5 % compression; lateral contraction and a smooth
    non-affine part), h = 8, l0 = 4.5 h, against the same pipeline run
    through the reference's own CPU code (tests/golden/gt_pipeline_*.npz):
    same crops, the recovered nodal field within 5e-3 vx, the same node
    sets and accuracy figures."""
    import hashlib
    from voxeldvc_gb300 import run_ground_truth_pipeline as RG
    from voxeldvc_gb300 import synth
    g = load_golden(f"gt_pipeline_{kind}.npz")
    ref, U = synth.gt_stand_in(kind)
    assert hashlib.sha256(ref.tobytes() + U.tobytes()).hexdigest() == str(g["digest"])
    np.save(tmp_path / "ref_in.npy", ref)
    np.save(tmp_path / "U_in.npy", U)
    out = tmp_path / "gt_run"
    assert RG.main(["--output-dir", str(out), "--gt-ref-file", str(tmp_path / "ref_in.npy"),
                    "--gt-displacement-file", str(tmp_path / "U_in.npy")]) == 0
    meta = json.load(open(out / "affine_prealign.json"))
    assert meta["h"] == 8
    assert meta["crop_lo"] == g["lo"].tolist() and meta["crop_hi"] == g["hi"].tolist()
    assert meta["def_lo"] == g["lo_def"].tolist() and meta["def_hi"] == g["hi_def"].tolist()
    assert np.abs(np.array(meta["affine_A"]) - g["A"]).max() < 1e-4
    U_rec = np.load(out / "U_recovered.npy") - np.array(meta["crop_lo"])
    assert np.abs(U_rec - g["U_grid"]).max() < 5e-3
    err = np.load(out / "U_error.npy")
    valid = np.load(out / "node_valid_mask.npy")
    rec = ~np.load(out / "node_truncated_mask.npy")
    assert np.array_equal(rec, g["rec"]) and np.array_equal(valid, g["valid"])
    rms_valid = float(np.sqrt(np.mean(err[valid] ** 2)))
    rms_rec = float(np.sqrt(np.mean(err[rec] ** 2)))
    assert abs(rms_valid - float(g["rms_valid"])) < max(0.05 * float(g["rms_valid"]), 5e-4), rms_valid
    assert abs(rms_rec - float(g["rms_rec"])) < max(0.05 * float(g["rms_rec"]), 5e-4), rms_rec
    log = (out / "ground_truth_comparison_log.txt").read_text()
    assert "valid (recoverable & unmasked)" in log
    for f in ("U_gt_vox.npy", "U_recovered_vox.npy", "voxel_valid_mask.npy", "node_oob_fraction.npy"):
        assert os.path.exists(out / f), f


def test_sweep_runs_each_pair(GT, tmp_path):
    """sweep-ground-truth over h in {4, 8}, l0 = 4.5 h on the tension stand-in:
    one run directory per pair, the h = 8 row equal to the single pipeline
    run (and so to the reference's own run), a CSV row per pair."""
    import csv
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300.ground_truth import sweep_ground_truth as SW
    ref, U = synth.gt_stand_in("z+0.01")
    np.save(tmp_path / "ref_in.npy", ref)
    np.save(tmp_path / "U_in.npy", U)
    root = tmp_path / "sweep"
    assert SW.main(["--gt-ref-file", str(tmp_path / "ref_in.npy"), "--gt-displacement-file",
                    str(tmp_path / "U_in.npy"), "--h", "4,8", "--l0-factor", "4.5", "--output-root", str(root),
                    "--csv", str(tmp_path / "sweep.csv")]) == 0
    rows = {int(r["h"]): r for r in csv.DictReader(open(tmp_path / "sweep.csv"))}
    assert set(rows) == {4, 8} and all(r["status"] == "ok" for r in rows.values())
    g = load_golden("gt_pipeline_z+0.01.npz")
    assert abs(float(rows[8]["rms_valid"]) - float(g["rms_valid"])) < max(0.05 * float(g["rms_valid"]), 5e-4)
    assert abs(float(rows[8]["rms"]) - float(g["rms_rec"])) < max(0.05 * float(g["rms_rec"]), 5e-4)
    assert float(rows[4]["rms"]) < 1.0  # not diverged
    assert (root / "h4_l0f4.5" / "U_error.npy").exists() and (root / "h8_l0f4.5" / "run_log.txt").exists()
