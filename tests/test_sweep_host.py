"""Host logic of the ground-truth sweep (no GPU): reading a run's saved
error arrays and log, the summary table and the CSV."""
import csv

import numpy as np

from voxeldvc_gb300.ground_truth import sweep_ground_truth as SW


def _fake_run(d, err_scale, valid=True):
    d.mkdir()
    rng = np.random.default_rng(0)
    err = rng.standard_normal((3, 3, 3, 3)) * err_scale
    trunc = np.zeros((3, 3, 3), bool)
    trunc[0] = True
    np.save(d / "U_error.npy", err)
    np.save(d / "node_truncated_mask.npy", trunc)
    if valid:
        v = ~trunc
        v[-1] = False
        np.save(d / "node_valid_mask.npy", v)
    (d / "run_log.txt").write_text("Iter # 1 | dU/U=1.0e-01\nIter # 2 | dU/U=4.5e-04 | active\n")
    return err, trunc


def test_summarize_combo(tmp_path):
    err, trunc = _fake_run(tmp_path / "a", 0.01)
    st = SW.summarize_combo(str(tmp_path / "a"))
    sel = err[~trunc]
    assert st["n_recoverable"] == 18 and st["n_total"] == 27 and st["n_valid"] == 9
    assert np.isclose(st["rms"], np.sqrt(np.mean(sel ** 2)))
    assert np.isclose(st["max_err"], np.linalg.norm(sel, axis=-1).max())
    assert st["du_final"] == 4.5e-4 and st["status"] == "ok"
    _fake_run(tmp_path / "b", 0.01, valid=False)
    st = SW.summarize_combo(str(tmp_path / "b"))
    assert st["n_valid"] == 0 and np.isnan(st["rms_valid"])
    assert np.isnan(SW.parse_final_du_over_u(str(tmp_path / "missing.txt")))


def test_table_best_and_csv(tmp_path, capsys):
    rows = [dict(h=8, l0_factor=4.5, l0=36.0, n_recoverable=10, n_total=27, rms=0.01, max_err=0.02, n_valid=5,
                 rms_valid=0.005, max_err_valid=0.01, du_final=1e-4, status="ok"),
            dict(h=4, l0_factor=2.25, l0=9.0, n_recoverable=10, n_total=27, rms=3.0, max_err=5.0, n_valid=5,
                 rms_valid=0.001, max_err_valid=2.0, du_final=1e-1, status="ok")]
    SW.print_summary_table(rows)
    out = capsys.readouterr().out
    assert "DIVERGED" in out and "Best by valid RMS (non-diverged, fair measure): h=8" in out
    SW.write_csv(str(tmp_path / "s.csv"), rows)
    got = list(csv.DictReader(open(tmp_path / "s.csv")))
    assert [r["h"] for r in got] == ["8", "4"] and set(got[0]) == set(SW.FIELDS)
