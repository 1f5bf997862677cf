"""Host logic of the ground-truth sweep (no GPU): one prepared input shared by
every pair, outcomes from the analysis figures, the solve log's last dU/U,
FAILED and DIVERGED pairs, the table, the best pairs and the CSV."""
import csv
import math

from voxeldvc_gb300.ground_truth import sweep_ground_truth as SW


def _figures(rms, rms_valid):
    return {"recoverable": (18, rms, 2 * rms), "valid": (9, rms_valid, 2 * rms_valid),
            "truncated": (9, 0.5, 1.0), "all": (27, 0.3, 1.0)}


def test_last_du_over_u():
    assert SW.last_du_over_u("Iter # 1 | dU/U=1.0e-01\nIter # 2 | dU/U=4.5e-04 | active\n") == 4.5e-4
    assert math.isnan(SW.last_du_over_u("no solve here"))


def test_outcome_from_analysis_and_row():
    o = SW.PairOutcome.from_analysis(8, 4.5, _figures(0.01, 0.005), 3e-4)
    r = o.row()
    assert set(r) == set(SW.FIELDS)
    assert (r["n_recoverable"], r["n_total"], r["n_valid"]) == (18, 27, 9)
    assert (r["rms"], r["max_err"], r["rms_valid"]) == (0.01, 0.02, 0.005)
    assert r["l0"] == 36.0 and r["status"] == "ok" and not o.diverged


def test_sweep_prepares_once_and_reports_failures(tmp_path, monkeypatch, capsys):
    calls = {"prepare": 0, "pairs": []}

    def prepare(gt_dir, *a, **k):
        calls["prepare"] += 1

    def solve(work, gt_dir, h, lf):
        calls["pairs"].append((h, lf))
        if h == 16:
            raise RuntimeError("boom")
        (tmp_path / f"h{h}_l0f{lf:g}" / "run_log.txt").write_text("Iter #  3 | dU/U=7.0e-04 |\n")
        return _figures(3.0 if lf < 3 else 0.02, 0.004 * h)

    monkeypatch.setattr(SW.pipeline, "prepare_input", prepare)
    monkeypatch.setattr(SW.pipeline, "solve_and_analyse", solve)
    out = SW.sweep([4, 8, 16], [2.25, 4.5], str(tmp_path), "ref.npy", tensile_strain=0.01)
    assert calls["prepare"] == 1 and len(calls["pairs"]) == 6
    assert [o.status for o in out] == ["ok", "ok", "ok", "ok", "FAILED", "FAILED"]
    assert (tmp_path / "h4_l0f4.5" / "gt_input").is_symlink()
    assert out[1].du_final == 7e-4
    lines = "\n".join(SW.summary_lines(out))
    assert "DIVERGED" in lines and "FAILED" in lines
    assert "Best by recoverable RMS (non-diverged): h=4, l0_factor=4.5" in lines
    assert "Best by valid RMS (non-diverged, fair measure): h=4, l0_factor=4.5" in lines
    SW.write_csv(str(tmp_path / "s.csv"), out)
    got = list(csv.DictReader(open(tmp_path / "s.csv")))
    assert [r["h"] for r in got] == ["4", "4", "8", "8", "16", "16"] and list(got[0]) == SW.FIELDS
