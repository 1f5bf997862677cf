"""The multi-rank host logic of bench.py on CPU: two gloo ranks (replicas,
no data-path collective) agree on the slowest rank's time, and the
reference arm prints from rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r "measured" 10 + 5 r ms; every rank must see the maximum
    out[rank] = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5


def test_reference_arm_prints_on_rank_zero_only(capsys, monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    args = bench.parse(["--impl", "reference"])
    bench.reference_arm(args)
    assert capsys.readouterr().out == ""


def test_reference_arm_json_contract(capsys, monkeypatch):
    """Rank 0 of the reference arm prints one JSON line with the metric of
    the GPU arm, the CPU baseline it measured -- the reference's own
    operators, installed in baseline/_ref -- and the end-to-end object; or,
    in a checkout without that install, its one-line `unavailable` record."""
    import json
    import bench
    monkeypatch.setenv("RANK", "0")
    args = bench.parse(["--impl", "reference", "--workload", "plain_small", "--steps", "1", "--warmup", "0",
                        "--cpu-procs", "2"])
    bench.reference_arm(args)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    if not os.path.isdir(os.path.join(bench.REF_DIR, "voxeldvc", "engine")):
        assert "baseline/_ref" in d["unavailable"]
        return
    assert d["unit"] == "s"
    assert d["higher_is_better"] is False and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "reference" and cb["cores"] == 2 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("plain_small")
