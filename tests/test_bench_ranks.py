"""The bench's replica path on CPU ranks (gloo, world size 2, 127.0.0.1):
max-over-ranks step time, whole-job throughput of independent replicas,
and the reference arm printing from rank 0 only."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    q.put((rank, ms, bench.replicas_value(1000, world, ms)))
    dist.destroy_process_group()


def _free_port():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    # both ranks see the slower rank's 15 ms; 2 x 1000 units over 15 ms
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == pytest.approx(2 * 1000 / 0.015)


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replicas_value(500, 1, 10.0) == pytest.approx(50000.0)


def test_reference_arm_prints_on_rank0_only(tmp_path):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", WORLD_SIZE="2", LOCAL_RANK="0")
    args = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
            "--cpu-sample-nx", "10", "--no-size-series"]
    r1 = subprocess.run(args, env=dict(env, RANK="1"), capture_output=True, text=True, timeout=300)
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    r0 = subprocess.run(args, env=dict(env, RANK="0"), capture_output=True, text=True, timeout=300)
    assert r0.returncode == 0, r0.stderr
    line = json.loads(r0.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_reference_size_series_fit():
    """The size series' power-law fit passes through its own points and
    extrapolates with the fitted exponent."""
    import bench
    ser = bench.size_series(nxs=(10, 15, 20), target_dof=10_000)
    pts = ser["points"]
    assert [q["cells"] for q in pts] == ["10x2x2", "15x3x3", "20x4x4"]
    assert all(q["dof_solves_per_s_per_core"] > 0 for q in pts)
    k = ser["exponent"]
    c = pts[-1]["dof_solves_per_s_per_core"] / pts[-1]["n_dof"] ** k
    assert ser["extrapolated_dof_solves_per_s_per_core"] == pytest.approx(c * 10_000 ** k, rel=0.5)
