"""The N > 1 path of bench.py on CPU (gloo, world size 2): replicas, the
max-over-ranks job time and the whole-job rate; the reference arm prints on
rank 0 only."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    dist.barrier()
    ms = bench.job_time_ms(10.0 + 2.5 * rank, dist)
    q.put((rank, ms, bench.whole_job_rate(256, 100, ws, ms)))
    dist.destroy_process_group()


def test_job_time_is_the_slowest_rank_and_rate_counts_every_replica():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, rate in out:
        assert ms == 12.5
        assert rate == pytest.approx(2 * 256 ** 3 * 100 / 12.5e-3)


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_runs_the_same_config_as_ours():
    """The reference arm times the oracle (array passes) on the same workload
    description as our arm: identical config dicts, so the two lines compare
    like for like."""
    import json
    import bench
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--n", "12", "--steps", "2",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 2
    assert line["config"] == bench.bench_config(12, 1)
    assert line["e2e"]["value"] == line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
