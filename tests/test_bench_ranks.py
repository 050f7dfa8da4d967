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


def test_profile_ingest_maps_kernels_to_families(tmp_path):
    """The ncu-csv reader of bench.py groups a step's launches into the launch
    families whose counts and traffic the bench line reports."""
    import bench
    names = {
        "void mhd::k_cfl<float, 0, 0>(mhd::KArg<T1, T3>, int)": "dt",
        "void mhd::k_emf_pdm<float, 1, 32, 1, 8, 256, 0, 0>(mhd::KArg<T1, T8>)": "emf",
        "void mhd::k_flux<float, 1, 0, 0, 0>(mhd::KArg<T1, T5>)": "flux_x",
        "void mhd::k_flux_sweep<float, 1, 0, 1>(mhd::KArg<T1, T3>)": "flux_y",
        "void mhd::k_flux_sweep<float, 2, 0, 1>(mhd::KArg<T1, T3>)": "flux_z_update",
        "void mhd::k_ct_fill<float, 0>(mhd::KArg<T1, T2>, int)": "ct",
        "void mhd::k_fill_bxyz<float, 0, 0>(mhd::KArg<T1, T3>, int, int)": "ct",
        "void mhd::k_emf_stream<float, 0, 8, 0, 0>(mhd::KArg<T1, T5>, mhd::Inp<T1>, mhd::Prm<T1>)": "emf",
        "void mhd::k_emf_rows<float, 0, 0>(mhd::KArg<T1, T3>, mhd::Inp<T1>, mhd::Prm<T1>)": "emf",
        "void mhd::k_cfl_final<float>(mhd::Dev<T1>, int)": "dt",
    }
    for k, fam in names.items():
        assert bench._family(k) == fam, k
    # classes with their own launches per RK2 step: the boundary-row launch and
    # the ghost shell are counted apart from their families' main kernels
    assert bench._class("void mhd::k_emf_rows<float, 0, 0>(x)") == "emf_rows"
    assert bench._class("void mhd::k_emf_stream<float, 2, 8, 0, 0>(x)") == "emf"
    assert bench._class("void mhd::k_fill_bxyz<float, 0, 0>(x)") == "shell"
    assert bench._class("void mhd::k_ct_fill<float, 0>(x)") == "ct_fill"
    assert bench._PER_STEP["emf"] == 6 and bench._PER_STEP["emf_rows"] == 2
    csv = tmp_path / "c.csv"
    lines = ['"ID","Kernel Name","Metric Name","Metric Unit","Metric Value"']
    for i, k in enumerate(names):
        lines.append(f'"{i}","{k}","gpu__time_duration.sum","ns","1,000"')
        lines.append(f'"{i}","{k}","smsp__thread_inst_executed.sum","inst","{100 * (i + 1)}"')
    csv.write_text("\n".join(lines) + "\n")
    rows = bench._ncu_rows(str(csv))
    assert [r[0] for r in rows] == list(names)
    assert rows[2][1]["smsp__thread_inst_executed.sum"] == 300.0
    assert rows[0][1]["gpu__time_duration.sum"] == 1000.0
    # per-step sums: each class scaled from its captured launches to its
    # launches per RK2 step, then summed into its family
    fam = bench._step_sums(str(csv), lambda m: {"inst": m["smsp__thread_inst_executed.sum"]})
    inst = {k: 100 * (i + 1) for i, k in enumerate(names)}
    ks = list(names)
    assert fam["emf"]["inst"] == 6 * (inst[ks[1]] + inst[ks[7]]) / 2 + 2 * inst[ks[8]]
    assert fam["ct"]["inst"] == 2 * inst[ks[5]] + 2 * inst[ks[6]]
    assert fam["dt"]["inst"] == (inst[ks[0]] + inst[ks[9]]) / 2
