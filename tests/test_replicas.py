"""Multi-process host logic of bench.py (replicas: one process per GPU, gloo only for the barrier and the
max-over-ranks timing), run as world_size-2 gloo groups on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    m = bench.max_over_ranks(pg, 1.5 + r)
    with open(os.path.join(out_dir, f"r{r}.json"), "w") as fh:
        json.dump({"world": w, "rank": r, "local": local, "max": m}, fh)
    pg.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    assert [x["rank"] for x in res] == [0, 1]
    assert all(x["world"] == 2 and x["max"] == 2.5 for x in res)


def test_reference_arm_under_torchrun(tmp_path):
    """`bench.py --impl reference` under torchrun with two ranks: rank 0 alone runs and prints one JSON line."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", "ico_nve", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    run = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=str(tmp_path))
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [ln for ln in run.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
