"""The N>1 host paths of bench.py on CPU with the gloo backend, two ranks on
127.0.0.1: the job time is the slowest rank's (max over ranks, the rule for
every timed figure of the line), and under torchrun the reference arm runs
on rank 0 alone and prints one line.  The GPU replicas themselves share no
data (one independent simulation per rank), so nothing else crosses ranks."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as td

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(td, 10.0 + 5.0 * rank)   # rank 1 is the slow one
    none = bench.max_over_ranks(None, 3.0)
    td.barrier()
    td.destroy_process_group()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"max": got, "none": none}, f)


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    mp.start_processes(_rank_main, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for r in (0, 1):
        d = json.load(open(tmp_path / f"r{r}.json"))
        assert d == {"max": 15.0, "none": 3.0}


def test_reference_arm_under_torchrun_rank0_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--nx", "64", "--steps", "3", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 3
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
