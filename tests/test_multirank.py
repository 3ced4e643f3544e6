"""The N > 1 path of bench.py on CPU with two gloo ranks: rendezvous on
127.0.0.1, the barrier, the max over ranks of the timed region, and the
reference arm under torchrun (rank 0 alone works and prints one line, the
other rank exits 0). The path itself runs independent replicas, one per GPU:
there is no data-path collective to test."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

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
    r, w = bench.dist_init(world)
    bench.barrier(w)
    got = bench.max_over_ranks(1.5 + r, w)
    with open(os.path.join(out_dir, f"rank{r}.txt"), "w") as f:
        f.write(f"{r} {w} {got}")
    import torch.distributed as dist
    dist.destroy_process_group()


def test_barrier_and_max_over_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    for r in range(2):
        rank, world, got = open(tmp_path / f"rank{r}.txt").read().split()
        assert int(rank) == r and int(world) == 2 and float(got) == 2.5


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
