"""The N > 1 path of the bench on CPU ranks (gloo, world size 2).

Codewords and frames are independent, so N GPUs run N replicas with no data-path
collective: each rank decodes its own seeded batches and the step time is the slowest
rank's (one all-reduce MAX after the timed region).  These tests run that reduction and
the whole-job value on two gloo ranks, and check that the ranks' inputs differ.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = 10.0 + 5.0 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(elapsed, "cpu")
        out[rank] = (slowest, bench.job_value(1000, world, 4, slowest))
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_slowest_rank_and_value_counts_every_rank():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1] == (15.0, 2 * 1000 * 4 / 15e-3)


def test_ranks_decode_distinct_replicas():
    from sicc_gb300 import channel, codes
    code = codes.short_code()
    # bench seeds: rank r uses 1000 * (r + 1) as the base of its batches
    a = channel.awgn_llrs(code, 16, 2.0, seed=1000 * 1 + 200)[2]
    b = channel.awgn_llrs(code, 16, 2.0, seed=1000 * 2 + 200)[2]
    assert a.shape == b.shape and not (a == b).all()


def test_bench_gpus_n_spawns_n_ranks():
    """`bench.py --gpus 2` without a launcher starts two ranks itself (torch.distributed.run on
    127.0.0.1) and rank 0 alone prints the line, labelled with both ranks.  The reference arm needs
    no GPU, so this runs the spawn path on CPU."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "1", "--cpu-sample", "64"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    line = json.loads(lines[0])
    assert line["n_gpus"] == 2 and line["impl"] == "reference"
