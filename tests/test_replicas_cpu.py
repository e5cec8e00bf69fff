"""Multi-process (N > 1) plumbing of bench.py on CPU: two gloo ranks.

Patches are independent and a solve exchanges nothing, so N GPUs run N replicas of the
workload; the only collectives are the barrier around the timed region, the max over the
ranks' times and the sum of the solves.  These tests run that logic as world_size-2 gloo
process groups on 127.0.0.1, and the reference arm under torchrun, where rank 0 alone
works and prints one JSON line.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        t_max = d.max(1.5 + rank)             # per-rank timed region (s)
        total = d.sum(100 * (rank + 1))       # solves done per rank
        q.put((rank, t_max, total))
    finally:
        d.close()


def test_gloo_two_ranks_max_and_sum():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, total in out:
        assert t_max == 2.5          # the slowest rank's time
        assert total == 300.0        # all ranks' solves


def test_reference_arm_under_torchrun_rank0_prints_once():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cpu-threads", "2", "--cpu-max-side", "40", "--patches", "256"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2
    assert rec["value"] > 0 and rec["cpu_baseline"]["kind"] == "port"
    assert rec["e2e"]["h2d_bytes_per_step"] == 0
