"""The N>1 host path of bench.py on CPU: two gloo ranks.

Every rank runs the per-GPU workload on its own elements (replicas, no
collective on the data path); the only collectives are the barrier around the
timed region and the max over ranks of the step time.  These tests run both
with world_size 2 on the gloo backend, and the reference arm under torchrun,
where rank 0 alone works and prints."""
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


def _rank_main(rank, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": "2", "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    r, ws, local = bench.dist_init()
    assert (r, ws, local) == (rank, 2, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(ws)
    out[rank] = bench.max_over_ranks(1.5 + rank, ws)
    bench.barrier(ws)
    dist.destroy_process_group()


def test_barrier_and_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(out) == {0: 2.5, 1: 2.5}


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once():
    import oracle
    oracle.build()
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=500, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
