"""The N > 1 host path of bench.py on CPU: two gloo ranks on 127.0.0.1.

Sims shard by replica (one sim per rank, seed + rank), so the only
cross-rank steps are the barrier around the timed region and the max over
ranks of the elapsed time; the reference arm runs on rank 0 alone and the
other ranks exit without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    mx = bench.max_over_ranks(float(10 * (r + 1)), w)
    import torch.distributed as dist
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f'rank{r}.json'), 'w') as f:
        json.dump({'world': w, 'rank': r, 'max': mx}, f)


def test_barrier_and_max_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method='spawn')
    for r in range(2):
        got = json.load(open(tmp_path / f'rank{r}.json'))
        assert got == {'world': 2, 'rank': r, 'max': 20.0}


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    port = _free_port()
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1', '--nproc-per-node=2',
           '--master-addr=127.0.0.1', f'--master-port={port}', 'bench.py', '--impl', 'reference', '--gpus', '2',
           '--steps', '1', '--warmup', '1', '--pop-size', '20000', '--days', '30']
    env = dict(os.environ, OMP_NUM_THREADS='1')
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith('{')]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line['impl'] == 'reference' and line['metric'] == 'agent-days/s' and line['value'] > 0
    assert line['cpu_baseline']['kind'] == 'port'
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['e2e']['d2h_bytes_per_step'] == 0
