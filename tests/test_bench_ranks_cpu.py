"""The multi-GPU path is replicas only (PSFs, wavelengths and segments are
independent; there is no data exchange): bench.py's one collective is the
MAX of the ranks' timed regions.  Two gloo ranks on the CPU check that every
rank gets the slowest rank's time and the whole-job throughput, and that the
reference arm prints from rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.slowest_rank(100.0 + 50.0 * rank, 20, world, 'cpu')
    q.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_slowest_rank_two_gloo_ranks():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, ms, value in got:
        assert ms == 150.0                       # the slowest rank's time everywhere
        assert value == pytest.approx(2 * 20 / 0.150)


def test_slowest_rank_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_rank(250.0, 10, 1, 'cpu') == (250.0, 40.0)


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK='1', WORLD_SIZE='2', LOCAL_RANK='1')
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference',
                        '--steps', '1', '--warmup', '0'], capture_output=True, text=True,
                       env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ''
