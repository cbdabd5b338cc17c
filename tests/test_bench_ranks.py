"""The multi-rank path of bench.py on CPU (gloo, world size 2): replicas, the
slowest rank's times over all ranks, whole-job solves/s; the reference arm does
no work on ranks other than 0."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip('torch')
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}', rank=rank, world_size=world)
    try:
        # rank r timed 10 (r + 1) ms on the device and 12 (r + 1) ms end to end for 5 steps
        out[rank] = bench.replica_rates(10.*(rank + 1), 12.*(rank + 1), 5, world)
    finally:
        dist.destroy_process_group()


def test_replica_rates_take_the_slowest_rank():
    ctx = torch.multiprocessing.get_context('spawn')
    with ctx.Manager() as manager:
        out = manager.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            ms, e_ms, value, e2e = out[r]
            assert ms == 20. and e_ms == 24.
            assert value == pytest.approx(2*5/0.020) and e2e == pytest.approx(2*5/0.024)


def test_single_rank_rates():
    sys.path.insert(0, ROOT)
    import bench
    ms, e_ms, value, e2e = bench.replica_rates(8., 10., 4, 1)
    assert (ms, e_ms) == (8., 10.) and value == pytest.approx(500.) and e2e == pytest.approx(400.)


def test_reference_arm_idle_on_other_ranks():
    env = dict(os.environ, RANK='1', WORLD_SIZE='2', LOCAL_RANK='1')
    proc = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--steps', '1',
                           '--warmup', '3'], env=env, capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0 and proc.stdout.strip() == ''
