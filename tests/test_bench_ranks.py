"""The replica path of bench.py on CPU: two gloo ranks combine their timings
into the whole-job figures (slowest rank's time, all ranks' particle-steps),
and the reference arm's non-zero ranks exit without work."""
import os
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, ps = bench.combine_ranks([12.5, 20.0][rank], [1e6, 3e6][rank], dist, "cpu")
    out[rank] = (ms, ps)
    dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn")
        assert dict(out) == {0: (20.0, 4e6), 1: (20.0, 4e6)}


def test_combine_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(7.0, 5.0, None, "cpu") == (7.0, 5.0)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
