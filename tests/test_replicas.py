"""Multi-GPU is replicas only: each rank renders its own frame, the job time
is the slowest rank's (max over ranks) and the value sums all ranks' work.
The host-side logic of bench.py runs here as two gloo ranks on CPU."""
import importlib.util
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = _bench()
    my_ms = [1.5, 2.25][rank]
    ms = b.max_over_ranks(my_ms, torch.device("cpu"))
    out[rank] = (ms, b.whole_job_rate(1048576, world, ms))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.25
    assert abs(res[0][1] - 1048576 * 2 / 2.25e-3 / 1e6) < 1e-9


def test_dist_env_defaults(monkeypatch):
    b = _bench()
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert b.dist_env() == (0, 1, 0)
    monkeypatch.setenv("RANK", "3")
    monkeypatch.setenv("WORLD_SIZE", "4")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert b.dist_env() == (3, 4, 1)
