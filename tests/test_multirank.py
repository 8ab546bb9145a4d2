"""The multi-rank logic of bench.py on CPU with two gloo ranks: each rank
times its own replica (weak scaling), the job's time is the slowest rank's
(an all-reduce MAX of one value, the only collective), `value` sums the
ranks' units over that time, and the reference arm prints from rank 0 only.
The same functions run under NCCL on GPUs."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_local = 0.5 + 0.25 * rank                  # rank 1 is the slower one
        t = bench.max_over_ranks(t_local, dist, "cpu")
        v = bench.job_value(1.0e9, world, t)
        dist.barrier()
        out.put((rank, bench.env_rank(), t, v))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_and_value():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (r, world, local), t, v in res:
        assert (r, world, local) == (rank, 2, rank)
        assert t == 0.75                              # the slowest rank's time, on every rank
        assert v == pytest.approx(2 * 1.0e9 / 0.75)  # both ranks' units over that time


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, None, "cpu") == 1.25
    assert bench.job_value(10.0, 1, 2.0) == 5.0


def test_reference_arm_prints_on_rank_zero_only(monkeypatch):
    """Ranks other than 0 exit without work or output."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_arm(None, None)   # returns before touching its arguments
    assert buf.getvalue() == ""
