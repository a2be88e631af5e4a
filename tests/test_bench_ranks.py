"""The multi-rank logic of bench.py on CPU: replicas (one per GPU) time their
own steps and the job's time is the slowest rank's, gathered with a MAX
all-reduce -- here over two gloo ranks; the reference arm runs on rank 0
only."""
import contextlib
import io
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank])
        out.put((rank, got, bench.job_rate(1000, world, got[0])))
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, rate in res:
        assert got == [2.0, 10.0, 0.5]          # every rank sees the slowest rank's times
        assert rate == 2 * 1000 / 2.0           # both replicas' units over the slowest time


def test_single_rank_is_identity():
    assert bench.max_over_ranks([3.0, 4.5]) == [3.0, 4.5]
    assert bench.job_rate(10, 1, 2.0) == 5.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"])
        bench.run_reference(bench.parse_args())
    assert buf.getvalue() == ""
