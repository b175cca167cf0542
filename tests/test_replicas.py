"""Several GPUs run independent replicas; only the timing is combined across ranks
(scatter_gb300.replicas, used by bench.py under torchrun).  Two gloo ranks on CPU: barrier,
the longest rank's time, and the units every rank processed."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from scatter_gb300 import replicas

        replicas.barrier()
        # rank r: its replica took 10 + 5 r ms for 1000 (r + 1) DOF-steps
        ms, rate = replicas.job_rate(10.0 + 5.0 * rank, 1000.0 * (rank + 1))
        replicas.barrier()
        out.put((rank, replicas.world(), ms, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_timing():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (world, r), ms, rate in results:
        assert world == 2 and r == rank
        assert ms == 15.0  # the longest rank
        assert abs(rate - 3000.0 / 0.015) <= 1e-9 * rate  # all ranks' DOF-steps over that time


def test_one_process_without_a_group():
    sys.path.insert(0, ROOT)
    from scatter_gb300 import replicas

    assert replicas.world() == (1, 0)
    replicas.barrier()
    ms, rate = replicas.job_rate(20.0, 500.0)
    assert ms == 20.0 and rate == 500.0 / 0.02
