"""The N>1 bench path: one replica per rank, no data-path collective; the
job's time is the maximum over ranks and its throughput sums the ranks'
units.  Runs as two gloo ranks on the CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        bench.barrier(2)
        t = bench.allmax(10.0 + 5.0 * rank, 2)  # rank 1 is the slower replica
        bench.barrier(2)
        q.put((rank, t, bench.replica_value(1000, 4, 2, t)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_max_time_and_summed_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in out:
        assert t == 15.0
        assert abs(v - 1000 * 4 * 2 / 0.015) < 1e-6 * v
