"""Replica aggregation across ranks (gloo, world_size 2, on the CPU): the
whole-job throughput is the sum of work over the slowest rank's time, and a
rank that fails is reported to the others by the process group."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out, fail_rank):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from qdeqcycle_fdm_gb300 import replicas
    r, w, _ = replicas.init("gloo", timeout_s=20.0)
    assert (r, w) == (rank, world)
    if rank == fail_rank:
        dist.destroy_process_group()
        raise SystemExit(3)
    try:
        units, secs, value = replicas.aggregate(10.0 * (rank + 1), 2.0 + rank)
        out.put((rank, units, secs, value))
    except Exception as e:       # the peer left: the collective errors out
        out.put((rank, "error", type(e).__name__, None))
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def _run(world, fail_rank=-1, timeout=60):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q, fail_rank)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout)
    for p in procs:
        if p.is_alive():
            p.kill()
    res = []
    while not q.empty():
        res.append(q.get())
    return sorted(res, key=lambda x: x[0]), [p.exitcode for p in procs]


def test_two_replicas_aggregate_sum_over_max():
    res, codes = _run(2)
    assert codes == [0, 0]
    for rank, units, secs, value in res:
        assert units == 30.0 and secs == 3.0 and value == 10.0


def test_failed_rank_is_reported_to_the_survivor():
    """A rank that leaves between steps (its process group torn down, exit
    code 3) makes the survivor's aggregation collective raise instead of
    hanging; the survivor reports the error and exits cleanly."""
    res, codes = _run(2, fail_rank=1)
    assert codes[1] == 3
    assert codes[0] == 0
    assert len(res) == 1 and res[0][0] == 0 and res[0][1] == "error", res


def test_single_rank_is_identity():
    from qdeqcycle_fdm_gb300 import replicas
    assert replicas.aggregate(5.0, 2.0) == (5.0, 2.0, 2.5)
