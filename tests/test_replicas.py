"""The replica path of the bench (torchrun, N > 1) on CPU: two gloo ranks.

Each rank renders its own seeded scenes; the only exchange is the host-side
measurement (slowest rank's time, whole-job rate).  No GPU is involved."""
import os
import socket

import pytest

from euc_gb300 import replicas, scenes


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = replicas.dist_env()
        seed = replicas.replica_seed(7, r)
        frames = scenes.batch_frames(seed=seed, n=3, tri_lo=50, tri_hi=200, resolutions=(64,), tex_size=8)
        step_ms = 10.0 * (r + 1)  # rank 1 is the slow one
        ms = replicas.max_over_ranks(step_ms)
        tris = replicas.sum_over_ranks(sum(f.ntris for f in frames))
        out.put((r, w, local, seed, [f.name for f in frames], ms, tris,
                 replicas.whole_job_rate(len(frames), w, ms / 1e3)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_measure_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, s0, n0, ms0, t0, v0), (r1, w1, l1, s1, n1, ms1, t1, v1) = res
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert s0 != s1 and n0 != n1                  # different scenes per rank
    assert ms0 == ms1 == 20.0                      # the slowest rank's time on both
    assert t0 == t1                                # the same job totals
    assert v0 == v1 == pytest.approx(2 * 3 / 0.020)  # whole-job scenes/s


def test_one_replica_needs_no_process_group():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.replica_seed(5, 0) == 5 and replicas.replica_seed(5, 2) == 2005
