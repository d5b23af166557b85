"""Multi-rank query sharding, exercised with 2 gloo ranks on the CPU (the
per-rank evaluator here is the CPU oracle; on GPUs it is the library call)."""
import os
import socket

import numpy as np
import pytest

from libigl_gb300.shard import evaluate_sharded, shard_bounds


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 7, 10, 1001):
        for world in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, F, Q = synth.exact_workload(seed=1, subdiv=2, nq=1001)
    W = evaluate_sharded(lambda Qs: O.winding_number(V, F, Qs, nthreads=1), Q)
    q.put((rank, W))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_identical_full_result():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, F, Q = synth.exact_workload(seed=1, subdiv=2, nq=1001)
    W = O.winding_number(V, F, Q, nthreads=1)
    assert np.array_equal(res[0], res[1])
    assert np.array_equal(res[0], W)
