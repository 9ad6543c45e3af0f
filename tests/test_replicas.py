"""Replicas across ranks (mke_gb300/replicas.py) on the CPU: two gloo ranks
shard an ensemble, time it, take the maximum over ranks and gather the
members' results on rank 0 -- the host-side part of `bench.py --gpus N`
(one process per GPU, no collective on the data path)."""
import os
import socket

import numpy as np
import pytest

from mke_gb300 import replicas


@pytest.mark.parametrize("world", [1, 2, 3, 5])
@pytest.mark.parametrize("n", [0, 1, 7, 32, 257])
def test_shard_covers_every_unit_once(world, n):
    seen = []
    sizes = []
    for r in range(world):
        a, b = replicas.shard(n, r, world)
        seen.extend(range(a, b))
        sizes.append(b - a)
    assert seen == list(range(n))
    assert max(sizes) - min(sizes) <= 1


def test_shard_rejects_bad_arguments():
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)
    with pytest.raises(ValueError):
        replicas.shard(4, 0, 0)


def test_alone_no_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert replicas.init("gloo") is False
    assert replicas.max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
    x = np.arange(6.0).reshape(3, 2)
    assert replicas.gather_rows(x) is x
    assert replicas.whole_job_rate(10, 2.0, 1) == 5.0


def member_state(k):
    """Stand-in for one ensemble member's result: depends only on the member index."""
    return np.sin(np.arange(5) + 0.1 * k)


def _rank(rank, world, port, n, outq):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    try:
        assert replicas.init("gloo") is True
        assert replicas.env() == (world, rank, rank)
        a, b = replicas.shard(n, rank, world)
        local = np.stack([member_state(k) for k in range(a, b)]) if b > a else np.zeros((0, 5))
        # per-rank "times": the slowest rank sets the whole-job rate
        t = replicas.max_over_ranks([0.5 + rank, 10.0 * rank])
        replicas.barrier()
        full = replicas.gather_rows(local)
        if rank == 0:
            outq.put(("ok", t, full, replicas.whole_job_rate(n / world, t[0], world)))
        replicas.finish()
    except Exception as e:   # reported to the parent
        outq.put(("error", repr(e), None, None))
        raise


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n", [9, 2])
def test_two_gloo_ranks(n):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    status, t, full, rate = q.get(timeout=10)
    assert status == "ok", t
    assert t == [1.5, 10.0]
    assert np.array_equal(full, np.stack([member_state(k) for k in range(n)]))
    assert rate == pytest.approx(n / 1.5)
