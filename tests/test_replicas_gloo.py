"""Multi-process (world_size 2, gloo, CPU) checks of the benchmark's N > 1 path.  A chain does not
shard, so N GPUs run independent replicas: the only cross-rank traffic is the barrier, the
max-over-ranks of the timed region, the sum of work done and the gather of per-request
latencies, and independent requests are partitioned across ranks with no overlap.  The replica
work itself is the oracle's gate step here (the product path needs a GPU); each rank's results
must equal what a single process computes for the same requests."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _requests(count):
    """Small independent gate steps: (site arrays, gate) with seeded inputs."""
    sys.path.insert(0, os.path.join(ROOT, "qrochet.jl_gb300"))
    from qrochet import random as R

    g = R.rng(77)
    out = []
    for _ in range(count):
        arrays = R.rand_chain_state_arrays(g, 6, 4, p=2)
        out.append((arrays, R.haar_unitary(g, 4)))
    return out


def _solve(req):
    """<Z_3> after one gate on bond (3, 4): the oracle's evolve_2site! + expect."""
    from oracle import chain_oracle as O

    arrays, u = req
    ch = O.from_reference_arrays(arrays)
    O.canonize_(ch)
    O.evolve_2site_(ch, 2, u, threshold=1e-14)
    phi = ch.copy()
    O.evolve_1site_(phi, 2, np.diag([1.0, -1.0]).astype(complex))
    return complex(O.overlap(phi, ch)).real


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    try:
        import bench

        d = bench.Dist(world)
        d.barrier()
        got = {
            "max": d.max(rank + 1.5),
            "sum": d.sum(rank + 1),
            "gather": d.gather([rank] * (rank + 1)),
            "shard": bench.shard(range(7), rank, world),
        }
        reqs = _requests(5)
        mine = bench.shard(list(range(len(reqs))), rank, world)
        vals = [(i, _solve(reqs[i])) for i in mine]
        got["replica"] = d.gather(vals)
        d.barrier()
        d.td.destroy_process_group()
        q.put((rank, got, None))
    except Exception as e:  # report the failure to the parent instead of hanging it
        q.put((rank, None, repr(e)))


def test_replica_path_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        rank, got, err = q.get(timeout=240)
        assert err is None, f"rank {rank}: {err}"
        res[rank] = got
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert res[r]["max"] == 2.5
        assert res[r]["sum"] == 3
        assert res[r]["gather"] == [0, 1, 1]
    # the partition covers every request exactly once
    assert sorted(res[0]["shard"] + res[1]["shard"]) == list(range(7))
    assert not set(res[0]["shard"]) & set(res[1]["shard"])
    # replicas reproduce the single-process results, every rank sees all of them
    sys.path.insert(0, ROOT)
    single = [_solve(r) for r in _requests(5)]
    for r in (0, 1):
        by_index = dict(res[r]["replica"])
        assert sorted(by_index) == list(range(5))
        for i, v in by_index.items():
            assert abs(v - single[i]) <= 1e-12
