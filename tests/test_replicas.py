"""The replica path of bench.py (one process per GPU, no data-path collective): the timing
reduction over ranks, run as two gloo ranks on the CPU."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w, local)
    d.barrier()
    slowest = d.max(1.0 + r)          # each rank's own time; the job's time is the slowest
    d.barrier()
    d.close()
    out.put((r, w, slowest))


def test_replica_timing_takes_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 2.0), (1, 2, 2.0)]


def _shard_rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    from graphyt_gb300 import scenes
    r, w, local = bench.dist_env()
    d = bench.Dist(w, local)
    sc = scenes.impact_batch(n_inst=12, seed=3, n_min=2000, n_max=6000, shard=(r, w))
    total = d.sum(float(sc.n))
    d.barrier()
    d.close()
    out.put((r, sorted(i.index for i in sc.instances), sc.n, total, sc.dt))


def test_batch_instances_shard_across_ranks():
    """The batch workload splits its instances across ranks (instance i on rank i mod N):
    two gloo ranks hold disjoint shares that together are the whole batch, with the whole
    batch's dt, and the job's particle count is the sum of the shares."""
    torch = pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    from graphyt_gb300 import scenes
    whole = scenes.impact_batch(n_inst=12, seed=3, n_min=2000, n_max=6000)
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, i0, n0, t0, dt0), (r1, i1, n1, t1, dt1) = res
    assert i0 == list(range(0, 12, 2)) and i1 == list(range(1, 12, 2))
    assert n0 + n1 == whole.n and t0 == t1 == float(whole.n)
    assert dt0 == dt1 == whole.dt
    for r, idx in ((0, i0), (1, i1)):
        for i in idx:
            own = scenes.batch_instance(scenes.impact_batch(n_inst=12, seed=3, n_min=2000, n_max=6000,
                                                            shard=(r, 2)), i)
            ref = scenes.batch_instance(whole, i)
            # the same instance (positions to the rounding of the box offsets; the particle
            # order follows each batch's own shuffle)
            a = own.pos[np.lexsort(np.round(own.pos, 9).T)]
            b = ref.pos[np.lexsort(np.round(ref.pos, 9).T)]
            assert np.allclose(a, b, rtol=0, atol=1e-12) and own.materials == ref.materials
