"""Failure paths, made to happen on the host side and through bounded device
waits; none of them faults, traps or hangs the GPU.

* Admission: a batch larger than what is left of a small arena is refused
  with FSIG_EADMISSION, and the same engine then matches a batch that fits
  with the oracle's results.  The reference has no admission: its memory
  manager ends the process on an allocation failure
  (memory_manager/memory_manager.h:31-61).
* Bounded wait: with fault injection on (fsig_set_queue_waits, unpublished =
  1), the first record handed off in an enumeration pass is written but never
  published; the warp that takes it gives up after a 2 ms limit, the other
  warps abandon the failed pass, and the call returns FSIG_ETIMEOUT within
  milliseconds.  With injection off the same
  engine matches the same batch again, with the results of a run that never
  had injection on.
"""
import time

import numpy as np
import pytest

import fsig_gb300 as F
from fsig_gb300.workloads import pattern
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def path_query(n):
    return F.Query(np.zeros(n, np.int32), np.array([(i, i + 1) for i in range(n - 1)], np.uint32))


def test_oversize_batch_is_refused_then_engine_recovers():
    g = F.gen_rmat(1 << 14, 1 << 17, 0.57, 0.19, 0.19, seed=21)
    off, adj = g.csr()
    # small enough for the oracle (a few million embeddings at most)
    triangle = F.Query(np.zeros(3, np.int32), np.array([[0, 1], [1, 2], [2, 0]], np.uint32))
    small = [triangle, path_query(3), path_query(2)]
    # 512 MiB: the graph store and one small batch (work queues ~310 MiB)
    # fit; 4,000 queries of 32 vertices need ~0.8 GiB of root lists alone
    with F.Engine(0, arena_bytes=512 << 20) as e:
        e.load_graph(g)
        big = [path_query(32)] * 4000
        with pytest.raises(F.FsigError) as ei:
            e.match_batch(big, algo=F.ALGO_FUSED)
        assert ei.value.status == F.EADMISSION
        for use_graph in (False, True):
            with pytest.raises(F.FsigError) as ei:
                e.match_batch(big, algo=F.ALGO_FUSED, use_graph=use_graph)
            assert ei.value.status == F.EADMISSION
            rs = e.match_batch(small, algo=F.ALGO_FUSED, use_graph=use_graph)
            for q, r in zip(small, rs):
                c, h, _ = O.match(g.labels, off, adj, q.labels, q.edges)
                assert (r.status, r.count, r.hash) == (0, c, h)


def test_unpublished_record_times_out_then_engine_recovers():
    g = F.gen_rmat(1 << 9, 1 << 12, 0.57, 0.19, 0.19, seed=3)
    qs = [pattern("house"), pattern("c5")]
    # hand off work often: short ranges, a small cycle budget
    kw = dict(algo=F.ALGO_FUSED, split_cycles=2000, split_len=32, chunk=1)
    with F.Engine(0, arena_bytes=2 << 30) as clean:
        clean.load_graph(g)
        want = [(r.count, r.hash) for r in clean.match_batch(qs, **kw)]
        assert clean.last_stats()["enum_handoffs"] > 0  # the path under test is taken
    with F.Engine(0, arena_bytes=2 << 30) as e:
        e.load_graph(g)
        e.set_queue_waits(ready_wait_ns=2_000_000, unpublished=True)
        statuses, walls = [], []
        for use_graph in (False, True, False):
            t = time.perf_counter()
            try:
                e.match_batch(qs, use_graph=use_graph, **kw)
                statuses.append(F.OK)
            except F.FsigError as err:
                statuses.append(err.status)
            walls.append(time.perf_counter() - t)
        # a hand-off whose record nobody takes in the pass runs in the next
        # pass without waiting; the waiter on it is the expected case
        assert F.ETIMEOUT in statuses, statuses
        assert set(statuses) <= {F.ETIMEOUT, F.OK}
        assert max(w for s, w in zip(statuses, walls) if s == F.ETIMEOUT) < 1.0
        e.set_queue_waits()
        for use_graph in (False, True):
            got = [(r.count, r.hash) for r in e.match_batch(qs, use_graph=use_graph, **kw)]
            assert got == want


def test_queue_wait_arguments_are_checked():
    with F.Engine(0, arena_bytes=1 << 30) as e:
        with pytest.raises(F.FsigError) as ei:
            e.set_queue_waits(ready_wait_ns=61 * 10**9)
        assert ei.value.status == F.EINVAL
        with pytest.raises(F.FsigError):
            e._check(e._L.fsig_set_queue_waits(e._h, 0, 0, 2), "set_queue_waits")
