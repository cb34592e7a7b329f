"""The allocation-free filter entry point (fsig_filter_noalloc).

It serves callers that cannot allocate device memory when they filter -- a
process that handed all device memory to its own pool allocator, or code that
cannot accept the device-wide synchronisation of cudaFree.  Its candidate
bitmaps live in a fixed device array instead of the engine arena.  This test
calls it through the C ABI twice in a row and checks each result against the
existing fsig_filter (no refinement): candidate flags are exact, so they must
be equal.  The test creates its own engine and device buffers, so it passes in
a fresh process as well as after the other tests.
"""
import numpy as np
import pytest

import fsig_gb300 as F

pytestmark = pytest.mark.gpu


def test_filter_noalloc_matches_filter_twice():
    torch = pytest.importorskip("torch")
    lab = F.gen_labels(50000, 8, "zipf", seed=11)
    g = F.gen_chung_lu(50000, 200000, 2.1, seed=11, labels=lab)
    off, adj = g.csr()
    qs = [F.gen_query(g, n, F.QUERY_DENSE, seed=500 + n, csr=(off, adj)) for n in (5, 9)]
    with F.Engine(0, arena_bytes=1 << 30) as e:
        e.load_graph(g)
        V = e.graph_info()["V"]
        for q, algo in ((qs[0], F.ALGO_GSI), (qs[1], F.ALGO_FUSED)):  # two calls in a row
            want = e.filter(q, algo, refine_iters=0)
            buf = torch.full((q.num_vertices * V,), 7, dtype=torch.uint8, device="cuda:0")
            torch.cuda.synchronize()
            e.filter_noalloc(q, algo, buf.data_ptr())
            got = buf.cpu().numpy().reshape(q.num_vertices, V)
            assert got.sum() > 0
            assert np.array_equal(got, want)


def test_filter_noalloc_absent_label_and_limits():
    """A query label no data vertex carries gives an all-zero row (as
    fsig_filter does); bitmaps over the fixed array's 2^21 words are refused
    with FSIG_EADMISSION, the caller's buffer left as it was; the largest
    label table a loaded graph can have fits."""
    torch = pytest.importorskip("torch")
    lab = F.gen_labels(4000, 6, "uniform", seed=12)
    g = F.gen_rmat(4000, 16000, seed=12, labels=lab)
    # vertex 2's label 999 is absent (a vertex without bitmap words); vertex
    # 0 (label 0, a neighbour of label 1) has candidates
    q = F.Query(np.array([0, 1, 999], np.int32), np.array([[0, 1], [1, 2]], np.uint32))
    with F.Engine(0, arena_bytes=1 << 30) as e:
        e.load_graph(g)
        V = e.graph_info()["V"]
        want = e.filter(q, F.ALGO_GSI, refine_iters=0)
        buf = torch.full((3 * V,), 7, dtype=torch.uint8, device="cuda:0")
        torch.cuda.synchronize()
        e.filter_noalloc(q, F.ALGO_GSI, buf.data_ptr())
        got = buf.cpu().numpy().reshape(3, V)
        assert not got[2].any() and got[0].any()
        assert np.array_equal(got, want)

        # one label class of 2^21 + 64 vertices: a 32-vertex query needs more
        # than 2^21 bitmap words
        big = F.gen_rmat((1 << 21) + 64, 1 << 21, seed=13)
        e.load_graph(big)
        path = F.Query(np.zeros(32, np.int32), np.array([(i, i + 1) for i in range(31)], np.uint32))
        sentinel = torch.full((64,), 0xAB, dtype=torch.uint8, device="cuda:0")
        torch.cuda.synchronize()
        with pytest.raises(F.FsigError) as ei:
            e.filter_noalloc(path, F.ALGO_GSI, sentinel.data_ptr())
        assert ei.value.status == F.EADMISSION
        assert (sentinel.cpu().numpy() == 0xAB).all()

        # the largest label table a loaded graph can have (4096 labels) fits;
        # the engine refuses graphs with more labels when they are loaded
        L = 4096
        labels = np.arange(L, dtype=np.int32)
        edges = np.array([(i, i + 1) for i in range(L - 1)], np.uint32)
        e.load_graph(F.Graph(labels, edges))
        q2 = F.Query(np.array([5, 6], np.int32), np.array([[0, 1]], np.uint32))
        out = torch.full((2 * L,), 0xAB, dtype=torch.uint8, device="cuda:0")
        torch.cuda.synchronize()
        e.filter_noalloc(q2, F.ALGO_GSI, out.data_ptr())
        flags = out.cpu().numpy().reshape(2, L)
        assert np.array_equal(flags, e.filter(q2, F.ALGO_GSI, refine_iters=0))
        assert flags[0, 5] == 1 and flags[1, 6] == 1 and flags.sum() == 2
        with pytest.raises(F.FsigError) as ei:
            e.load_graph(F.Graph(np.arange(L + 1, dtype=np.int32),
                                 np.array([(i, i + 1) for i in range(L)], np.uint32)))
        assert ei.value.status == F.EINVAL
