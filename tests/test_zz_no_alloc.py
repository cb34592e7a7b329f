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
