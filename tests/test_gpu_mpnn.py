"""Order-scoring network on the GPU: forward and backward kernels against the
CPU fp32 reference (tests/mpnn_ref.py), device features against their host
restatement, learned-order results against the heuristic order, and the gain
of a network trained on the engine's own logs."""
import numpy as np
import pytest

import fsig_gb300 as F
import mpnn_ref as R
from conftest import GOLDEN
from fsig_gb300 import learn
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# Forward: BF16 weights and activations on both sides, so the remaining
# difference is FP32 accumulation order and the occasional BF16 rounding that
# lands on the other side of a tie: 2% of the largest |score|.
FWD_TOL = 2e-2
# Gradients: the device rounds the pre-activation gradients to BF16 before the
# weight-gradient products (the reference keeps them FP32): 3% relative L2
# error per parameter block.
GRAD_TOL = 3e-2


def random_graphs(rng, count, max_n=32):
    sizes = rng.integers(1, max_n + 1, count)
    goff = np.zeros(count + 1, np.uint32)
    goff[1:] = np.cumsum(sizes)
    nbr = np.zeros(int(goff[-1]), np.uint32)
    for g, n in enumerate(sizes):
        n = int(n)
        edges = [(i, int(rng.integers(0, i))) for i in range(1, n)]  # spanning tree
        for _ in range(int(rng.integers(0, 2 * n))):
            a, b = rng.integers(0, n, 2)
            if a != b:
                edges.append((int(a), int(b)))
        for a, b in edges:
            nbr[goff[g] + a] |= np.uint32(1 << b)
            nbr[goff[g] + b] |= np.uint32(1 << a)
    feat = rng.random((int(goff[-1]), 8)).astype(np.float32)
    return goff, feat, nbr


def test_param_count():
    assert F.mpnn_param_count() == R.N_PARAMS == learn.N_PARAMS


def test_forward_matches_cpu_reference(engine):
    rng = np.random.default_rng(11)
    goff, feat, nbr = random_graphs(rng, 96)
    p = learn.init_params(3)
    p[R.P_BIN:R.P_WS] = rng.normal(0, 0.1, R.H)
    p[R.P_B:R.P_WOUT] = rng.normal(0, 0.1, R.LAYERS * R.H)
    engine.mpnn_set_params(p)
    assert np.array_equal(engine.mpnn_get_params(), p)
    dev = engine.mpnn_forward(goff, feat, nbr)
    import torch
    ref = R.forward(torch.tensor(p), goff, feat, nbr).numpy()
    scale = np.abs(ref).max()
    assert np.abs(dev - ref).max() <= FWD_TOL * scale, np.abs(dev - ref).max() / scale


def test_gradients_match_cpu_reference(engine):
    rng = np.random.default_rng(12)
    goff, feat, nbr = random_graphs(rng, 80)
    tgt = rng.random(int(goff[-1])).astype(np.float32)
    p = learn.init_params(4)
    p[R.P_B:R.P_WOUT] = rng.normal(0, 0.1, R.LAYERS * R.H)
    engine.mpnn_set_params(p)
    loss, g = engine.mpnn_train_step(goff, feat, nbr, tgt, lr=0.0)
    rloss, rg, _ = R.loss_and_grads(p, goff, feat, nbr, tgt)
    assert abs(loss - rloss) <= 1e-2 * rloss
    for name, sl in R.blocks():
        if name == "w_in":  # padding rows 8..15 have zero gradient on both sides
            assert np.all(g[sl].reshape(16, 64)[8:] == 0)
        err = np.linalg.norm(g[sl] - rg[sl]) / max(np.linalg.norm(rg[sl]), 1e-12)
        assert err <= GRAD_TOL, (name, err)
    # lr = 0 leaves the parameters alone
    assert np.array_equal(engine.mpnn_get_params(), p)


def test_adam_steps_reduce_loss(engine):
    rng = np.random.default_rng(13)
    goff, feat, nbr = random_graphs(rng, 64)
    tgt = feat[:, 2] * 0.5 + feat[:, 1]  # a learnable function of the inputs
    engine.mpnn_set_params(learn.init_params(5))
    first, _ = engine.mpnn_train_step(goff, feat, nbr, tgt, lr=0.0)
    for _ in range(150):
        loss, _ = engine.mpnn_train_step(goff, feat, nbr, tgt, lr=3e-3)
    assert loss < 0.2 * first, (first, loss)


def query_signature_bits(q):
    n = q.num_vertices
    masks = learn.adjacency_masks(q)
    off = np.zeros(n + 1, np.uint32)
    adj = []
    for u in range(n):
        adj += [w for w in range(n) if (int(masks[u]) >> w) & 1]
        off[u + 1] = len(adj)
    sig = O.signature(q.labels, off, np.asarray(adj, np.uint32)).reshape(n, 16)
    return [sum(bin(int(x)).count("1") for x in sig[u, 1:]) for u in range(n)], masks


def golden_graph_and_queries(engine, golden):
    rec = golden["graphs"]["cl_zipf16"]
    g = F.read_graph(GOLDEN / rec["file"], True)
    engine.load_graph(g)
    qs = [F.read_query(GOLDEN / r["file"]) for _, r in sorted(golden["queries"].items())]
    return g, qs


def test_features_match_host(engine, golden):
    g, qs = golden_graph_and_queries(engine, golden)
    res = engine.match_batch(qs, algo=F.ALGO_FUSED)
    cand = [r.candidates for r in res]
    dev = engine.mpnn_features(qs, cand, F.ALGO_FUSED)
    lab = np.asarray(g.labels)
    cls_of = np.bincount(lab[lab >= 0], minlength=int(lab.max()) + 1)
    row = 0
    for q, c, r in zip(qs, cand, res):
        bits, masks = query_signature_bits(q)
        cls = [int(cls_of[l]) if 0 <= l < len(cls_of) else 0 for l in q.labels]
        host = R.features(q.num_vertices, [int(m) for m in masks], bits, c, cls, r.order)
        assert np.array_equal(dev[row:row + q.num_vertices], host)
        row += q.num_vertices


def connected_permutation(order, q):
    masks = learn.adjacency_masks(q)
    return sorted(order) == list(range(q.num_vertices)) and learn.is_connected_order(order, masks)


@pytest.mark.parametrize("algo", [F.ALGO_FSIG, F.ALGO_GSI, F.ALGO_FUSED])
def test_learned_order_results_identical(engine, golden, algo):
    _, qs = golden_graph_and_queries(engine, golden)
    engine.mpnn_set_params(learn.init_params(7))
    heur = engine.match_batch(qs, algo=algo, order_source=F.ORDER_HEURISTIC)
    lrn = engine.match_batch(qs, algo=algo, order_source=F.ORDER_LEARNED)
    for q, h, l in zip(qs, heur, lrn):
        assert (h.status, h.count, h.hash) == (l.status, l.count, l.hash)
        assert connected_permutation(l.order, q)


def test_learned_batch_keeps_given_orders(engine, golden):
    """In a learned-order batch, queries that carry an order keep it."""
    _, qs = golden_graph_and_queries(engine, golden)
    engine.mpnn_set_params(learn.init_params(8))
    heur = engine.match_batch(qs, algo=F.ALGO_FUSED)
    mixed = []
    for i, (q, h) in enumerate(zip(qs, heur)):
        if i % 2 and q.num_vertices > 2:
            mixed.append(F.Query(q.labels, q.edges, order=np.asarray(h.order[::-1] if learn.is_connected_order(
                h.order[::-1], learn.adjacency_masks(q)) else h.order, np.uint32)))
        else:
            mixed.append(q)
    rs = engine.match_batch(mixed, algo=F.ALGO_FUSED, order_source=F.ORDER_LEARNED)
    for q, h, r in zip(mixed, heur, rs):
        assert (r.count, r.hash) == (h.count, h.hash)
        if q.order is not None:
            assert r.order == [int(x) for x in q.order]


def test_learned_order_needs_a_network():
    with F.Engine(0, arena_bytes=1 << 28) as e:
        e.load_graph(F.gen_rmat(1000, 4000, seed=1, labels=F.gen_labels(1000, 4, seed=1)))
        q = F.Query(np.array([0, 1], np.int32), np.array([[0, 1]], np.uint32))
        with pytest.raises(F.FsigError) as ei:
            e.match_batch([q], order_source=F.ORDER_LEARNED)
        assert ei.value.status == F.EINVAL


def test_packaged_network_keeps_results(engine, golden):
    if not learn.WEIGHTS.exists():
        pytest.skip("no packaged order network")
    _, qs = golden_graph_and_queries(engine, golden)
    engine.mpnn_set_params(learn.load_params())
    heur = engine.match_batch(qs, algo=F.ALGO_FUSED)
    lrn, _ = learn.match_learned(engine, qs, work_limit=1 << 40)
    assert [(h.count, h.hash) for h in heur] == [(l.count, l.hash) for l in lrn]


def gain_workload(engine):
    lab = F.gen_labels(100_000, 16, "zipf", seed=21)
    g = F.gen_chung_lu(100_000, 400_000, 2.1, seed=21, labels=lab)
    csr = g.csr()
    engine.load_graph(g)
    rng = np.random.default_rng(21)
    specs = [(int(n), F.QUERY_DENSE if i % 2 else F.QUERY_SPARSE, 9000 + i, 4)
             for i, n in enumerate(rng.integers(8, 21, 2400))]
    cands = F.gen_queries(g, specs, csr=csr)
    return F.select_within_budget(engine, cands, 800, 1 << 22)


def total_work(engine, qs, order_source, cap):
    res = engine.match_batch(qs, algo=F.ALGO_FUSED, order_source=order_source, max_work=cap)
    return sum(r.work if r.status == F.OK else cap for r in res), res


def test_trained_network_gains_over_heuristic(engine):
    """Trained on logs of 400 queries, the network orders the held-out queries
    with less total enumeration work than the heuristic order, and with less
    than the untrained network."""
    qs = gain_workload(engine)
    train_q, test_q = qs[:400], qs[400:]
    logs = learn.collect_logs(engine, train_q, per_query=16, seed=1)
    data = learn.training_set(engine, logs)
    params, losses = learn.train(engine, data, epochs=60, seed=1)
    assert losses[-1] < losses[0]
    cap = 1 << 24
    heur, hres = total_work(engine, test_q, F.ORDER_HEURISTIC, cap)
    lrn, lres = total_work(engine, test_q, F.ORDER_LEARNED, cap)
    for h, l in zip(hres, lres):
        if l.status == F.OK:
            assert (h.count, h.hash) == (l.count, l.hash)
    engine.mpnn_set_params(learn.init_params(1))
    untrained, _ = total_work(engine, test_q, F.ORDER_LEARNED, cap)
    print(f"held-out work: heuristic {heur}, learned {lrn}, untrained {untrained}")
    assert lrn < heur
    assert lrn < untrained
