"""CPU fp32 reference of the order-scoring network (torch), used to check the
device forward and backward kernels.  BF16 rounding is applied at the points
where the device rounds (weights, inputs, hidden states, neighbour means), as a
straight-through operation, so the comparison measures the kernels and not the
number format.  Test infrastructure only."""
import numpy as np
import torch

F_IN, F_PAD, H, LAYERS = 8, 16, 64, 3
P_WIN = 0
P_BIN = P_WIN + F_PAD * H
P_WS = P_BIN + H
P_WN = P_WS + LAYERS * H * H
P_B = P_WN + LAYERS * H * H
P_WOUT = P_B + LAYERS * H
P_BOUT = P_WOUT + H
N_PARAMS = P_BOUT + 1


def bf(x):
    return x + (x.to(torch.bfloat16).to(torch.float32) - x).detach()


def unpack(p):
    return dict(
        w_in=p[P_WIN:P_BIN].view(F_PAD, H),
        b_in=p[P_BIN:P_WS],
        w_s=p[P_WS:P_WN].view(LAYERS, H, H),
        w_n=p[P_WN:P_B].view(LAYERS, H, H),
        b=p[P_B:P_WOUT].view(LAYERS, H),
        w_out=p[P_WOUT:P_BOUT],
        b_out=p[P_BOUT],
    )


def forward(params, goff, feat, nbr):
    """Scores of every node; params is a torch fp32 tensor (may require grad)."""
    W = unpack(params)
    w_in, w_s, w_n = bf(W["w_in"]), bf(W["w_s"]), bf(W["w_n"])
    feat = torch.as_tensor(np.asarray(feat, np.float32)).view(-1, F_IN)
    out = []
    for g in range(len(goff) - 1):
        a, b = int(goff[g]), int(goff[g + 1])
        n = b - a
        if n == 0:
            continue
        x = torch.zeros(n, F_PAD)
        x[:, :F_IN] = feat[a:b]
        x = bf(x)
        A = torch.zeros(n, n)
        for i in range(n):
            m = int(nbr[a + i])
            for j in range(n):
                if (m >> j) & 1:
                    A[i, j] = 1.0
        deg = A.sum(1)
        inv = torch.where(deg > 0, 1.0 / deg.clamp(min=1), torch.zeros_like(deg))
        h = bf(torch.relu(x @ w_in + W["b_in"]))
        for l in range(LAYERS):
            m = bf((A @ h) * inv[:, None])
            h = bf(torch.relu(h @ w_s[l] + m @ w_n[l] + W["b"][l]))
        out.append(h @ W["w_out"] + W["b_out"])
    return torch.cat(out) if out else torch.zeros(0)


def loss_and_grads(params_np, goff, feat, nbr, targets):
    p = torch.tensor(np.asarray(params_np, np.float32), requires_grad=True)
    s = forward(p, goff, feat, nbr)
    t = torch.as_tensor(np.asarray(targets, np.float32))
    loss = ((s - t) ** 2).mean()
    loss.backward()
    return float(loss), p.grad.numpy().copy(), s.detach().numpy()


def blocks():
    """(name, slice) of each parameter block."""
    return [("w_in", slice(P_WIN, P_BIN)), ("b_in", slice(P_BIN, P_WS)), ("w_s", slice(P_WS, P_WN)),
            ("w_n", slice(P_WN, P_B)), ("b", slice(P_B, P_WOUT)), ("w_out", slice(P_WOUT, P_BOUT)),
            ("b_out", slice(P_BOUT, N_PARAMS))]


def plog2(x):
    """e + x / 2^e - 1 with e = floor(log2 x), in float32; 0 for x = 0."""
    x = int(x)
    if x == 0:
        return np.float32(0)
    e = x.bit_length() - 1
    return np.float32(np.float32(e) + (np.float32(x) / np.float32(1 << e) - np.float32(1)))


def features(n, adj_masks, sig_bits, cand, class_size, order):
    """Host restatement of the device feature kernel for one query (float32,
    same operation order); order is the heuristic order."""
    f32 = np.float32
    out = np.zeros((n, F_IN), np.float32)
    for u in range(n):
        deg = bin(adj_masks[u]).count("1")
        nsum = f32(0)
        for w in range(n):
            if (adj_masks[u] >> w) & 1:
                nsum = f32(nsum + plog2(cand[w]))
        cls = class_size[u]
        pos = list(order).index(u)
        out[u] = [(f32(pos) / f32(n - 1)) if n > 1 else f32(0), f32(deg) / f32(8), plog2(cand[u]) / f32(20),
                  plog2(cls) / f32(20), (f32(cand[u]) / f32(cls)) if cls else f32(0), f32(sig_bits[u]) / f32(16),
                  f32(n) / f32(32), (nsum / f32(20 * deg)) if deg else f32(0)]
    return out
