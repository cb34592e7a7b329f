"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this module.  It checks the product; it is never the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None

u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def _load():
    global _lib
    if _lib is not None:
        return _lib
    path = HERE / "_build" / "liboracle.so"
    if not path.exists():
        from oracle.build import build_oracle
        build_oracle()
    L = C.CDLL(str(path))
    L.orc_read_tve.restype = C.c_void_p
    L.orc_read_tve.argtypes = [C.c_char_p, C.c_int]
    L.orc_plain_sizes.argtypes = [C.c_void_p] + [C.POINTER(C.c_uint32)] * 2 + [C.POINTER(C.c_int32),
                                                                                 C.POINTER(C.c_uint64),
                                                                                 C.POINTER(C.c_uint32)]
    L.orc_plain_to_csr.argtypes = [C.c_void_p, i32p, u32p, u32p]
    L.orc_free.argtypes = [C.c_void_p]
    L.orc_murmur2.restype = C.c_uint32
    L.orc_murmur2.argtypes = [C.c_void_p, C.c_int, C.c_uint32]
    L.orc_fmix64.restype = C.c_uint64
    L.orc_fmix64.argtypes = [C.c_uint64]
    L.orc_build_signature.argtypes = [C.c_uint32, i32p, u32p, u32p, C.c_int, u32p]
    L.orc_pcsr_num_units.restype = C.c_uint32
    L.orc_pcsr_num_units.argtypes = [C.c_int32]
    L.orc_edge_label.restype = C.c_int32
    L.orc_edge_label.argtypes = [C.c_int32, C.c_int32]
    L.orc_pcsr_sizes.argtypes = [C.c_uint32, C.c_int32, i32p, u32p, u32p, u32p, u32p]
    L.orc_build_pcsr.argtypes = [C.c_uint32, C.c_int32, i32p, u32p, u32p, u32p, u32p]
    L.orc_gsi_filter.argtypes = [C.c_uint32, u32p, u32p, u8p]
    L.orc_mmatch_init.argtypes = [C.c_uint32, i32p, u32p, C.c_int32, C.c_uint32, u8p]
    L.orc_simplify.restype = C.c_uint64
    L.orc_simplify.argtypes = [C.c_uint32, u32p, u32p, u32p, u32p]
    L.orc_refine.argtypes = [C.c_uint32, i32p, u32p, u32p, C.c_uint32, u32p, C.c_void_p, C.c_int, u8p]
    L.orc_match.restype = C.c_int
    L.orc_match.argtypes = [C.c_uint32, i32p, u32p, u32p, C.c_uint32, i32p, C.c_uint32, u32p, C.c_void_p, C.c_int,
                            C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), u64p]
    L.orc_k4_pendant.restype = C.c_int
    L.orc_k4_pendant.argtypes = [C.c_uint32, u32p, u32p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    _lib = L
    return L


def read_tve(path, labeled=True):
    """Reference reader + CSR transform: dict with V, E, L, min_degree, labels, offsets, edges."""
    L = _load()
    h = L.orc_read_tve(str(path).encode(), 1 if labeled else 0)
    if not h:
        raise IOError(f"oracle could not read {path}")
    try:
        nv, ne, mind = C.c_uint32(), C.c_uint32(), C.c_uint32()
        nl, nadj = C.c_int32(), C.c_uint64()
        L.orc_plain_sizes(h, C.byref(nv), C.byref(ne), C.byref(nl), C.byref(nadj), C.byref(mind))
        labels = np.zeros(nv.value, np.int32)
        offsets = np.zeros(nv.value + 1, np.uint32)
        edges = np.zeros(max(nadj.value, 1), np.uint32)
        L.orc_plain_to_csr(h, labels, offsets, edges)
        return dict(V=nv.value, E=ne.value, L=nl.value, min_degree=mind.value, labels=labels, offsets=offsets,
                    edges=edges[: nadj.value])
    finally:
        L.orc_free(h)


def fmix64(k):
    return int(_load().orc_fmix64(int(k) & 0xFFFFFFFFFFFFFFFF))


def murmur2_u32(x):
    v = C.c_uint32(int(x) & 0xFFFFFFFF)
    return int(_load().orc_murmur2(C.byref(v), 4, 17))


def signature(labels, offsets, edges, column_oriented=False):
    labels = np.ascontiguousarray(labels, np.int32)
    V = len(labels)
    out = np.zeros(16 * V, np.uint32)
    e = np.ascontiguousarray(edges, np.uint32)
    if e.size == 0:
        e = np.zeros(1, np.uint32)
    _load().orc_build_signature(V, labels, np.ascontiguousarray(offsets, np.uint32), e, 1 if column_oriented else 0, out)
    return out


def pcsr(labels, offsets, edges, num_labels):
    L = _load()
    labels = np.ascontiguousarray(labels, np.int32)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    edges = np.ascontiguousarray(edges, np.uint32)
    if edges.size == 0:
        edges = np.zeros(1, np.uint32)
    V = len(labels)
    U = L.orc_pcsr_num_units(num_labels)
    keys = np.zeros(max(U, 1), np.uint32)
    ne = np.zeros(max(U, 1), np.uint32)
    L.orc_pcsr_sizes(V, num_labels, labels, offsets, edges, keys, ne)
    off_out = np.zeros(max(int(keys[:U].sum()) * 32, 1), np.uint32)
    e_out = np.zeros(max(int(ne[:U].sum()), 1), np.uint32)
    L.orc_build_pcsr(V, num_labels, labels, offsets, edges, off_out, e_out)
    units = []
    ob = eb = 0
    for u in range(U):
        k, m = int(keys[u]), int(ne[u])
        units.append((k, m, off_out[ob: ob + 32 * k].copy(), e_out[eb: eb + m].copy()))
        ob += 32 * k
        eb += m
    return units


def gsi_filter(data_sig_rowmajor, query_sig16):
    V = len(data_sig_rowmajor) // 16
    out = np.zeros(V, np.uint8)
    _load().orc_gsi_filter(V, np.ascontiguousarray(data_sig_rowmajor, np.uint32),
                           np.ascontiguousarray(query_sig16, np.uint32), out)
    return out


def mmatch_init(labels, offsets, label, degree):
    V = len(labels)
    out = np.zeros(V, np.uint8)
    _load().orc_mmatch_init(V, np.ascontiguousarray(labels, np.int32), np.ascontiguousarray(offsets, np.uint32),
                            int(label), int(degree), out)
    return out


def simplify(offsets, edges):
    offsets = np.ascontiguousarray(offsets, np.uint32)
    V = len(offsets) - 1
    e = np.ascontiguousarray(edges, np.uint32)
    if e.size == 0:
        e = np.zeros(1, np.uint32)
    oo = np.zeros(V + 1, np.uint32)
    oe = np.zeros(max(int(offsets[-1]), 1), np.uint32)
    n = _load().orc_simplify(V, offsets, e, oo, oe)
    return oo, oe[:n]


def refine(labels, offsets, edges, qadj_mask, cand, iterations, classes=None):
    """Refined candidate flags; classes[u] groups u's query neighbours
    (None: every vertex its own class, every threshold one)."""
    cand = np.ascontiguousarray(cand, np.uint8).copy()
    n = len(qadj_mask)
    V = len(labels)
    e = np.ascontiguousarray(edges, np.uint32)
    if e.size == 0:
        e = np.zeros(1, np.uint32)
    cls = None if classes is None else np.ascontiguousarray(classes, np.uint32)
    _load().orc_refine(V, np.ascontiguousarray(labels, np.int32), np.ascontiguousarray(offsets, np.uint32), e, n,
                       np.ascontiguousarray(qadj_mask, np.uint32),
                       None if cls is None else cls.ctypes.data_as(C.c_void_p), int(iterations),
                       cand.reshape(-1))
    return cand


def query_signature(qlabels, qadj_mask):
    """Signatures of the query vertices over their distinct neighbours, by the
    data-graph rule (graph_format_transformer.cc:217-262); [n, 16]."""
    n = len(qlabels)
    rows = [[w for w in range(n) if (int(qadj_mask[u]) >> w) & 1] for u in range(n)]
    off = np.zeros(n + 1, np.uint32)
    off[1:] = np.cumsum([len(r) for r in rows])
    adj = np.array([w for r in rows for w in r], np.uint32)
    return signature(qlabels, off, adj).reshape(n, 16)


def refine_classes(qlabels, qadj_mask):
    """Refinement classes: the coarsest partition of the query vertices that
    keeps apart vertices of different (label, degree, signature) and in which
    members of a class have the same multiset of neighbour classes (colour
    refinement to a fixpoint).  classes[u] = the smallest member of u's class."""
    n = len(qlabels)
    sig = query_signature(qlabels, qadj_mask)
    nbrs = [[w for w in range(n) if (int(qadj_mask[u]) >> w) & 1] for u in range(n)]
    key0 = [(int(qlabels[u]), len(nbrs[u]), tuple(int(x) for x in sig[u])) for u in range(n)]
    col = [min(v for v in range(n) if key0[v] == key0[u]) for u in range(n)]
    while True:
        key = [(col[u], tuple(sorted(col[w] for w in nbrs[u]))) for u in range(n)]
        new = [min(v for v in range(n) if key[v] == key[u]) for u in range(n)]
        if new == col:
            return col
        col = new


def match(labels, offsets, edges, qlabels, qedges, order=None, threads=0, seed=None):
    """Count + set hash + per-depth partial-embedding counts (simple data graph)."""
    from fsig_gb300 import HASH_SEED
    seed = HASH_SEED if seed is None else seed
    L = _load()
    qlabels = np.ascontiguousarray(qlabels, np.int32)
    qe = np.ascontiguousarray(np.asarray(qedges, np.uint32).reshape(-1))
    if qe.size == 0:
        qe = np.zeros(2, np.uint32)
        m = 0
    else:
        m = qe.size // 2
    n = len(qlabels)
    e = np.ascontiguousarray(edges, np.uint32)
    if e.size == 0:
        e = np.zeros(1, np.uint32)
    cnt, hsh = C.c_uint64(), C.c_uint64()
    lv = np.zeros(32, np.uint64)
    ordp = None
    if order is not None:
        ordarr = np.ascontiguousarray(order, np.uint32)
        ordp = ordarr.ctypes.data_as(C.c_void_p)
    rc = L.orc_match(len(labels), np.ascontiguousarray(labels, np.int32), np.ascontiguousarray(offsets, np.uint32), e,
                     n, qlabels, m, qe, ordp, int(threads), int(seed), C.byref(cnt), C.byref(hsh), lv)
    if rc != 0:
        raise ValueError(f"oracle rejected the query (code {rc})")
    return cnt.value, hsh.value, lv[:n].copy()


def k4_pendant(offsets, edges, threads=0):
    """(K4 subgraphs, embeddings of K4 plus a pendant) of a simple graph, by
    clique listing and the identity 6 * sum over K4s of sum of (deg - 3)."""
    L = _load()
    off = np.ascontiguousarray(offsets, np.uint32)
    e = np.ascontiguousarray(edges, np.uint32)
    if e.size == 0:
        e = np.zeros(1, np.uint32)
    k4, pend = C.c_uint64(), C.c_uint64()
    rc = L.orc_k4_pendant(len(off) - 1, off, e, int(threads), C.byref(k4), C.byref(pend))
    if rc != 0:
        raise ValueError(f"oracle rejected the graph (code {rc})")
    return k4.value, pend.value


def ref_dump(*args) -> str:
    """Runs the reference-built dump tool (oracle/_ref/ref_dump); None when it was not built."""
    exe = HERE / "_ref" / "ref_dump"
    if not exe.exists():
        return None
    out = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=120)
    if out.returncode != 0:
        raise RuntimeError(f"ref_dump {args} failed ({out.returncode}): {out.stderr[-2000:]}")
    return out.stdout


def parse_dump(text: str) -> dict:
    d = {}
    for line in text.splitlines():
        if line.startswith("@"):
            parts = line.split()
            key = parts[0][1:]
            vals = [int(x) for x in parts[1:]]
            d.setdefault(key, []).append(vals)
    return d

