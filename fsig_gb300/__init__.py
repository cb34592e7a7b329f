"""fsig_gb300: a GB300-native subgraph-matching engine behind FSIG's interface.

The engine is libfsig.so (hand-written sm_103a CUDA behind the C ABI in
include/fsig.h); this module binds it with ctypes and mirrors the reference's
host-side interface:

  UndirectedSurveyPlainReader.read  -> read_graph(path, is_labeled)   (IO/graph_reader.h:27-34)
  GPUSubgraphMatcher / MMatch / GSI -> MMatch(query, data).match(), GSI(...).match()
                                       (match/subgraph_match.h:39-81, MMatch.h:75, GSI.h:47)
  GraphFormatTransformer.transform   -> Engine.build_csr / Engine.build_signature

There is no CPU fallback: when libfsig.so is missing or no sm_103 device is
present, Engine() raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
_BUILD = _PKG / "_build"

HASH_SEED = 0x46534947B3000001
MAX_QUERY = 32

OK, EINVAL, ENODEV, ECUDA, EADMISSION, ENOGRAPH, EQUERY, EIO, ETIMEOUT, EOVERFLOW, ELIMIT = (
    0, -1, -2, -3, -4, -5, -6, -7, -8, -9, -10)
ALGO_FSIG, ALGO_GSI, ALGO_FUSED = 1, 2, 3
ORDER_HEURISTIC, ORDER_LEARNED, ORDER_GIVEN = 0, 1, 2
SEGMENTS_AUTO, SEGMENTS_TABLE, SEGMENTS_ROWS = 0, 1, 2
QUERY_INDUCED, QUERY_DENSE, QUERY_SPARSE = 0, 1, 2


class FsigError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class _Query(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint32), ("labels", C.POINTER(C.c_int32)),
                ("edges", C.POINTER(C.c_uint32)), ("order", C.POINTER(C.c_uint32))]


class _Result(C.Structure):
    _fields_ = [("count", C.c_uint64), ("hash", C.c_uint64), ("status", C.c_int32), ("num_vertices", C.c_uint32),
                ("order", C.c_uint32 * MAX_QUERY), ("candidates", C.c_uint32 * MAX_QUERY),
                ("level_counts", C.c_uint64 * MAX_QUERY), ("ms_filter", C.c_float), ("ms_join", C.c_float),
                ("work", C.c_uint64)]


class _BatchOpts(C.Structure):
    _fields_ = [("algo", C.c_int), ("order_source", C.c_int), ("refine_iters", C.c_int), ("use_graph", C.c_int),
                ("chunk", C.c_uint32), ("split_len", C.c_uint32), ("split_cycles", C.c_uint64),
                ("max_work", C.c_uint64), ("warps_per_block", C.c_uint32), ("learned_window", C.c_uint32),
                ("no_classes", C.c_uint32), ("isect", C.c_uint32), ("refine_coop", C.c_uint32),
                ("learned_prefix", C.c_uint32)]


class _Stats(C.Structure):
    _fields_ = [("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("enum_bytes", C.c_uint64),
                ("kernel_launches", C.c_uint32), ("enum_passes", C.c_uint32), ("ms_filter", C.c_float),
                ("ms_join", C.c_float), ("ms_enum", C.c_float), ("graph", C.c_uint32), ("enum_tasks", C.c_uint64),
                ("enum_pops", C.c_uint64), ("enum_handoffs", C.c_uint64), ("enum_records", C.c_uint64),
                ("enum_examines", C.c_uint64)]


_eng = None
_gen = None


def _u32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _i32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


_SINK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint32), C.c_uint64, C.c_uint32)
MPNN_FEATURES = 8


def mpnn_param_count() -> int:
    return int(engine_library().fsig_mpnn_param_count())


def engine_library() -> C.CDLL:
    """Loads libfsig.so (built in-tree by fsig_gb300._build); raises if absent."""
    global _eng
    if _eng is not None:
        return _eng
    path = _BUILD / "libfsig.so"
    if not path.exists():
        raise FsigError(ENODEV, f"{path} is missing: build it with fsig_gb300._build.build_all()")
    L = C.CDLL(str(path))
    vp = C.c_void_p
    L.fsig_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(vp)]
    L.fsig_destroy.argtypes = [vp]
    L.fsig_last_error.restype = C.c_char_p
    L.fsig_last_error.argtypes = [vp]
    L.fsig_status_string.restype = C.c_char_p
    L.fsig_status_string.argtypes = [C.c_int]
    L.fsig_load_graph.argtypes = [vp, C.c_uint32, C.POINTER(C.c_int32), C.c_uint64, C.POINTER(C.c_uint32)]
    L.fsig_load_graph_file.argtypes = [vp, C.c_char_p, C.c_int]
    L.fsig_graph_info.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_uint32)]
    L.fsig_match.argtypes = [vp, C.POINTER(_Query), C.c_int, C.POINTER(_Result)]
    L.fsig_match_batch.argtypes = [vp, C.c_uint32, C.POINTER(_Query), C.POINTER(_BatchOpts), C.POINTER(_Result)]
    L.fsig_build_csr.argtypes = [vp, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                 C.POINTER(C.c_uint32)]
    L.fsig_build_signature.argtypes = [vp, C.c_uint32, C.POINTER(C.c_int32), C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint32), C.c_int, C.POINTER(C.c_uint32)]
    L.fsig_filter.argtypes = [vp, C.POINTER(_Query), C.c_int, C.c_int, C.POINTER(C.c_uint8)]
    L.fsig_filter_classes.argtypes = [vp, C.POINTER(_Query), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint8)]
    u32p = C.POINTER(C.c_uint32)
    L.fsig_refine_classes.argtypes = [C.POINTER(_Query), u32p, u32p]
    L.fsig_build_pcsr.argtypes = [vp, C.c_uint32, C.c_int32, C.POINTER(C.c_int32), u32p, u32p, u32p, u32p, u32p, u32p]
    L.fsig_plan_order.argtypes = [C.POINTER(_Query), C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.fsig_last_stats.argtypes = [vp, C.POINTER(_Stats)]
    L.fsig_filter_noalloc.argtypes = [vp, C.POINTER(_Query), C.c_int, C.c_void_p]
    L.fsig_set_queue_waits.argtypes = [vp, C.c_uint64, C.c_uint64, C.c_int]
    L.fsig_set_segment_index.argtypes = [vp, C.c_int]
    L.fsig_graph_layout.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]
    L.fsig_match_range.argtypes = [vp, C.POINTER(_Query), C.c_int, C.c_uint32, C.c_uint32, C.c_uint32,
                                   C.POINTER(_Result), C.POINTER(C.c_uint32)]
    fp = C.POINTER(C.c_float)
    L.fsig_mpnn_param_count.restype = C.c_uint32
    L.fsig_mpnn_param_count.argtypes = []
    L.fsig_mpnn_set_params.argtypes = [vp, fp, C.c_uint32]
    L.fsig_mpnn_get_params.argtypes = [vp, fp, C.c_uint32]
    L.fsig_mpnn_features.argtypes = [vp, C.c_uint32, C.POINTER(_Query), C.c_int, C.POINTER(C.c_uint32), fp]
    L.fsig_mpnn_forward.argtypes = [vp, C.c_uint32, C.POINTER(C.c_uint32), fp, C.POINTER(C.c_uint32), fp]
    L.fsig_mpnn_train_step.argtypes = [vp, C.c_uint32, C.POINTER(C.c_uint32), fp, C.POINTER(C.c_uint32), fp,
                                       C.c_float, fp, fp]
    L.fsig_read_graph_file.argtypes = [C.c_char_p, C.c_int, C.POINTER(vp)]
    L.fsig_graph_file_data.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.POINTER(C.c_int32)),
                                       C.POINTER(C.c_uint64), C.POINTER(C.POINTER(C.c_uint32))]
    L.fsig_save_graph_cache.argtypes = [vp, C.c_char_p]
    L.fsig_load_graph_cache.argtypes = [vp, C.c_char_p]
    L.fsig_read_graph_file_threads.argtypes = [C.c_char_p, C.c_int, C.c_uint64, C.POINTER(vp)]
    L.fsig_free_graph_file.argtypes = [vp]
    L.fsig_free_graph_file.restype = None
    L.fsig_match_embeddings.argtypes = [vp, C.POINTER(_Query), C.c_int, C.c_uint64, _SINK, vp, C.POINTER(_Result)]
    L.fsig_write_embeddings.argtypes = [vp, C.POINTER(_Query), C.c_int, C.c_char_p, C.POINTER(_Result)]
    for name in ("fsig_mpnn_set_params", "fsig_mpnn_get_params", "fsig_mpnn_features", "fsig_mpnn_forward",
                 "fsig_mpnn_train_step", "fsig_read_graph_file", "fsig_read_graph_file_threads", "fsig_save_graph_cache", "fsig_load_graph_cache", "fsig_graph_file_data", "fsig_match_embeddings",
                 "fsig_write_embeddings", "fsig_build_pcsr", "fsig_filter_noalloc", "fsig_set_queue_waits", "fsig_set_segment_index", "fsig_graph_layout", "fsig_match_range", "fsig_last_stats", "fsig_plan_order", "fsig_create", "fsig_destroy", "fsig_load_graph", "fsig_load_graph_file", "fsig_graph_info",
                 "fsig_match", "fsig_match_batch", "fsig_build_csr", "fsig_build_signature", "fsig_filter",
                 "fsig_filter_classes", "fsig_refine_classes"):
        getattr(L, name).restype = C.c_int
    _eng = L
    return L


_gen_path = None


def use_generator_library(path) -> None:
    """Binds the workload generators to another build of csrc/gen.cpp (the
    CPU benchmark arm uses the copy oracle/build.py makes, so that it loads
    none of this package's libraries).  Call before the first generator."""
    global _gen, _gen_path
    if _gen is not None and Path(path) != _gen_path:
        raise RuntimeError("the generator library is already loaded")
    _gen_path = Path(path)


def gen_library() -> C.CDLL:
    global _gen, _gen_path
    if _gen is not None:
        return _gen
    path = _gen_path or _BUILD / "libfsig_gen.so"
    if _gen_path is None and not path.exists():
        from . import _build
        _build.build_gen()
    _gen_path = path
    L = C.CDLL(str(path))
    L.fsig_gen_rmat.argtypes = [C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int,
                                C.POINTER(C.c_uint32)]
    L.fsig_gen_chung_lu.argtypes = [C.c_uint32, C.c_uint64, C.c_double, C.c_uint64, C.c_int, C.POINTER(C.c_uint32)]
    L.fsig_gen_labels_uniform.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(C.c_int32)]
    L.fsig_gen_labels_zipf.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_uint64, C.POINTER(C.c_int32)]
    L.fsig_gen_csr.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                               C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]
    L.fsig_gen_query.argtypes = [C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_int32),
                                 C.c_uint32, C.c_int, C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_uint32),
                                 C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.fsig_gen_query_ex.argtypes = [C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_int32),
                                    C.c_uint32, C.c_int, C.c_uint64, C.c_int32, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.fsig_write_tve.argtypes = [C.c_char_p, C.c_uint32, C.POINTER(C.c_int32), C.c_uint64, C.POINTER(C.c_uint32)]
    _gen = L
    return L


# ---------------------------------------------------------------------------
# graphs and queries
# ---------------------------------------------------------------------------
@dataclass
class Graph:
    """A data graph: labels[V] and an undirected edge list edges[E, 2]."""
    labels: np.ndarray
    edges: np.ndarray

    @property
    def num_vertices(self) -> int:
        return int(len(self.labels))

    @property
    def num_edges(self) -> int:
        return int(len(self.edges))

    def csr(self):
        """Simple CSR (rows ascending, duplicates and self-loops dropped): (offsets, adj)."""
        V = self.num_vertices
        e = np.ascontiguousarray(self.edges, np.uint32).reshape(-1)
        off = np.zeros(V + 1, np.uint32)
        adj = np.zeros(max(2 * self.num_edges, 1), np.uint32)
        n = C.c_uint64()
        rc = gen_library().fsig_gen_csr(V, self.num_edges, _u32p(e), _u32p(off), _u32p(adj), C.byref(n))
        if rc:
            raise FsigError(rc, "csr build failed")
        return off, adj[: n.value]

    def write_tve(self, path) -> None:
        lab = np.ascontiguousarray(self.labels, np.int32)
        e = np.ascontiguousarray(self.edges, np.uint32).reshape(-1)
        rc = gen_library().fsig_write_tve(str(path).encode(), self.num_vertices, _i32p(lab), self.num_edges, _u32p(e))
        if rc:
            raise FsigError(rc, f"cannot write {path}")


@dataclass
class Query:
    """A query graph: n <= 32 vertices with labels, undirected edges (m, 2)."""
    labels: np.ndarray
    edges: np.ndarray
    order: np.ndarray | None = None
    source: np.ndarray | None = None  # data vertices it was extracted from (an embedding)

    @property
    def num_vertices(self) -> int:
        return int(len(self.labels))

    def write_tve(self, path) -> None:
        Graph(np.asarray(self.labels, np.int32), np.asarray(self.edges, np.uint32).reshape(-1, 2)).write_tve(path)


@dataclass
class Result:
    count: int
    hash: int
    status: int
    order: list
    candidates: list
    level_counts: list
    ms_filter: float = 0.0
    ms_join: float = 0.0
    work: int = 0


def read_graph_native(path, is_labeled: bool = True, parallel_min_bytes: int = 0) -> Graph:
    """The C++ reader (fsig_read_graph_file_threads): labels (-1 for ids
    without a v record) and the edge list in file order, duplicates kept.
    Needs no GPU."""
    L = engine_library()
    h = C.c_void_p()
    rc = L.fsig_read_graph_file_threads(str(path).encode(), 1 if is_labeled else 0, parallel_min_bytes, C.byref(h))
    if rc:
        raise FsigError(rc, f"cannot read {path}: {L.fsig_last_error(None).decode()}")
    try:
        V, E = C.c_uint32(), C.c_uint64()
        lab, edg = C.POINTER(C.c_int32)(), C.POINTER(C.c_uint32)()
        L.fsig_graph_file_data(h, C.byref(V), C.byref(lab), C.byref(E), C.byref(edg))
        labels = np.ctypeslib.as_array(lab, shape=(V.value,)).copy() if V.value else np.zeros(0, np.int32)
        edges = (np.ctypeslib.as_array(edg, shape=(2 * E.value,)).copy() if E.value else np.zeros(0, np.uint32))
    finally:
        L.fsig_free_graph_file(h)
    return Graph(labels, edges.reshape(-1, 2))


def read_graph(path, is_labeled: bool = True) -> Graph:
    """Host reader with the reference's semantics (IO/graph_reader.cc:12-55),
    returning the edge list (duplicates kept) and labels."""
    labels, edges = [], []
    vmax = -1
    lab = {}
    text = Path(path).read_text()
    toks = text.split()
    if not toks or toks[0] != "t":
        raise FsigError(EIO, f"{path}: not a t/v/e file")
    i = 3
    while i < len(toks):
        t = toks[i]
        if t == "v":
            vid, l = int(toks[i + 1]), int(toks[i + 2])
            lab[vid] = l if is_labeled else 0
            vmax = max(vmax, vid)
            i += 4
        elif t == "e":
            edges.append((int(toks[i + 1]), int(toks[i + 2])))
            i += 3
        else:
            i += 1
    if text and text[-1].isspace() and toks and edges and toks[-3] == "e":
        edges.append(edges[-1])  # the reference's loop applies its last record twice
    labels = np.full(vmax + 1, -1, np.int32)
    for k, v in lab.items():
        labels[k] = v
    return Graph(labels, np.asarray(edges, np.uint32).reshape(-1, 2))


def read_query(path, is_labeled: bool = True) -> Query:
    g = read_graph(path, is_labeled)
    return Query(g.labels, g.edges)


# ---------------------------------------------------------------------------
# generators (seeded synthetic workloads)
# ---------------------------------------------------------------------------
def gen_rmat(V: int, E: int, a=0.57, b=0.19, c=0.19, seed=1, labels=None, threads=0) -> Graph:
    e = np.zeros(2 * E, np.uint32)
    rc = gen_library().fsig_gen_rmat(V, E, a, b, c, seed, threads, _u32p(e))
    if rc:
        raise FsigError(rc, "R-MAT generation failed")
    lab = np.zeros(V, np.int32) if labels is None else labels
    return Graph(lab, e.reshape(-1, 2))


def gen_chung_lu(V: int, E: int, gamma: float, seed=2, labels=None, threads=0) -> Graph:
    e = np.zeros(2 * E, np.uint32)
    rc = gen_library().fsig_gen_chung_lu(V, E, gamma, seed, threads, _u32p(e))
    if rc:
        raise FsigError(rc, "Chung-Lu generation failed")
    lab = np.zeros(V, np.int32) if labels is None else labels
    return Graph(lab, e.reshape(-1, 2))


def gen_labels(V: int, L: int, dist: str = "uniform", seed=1, s: float = 1.0) -> np.ndarray:
    lab = np.zeros(V, np.int32)
    if dist == "uniform":
        rc = gen_library().fsig_gen_labels_uniform(V, L, seed, _i32p(lab))
    else:
        rc = gen_library().fsig_gen_labels_zipf(V, L, s, seed, _i32p(lab))
    if rc:
        raise FsigError(rc, "label generation failed")
    return lab


def gen_query(g: Graph, n: int, mode: int = QUERY_INDUCED, seed: int = 1, csr=None, min_label: int = None) -> Query:
    off, adj = csr if csr is not None else g.csr()
    lab = np.ascontiguousarray(g.labels, np.int32)
    ql = np.zeros(n, np.int32)
    qe = np.zeros(n * (n - 1), np.uint32)
    m = C.c_uint32()
    src = np.zeros(n, np.uint32)
    adj = np.ascontiguousarray(adj if len(adj) else np.zeros(1, np.uint32), np.uint32)
    if min_label is None:
        rc = gen_library().fsig_gen_query(g.num_vertices, _u32p(off), _u32p(adj), _i32p(lab), n, mode, seed,
                                          _i32p(ql), _u32p(qe), C.byref(m), _u32p(src))
    else:
        rc = gen_library().fsig_gen_query_ex(g.num_vertices, _u32p(off), _u32p(adj), _i32p(lab), n, mode, seed,
                                             int(min_label), _i32p(ql), _u32p(qe), C.byref(m), _u32p(src))
    if rc:
        raise FsigError(rc, f"query extraction gave up (n={n}, mode={mode}, seed={seed})")
    return Query(ql, qe[: 2 * m.value].reshape(-1, 2).copy(), source=src)


def gen_queries(g: Graph, specs, csr=None, threads: int = 0) -> list:
    """Many queries at once: specs is a list of (n, mode, seed); extraction
    runs on host threads (the generator library releases the GIL)."""
    import concurrent.futures as cf
    import os
    csr = csr if csr is not None else g.csr()
    threads = threads or min(32, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(lambda s: gen_query(g, s[0], s[1], s[2], csr=csr,
                                               min_label=s[3] if len(s) > 3 else None), specs))


# ---------------------------------------------------------------------------
# engine
# ---------------------------------------------------------------------------
def _as_cquery(q: Query, keep: list) -> _Query:
    lab = np.ascontiguousarray(q.labels, np.int32)
    e = np.ascontiguousarray(np.asarray(q.edges, np.uint32).reshape(-1))
    keep += [lab, e]
    cq = _Query(len(lab), len(e) // 2, _i32p(lab), _u32p(e) if e.size else None, None)
    if q.order is not None:
        o = np.ascontiguousarray(q.order, np.uint32)
        keep.append(o)
        cq.order = _u32p(o)
    return cq


_QUERY_DTYPE = np.dtype({"names": ["nv", "ne", "labels", "edges", "order"],
                          "formats": ["<u4", "<u4", "<u8", "<u8", "<u8"],
                          "offsets": [0, 4, 8, 16, 24], "itemsize": 32})


def _pack_queries(qs: Sequence[Query]):
    """fsig_query[len(qs)] for a batch, built with a few array operations: the
    labels, edges and orders of all queries in three arrays, the structs as one
    structured array pointing into them.  Returns (pointer, arrays to keep)."""
    n = len(qs)
    for i, q in enumerate(qs):
        # each order pointer is placed by its query's vertex count
        if q.order is not None and np.asarray(q.order).size != np.asarray(q.labels).size:
            raise ValueError(f"query {i}: an order of {np.asarray(q.order).size} vertices for "
                             f"{np.asarray(q.labels).size} query vertices")
    labs = [np.asarray(q.labels, np.int32).reshape(-1) for q in qs]
    eds = [np.asarray(q.edges, np.uint32).reshape(-1) for q in qs]
    ords = [np.asarray(q.order, np.uint32).reshape(-1) for q in qs if q.order is not None]
    lab = np.ascontiguousarray(np.concatenate(labs) if n else np.zeros(0, np.int32), np.int32)
    edg = np.ascontiguousarray(np.concatenate(eds) if n else np.zeros(0, np.uint32), np.uint32)
    ordv = np.ascontiguousarray(np.concatenate(ords) if ords else np.zeros(0, np.uint32), np.uint32)
    nv = np.fromiter((len(x) for x in labs), np.uint64, n)
    ne2 = np.fromiter((len(x) for x in eds), np.uint64, n)
    arr = np.zeros(max(n, 1), _QUERY_DTYPE)
    if n:
        arr["nv"][:n] = nv
        arr["ne"][:n] = ne2 // 2
        lo = np.concatenate([[0], np.cumsum(nv)[:-1]]).astype(np.uint64)
        eo = np.concatenate([[0], np.cumsum(ne2)[:-1]]).astype(np.uint64)
        arr["labels"][:n] = np.uint64(lab.ctypes.data) + 4 * lo
        arr["edges"][:n] = np.where(ne2 > 0, np.uint64(edg.ctypes.data) + 4 * eo, 0)
        has = np.fromiter((q.order is not None for q in qs), bool, n)
        if has.any():
            oo = np.concatenate([[0], np.cumsum(np.where(has, nv, 0))[:-1]]).astype(np.uint64)
            arr["order"][:n] = np.where(has, np.uint64(ordv.ctypes.data) + 4 * oo, 0)
    return arr.ctypes.data_as(C.POINTER(_Query)), (arr, lab, edg, ordv)


def _result(r: _Result) -> Result:
    n = r.num_vertices
    return Result(int(r.count), int(r.hash), int(r.status), list(r.order[:n]), list(r.candidates[:n]),
                  [int(x) for x in r.level_counts[:n]], float(r.ms_filter), float(r.ms_join), int(r.work))


class Engine:
    """One device arena on one GPU; replaces init_GPU + MemoryManager."""

    def __init__(self, device: int = 0, arena_bytes: int = 0):
        self._L = engine_library()
        h = C.c_void_p()
        rc = self._L.fsig_create(device, arena_bytes, C.byref(h))
        if rc:
            raise FsigError(rc, "fsig_create: " + self._L.fsig_last_error(None).decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.fsig_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int, what: str):
        if rc:
            raise FsigError(rc, f"{what}: {self._L.fsig_last_error(self._h).decode()}")

    # data graph
    def load_graph(self, g: Graph) -> None:
        lab = np.ascontiguousarray(g.labels, np.int32)
        e = np.ascontiguousarray(g.edges, np.uint32).reshape(-1)
        if e.size == 0:
            e = np.zeros(2, np.uint32)
        self._check(self._L.fsig_load_graph(self._h, len(lab), _i32p(lab), g.num_edges, _u32p(e)), "load_graph")

    def load_graph_file(self, path, is_labeled: bool = True) -> None:
        self._check(self._L.fsig_load_graph_file(self._h, str(path).encode(), 1 if is_labeled else 0),
                    "load_graph_file")

    def save_graph_cache(self, path) -> None:
        self._check(self._L.fsig_save_graph_cache(self._h, str(path).encode()), "save_graph_cache")

    def load_graph_cache(self, path) -> None:
        self._check(self._L.fsig_load_graph_cache(self._h, str(path).encode()), "load_graph_cache")

    def set_segment_index(self, mode: int = SEGMENTS_AUTO) -> None:
        """Segment index of the graphs loaded from now on: SEGMENTS_TABLE (a
        dense V x (L+1) table, one load per lookup), SEGMENTS_ROWS (no table,
        binary search in the row) or SEGMENTS_AUTO (the table when it takes at
        most 4 words per adjacency entry).  Results do not depend on it."""
        self._check(self._L.fsig_set_segment_index(self._h, int(mode)), "set_segment_index")

    def graph_layout(self) -> dict:
        """The resident store's segment index and its device bytes."""
        mode, nbytes = C.c_int(), C.c_uint64()
        self._check(self._L.fsig_graph_layout(self._h, C.byref(mode), C.byref(nbytes)), "graph_layout")
        return dict(segment_index=mode.value, bytes=nbytes.value)

    def graph_info(self) -> dict:
        V, nadj, L, md = C.c_uint32(), C.c_uint64(), C.c_int32(), C.c_uint32()
        self._check(self._L.fsig_graph_info(self._h, C.byref(V), C.byref(nadj), C.byref(L), C.byref(md)),
                    "graph_info")
        return dict(V=V.value, adj=nadj.value, L=L.value, max_degree=md.value)

    # matching
    def match(self, q: Query, algo: int = ALGO_FSIG) -> Result:
        keep = []
        cq = _as_cquery(q, keep)
        r = _Result()
        self._check(self._L.fsig_match(self._h, C.byref(cq), algo, C.byref(r)), "match")
        return _result(r)

    def match_batch(self, qs: Sequence[Query], algo: int = ALGO_FUSED, order_source: int = ORDER_HEURISTIC,
                    refine_iters: int = -1, chunk: int = 0, use_graph: bool = False, split_len: int = 0,
                    split_cycles: int = 0, max_work: int = 0, warps_per_block: int = 0,
                    learned_window: int = 0, classes: bool = True, isect: int = 0, refine_coop: int = 0,
                    learned_prefix: int = 0) -> list:
        arr, keep = _pack_queries(qs)
        res = (_Result * max(len(qs), 1))()
        opts = _BatchOpts(algo, order_source, refine_iters, 1 if use_graph else 0, chunk, split_len, split_cycles,
                          max_work, warps_per_block, learned_window, 0 if classes else 1, isect, refine_coop,
                          learned_prefix)
        self._check(self._L.fsig_match_batch(self._h, len(qs), arr, C.byref(opts), res), "match_batch")
        return [_result(res[i]) for i in range(len(qs))]

    def set_queue_waits(self, ready_wait_ns: int = 0, idle_wait_ns: int = 0, unpublished: bool = False) -> None:
        """Bounded waits of the enumeration's work queue (0: defaults, 200 ms
        and 2 s); unpublished=True leaves each pass's first handed-off record
        unpublished (fault injection for tests: the call returns ETIMEOUT)."""
        self._check(self._L.fsig_set_queue_waits(self._h, int(ready_wait_ns), int(idle_wait_ns), int(unpublished)),
                    "set_queue_waits")

    def match_range(self, q: Query, algo: int = ALGO_FSIG, task_begin: int = 0, task_end: int = 0xFFFFFFFF,
                    split_len: int = 0):
        """Count and hash of the query over root tasks [task_begin, task_end);
        returns (Result, size of the task space).  Ranges that partition the
        space add up to the whole query's result (hashes modulo 2^64)."""
        keep = []
        cq = _as_cquery(q, keep)
        r = _Result()
        T = C.c_uint32()
        self._check(self._L.fsig_match_range(self._h, C.byref(cq), algo, split_len, task_begin, task_end, C.byref(r),
                                             C.byref(T)), "match_range")
        return _result(r), int(T.value)

    def last_stats(self) -> dict:
        st = _Stats()
        self._check(self._L.fsig_last_stats(self._h, C.byref(st)), "last_stats")
        return {k: getattr(st, k) for k, _ in _Stats._fields_}

    # transforms and filter probe
    def build_csr(self, V: int, edges: np.ndarray):
        e = np.ascontiguousarray(edges, np.uint32).reshape(-1)
        E = e.size // 2
        off = np.zeros(V + 1, np.uint32)
        adj = np.zeros(max(2 * E, 1), np.uint32)
        if e.size == 0:
            e = np.zeros(2, np.uint32)
        self._check(self._L.fsig_build_csr(self._h, V, E, _u32p(e), _u32p(off), _u32p(adj)), "build_csr")
        return off, adj[: 2 * E]

    def build_signature(self, labels, offsets, adj, column_oriented: bool = False) -> np.ndarray:
        lab = np.ascontiguousarray(labels, np.int32)
        off = np.ascontiguousarray(offsets, np.uint32)
        a = np.ascontiguousarray(adj, np.uint32)
        if a.size == 0:
            a = np.zeros(1, np.uint32)
        out = np.zeros(16 * len(lab), np.uint32)
        self._check(self._L.fsig_build_signature(self._h, len(lab), _i32p(lab), _u32p(off), _u32p(a),
                                                 1 if column_oriented else 0, _u32p(out)), "build_signature")
        return out

    def build_pcsr(self, labels, offsets, adj, num_labels: int) -> list:
        """The reference's PCSR units, built on the device: a list of
        (keys, list entries, slot table, lists) per unit, as the oracle's pcsr()."""
        lab = np.ascontiguousarray(labels, np.int32)
        off = np.ascontiguousarray(offsets, np.uint32)
        a = np.ascontiguousarray(adj, np.uint32)
        if a.size == 0:
            a = np.zeros(1, np.uint32)
        U = num_labels * (num_labels + 1) // 2
        keys = np.zeros(max(U, 1), np.uint32)
        ne = np.zeros(max(U, 1), np.uint32)
        self._check(self._L.fsig_build_pcsr(self._h, len(lab), num_labels, _i32p(lab), _u32p(off), _u32p(a),
                                            _u32p(keys), _u32p(ne), None, None), "build_pcsr")
        table = np.zeros(max(int(keys[:U].sum()) * 32, 1), np.uint32)
        edges = np.zeros(max(int(ne[:U].sum()), 1), np.uint32)
        self._check(self._L.fsig_build_pcsr(self._h, len(lab), num_labels, _i32p(lab), _u32p(off), _u32p(a),
                                            _u32p(keys), _u32p(ne), _u32p(table), _u32p(edges)), "build_pcsr")
        units, ob, eb = [], 0, 0
        for u in range(U):
            k, m = int(keys[u]), int(ne[u])
            units.append((k, m, table[ob: ob + 32 * k].copy(), edges[eb: eb + m].copy()))
            ob += 32 * k
            eb += m
        return units

    def filter(self, q: Query, algo: int = ALGO_GSI, refine_iters: int = -1, classes: bool = True) -> np.ndarray:
        keep = []
        cq = _as_cquery(q, keep)
        V = self.graph_info()["V"]
        out = np.zeros(q.num_vertices * V, np.uint8)
        self._check(self._L.fsig_filter_classes(self._h, C.byref(cq), algo, refine_iters, 1 if classes else 0,
                                                out.ctypes.data_as(C.POINTER(C.c_uint8))), "filter")
        return out.reshape(q.num_vertices, V)

    # embeddings (EmbeddingWriter)
    def match_embeddings(self, q: Query, algo: int = ALGO_FSIG, buffer_rows: int = 0):
        """(Result, rows[count, n]): every embedding, column u = the data
        vertex of query vertex u, in no particular row order."""
        keep = []
        cq = _as_cquery(q, keep)
        chunks = []

        def sink(_user, rows, num, width):
            chunks.append(np.ctypeslib.as_array(rows, shape=(int(num) * int(width),)).copy().reshape(-1, width))
            return 0

        cb = _SINK(sink)
        r = _Result()
        self._check(self._L.fsig_match_embeddings(self._h, C.byref(cq), algo, buffer_rows, cb, None, C.byref(r)),
                    "match_embeddings")
        n = q.num_vertices
        rows = np.concatenate(chunks) if chunks else np.zeros((0, n), np.uint32)
        return _result(r), rows

    def write_embeddings(self, q: Query, path, algo: int = ALGO_FSIG) -> Result:
        keep = []
        cq = _as_cquery(q, keep)
        r = _Result()
        self._check(self._L.fsig_write_embeddings(self._h, C.byref(cq), algo, str(path).encode(), C.byref(r)),
                    "write_embeddings")
        return _result(r)

    # order-scoring network (ORDER_LEARNED)
    def mpnn_set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        self._check(self._L.fsig_mpnn_set_params(self._h, _f32p(p), p.size), "mpnn_set_params")

    def mpnn_get_params(self) -> np.ndarray:
        p = np.zeros(mpnn_param_count(), np.float32)
        self._check(self._L.fsig_mpnn_get_params(self._h, _f32p(p), p.size), "mpnn_get_params")
        return p

    def mpnn_features(self, qs: Sequence[Query], candidates: Sequence, algo: int = ALGO_FUSED) -> np.ndarray:
        """Device-computed features [total vertices, 8] from candidate counts
        and algo's heuristic order."""
        keep = []
        arr = (_Query * max(len(qs), 1))()
        for i, q in enumerate(qs):
            arr[i] = _as_cquery(q, keep)
        cand = np.ascontiguousarray(np.concatenate([np.asarray(c, np.uint32) for c in candidates])
                                    if len(candidates) else np.zeros(1, np.uint32), np.uint32)
        G = sum(q.num_vertices for q in qs)
        out = np.zeros(max(G, 1) * MPNN_FEATURES, np.float32)
        self._check(self._L.fsig_mpnn_features(self._h, len(qs), arr, algo, _u32p(cand), _f32p(out)),
                    "mpnn_features")
        return out[: G * MPNN_FEATURES].reshape(G, MPNN_FEATURES)

    def mpnn_forward(self, node_offsets, features, neighbours) -> np.ndarray:
        off = np.ascontiguousarray(node_offsets, np.uint32)
        f = np.ascontiguousarray(features, np.float32).reshape(-1)
        nb = np.ascontiguousarray(neighbours, np.uint32)
        out = np.zeros(max(int(off[-1]), 1), np.float32)
        self._check(self._L.fsig_mpnn_forward(self._h, len(off) - 1, _u32p(off), _f32p(f), _u32p(nb), _f32p(out)),
                    "mpnn_forward")
        return out[: int(off[-1])]

    def mpnn_train_step(self, node_offsets, features, neighbours, targets, lr: float = 0.0):
        """One step on the mean squared error: (loss, gradients), Adam update if lr > 0."""
        off = np.ascontiguousarray(node_offsets, np.uint32)
        f = np.ascontiguousarray(features, np.float32).reshape(-1)
        nb = np.ascontiguousarray(neighbours, np.uint32)
        t = np.ascontiguousarray(targets, np.float32)
        loss = np.zeros(1, np.float32)
        grads = np.zeros(mpnn_param_count(), np.float32)
        self._check(self._L.fsig_mpnn_train_step(self._h, len(off) - 1, _u32p(off), _f32p(f), _u32p(nb), _f32p(t),
                                                 float(lr), _f32p(loss), _f32p(grads)), "mpnn_train_step")
        return float(loss[0]), grads


def plan_order(q: Query, algo: int, candidates) -> dict:
    """The reference-exact join order for given candidate counts (host only)."""
    keep = []
    cq = _as_cquery(q, keep)
    n = q.num_vertices
    cand = np.ascontiguousarray(candidates, np.uint32)
    order = np.zeros(n, np.uint32)
    types = np.zeros(n, np.uint32)
    classes = np.zeros(n, np.uint32)
    rc = engine_library().fsig_plan_order(C.byref(cq), algo, _u32p(cand), _u32p(order), _u32p(types),
                                          _u32p(classes))
    if rc:
        raise FsigError(rc, "plan_order failed")
    return dict(order=order.tolist(), types=types.tolist(), classes=classes.tolist())


def refine_classes(q: Query) -> dict:
    """Refinement classes of a query (host only): classes[u] = the smallest
    member of u's class; dominated[u] = a class whose candidate set contains
    u's class's (FSIG_NO_CLASS = 255: none, and for every non-smallest member)."""
    keep = []
    cq = _as_cquery(q, keep)
    n = q.num_vertices
    classes = np.zeros(n, np.uint32)
    dominated = np.zeros(n, np.uint32)
    rc = engine_library().fsig_refine_classes(C.byref(cq), _u32p(classes), _u32p(dominated))
    if rc:
        raise FsigError(rc, "refine_classes failed")
    return dict(classes=classes.tolist(), dominated=dominated.tolist())


NO_CLASS = 0xFF


def select_within_budget(engine: "Engine", candidates: Sequence[Query], want: int, max_work: int,
                         batch: int = 512, algo: int = ALGO_FUSED) -> list:
    """The first `want` candidates, in order, whose enumeration under the
    heuristic order examines at most `max_work` driver entries.  The choice
    depends only on the queries and the data graph, not on scheduling."""
    chosen = []
    for i in range(0, len(candidates), batch):
        part = list(candidates[i:i + batch])
        rs = engine.match_batch(part, algo=algo, max_work=max_work)
        chosen += [q for q, r in zip(part, rs) if r.status == OK]
        if len(chosen) >= want:
            break
    return chosen[:want]


def _filter_noalloc(self, q: Query, algo: int, d_flags: int) -> None:
    """Candidate flags (no refinement) into the caller's device buffer at
    address d_flags (n * V bytes), allocating nothing: for callers that cannot
    allocate device memory at that point (see fsig_filter_noalloc)."""
    keep = []
    cq = _as_cquery(q, keep)
    self._check(self._L.fsig_filter_noalloc(self._h, C.byref(cq), algo, C.c_void_p(d_flags)), "filter_noalloc")


Engine.filter_noalloc = _filter_noalloc


class GPUSubgraphMatcher:
    """Mirror of GPUSubgraphMatcher(Graph* query, Graph* data) with match()
    (match/subgraph_match.h:39-81).  The data graph is loaded into the engine
    on construction; match() returns the Result instead of printing it."""
    algo = ALGO_FUSED

    def __init__(self, query_graph: Query, data_graph: Graph, dev_id: int = 0, engine: Engine | None = None):
        self.query_graph = query_graph
        self.data_graph = data_graph
        self.engine = engine or Engine(dev_id)
        if engine is None:
            self.engine.load_graph(data_graph)

    def match(self) -> Result:
        return self.engine.match(self.query_graph, self.algo)


class MMatch(GPUSubgraphMatcher):
    algo = ALGO_FSIG


class GSI(GPUSubgraphMatcher):
    algo = ALGO_GSI
