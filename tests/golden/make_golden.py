"""Generates the golden fixtures in this directory from the reference itself.

The reference's CPU-side sources (reader, graph, format transformer, GSI and
MMatch host planning) are compiled from the reference tree by oracle/build.py
into oracle/_ref/ref_dump; this script feeds it small seeded graphs and
queries and records what it prints.  Run it in a container that has the
reference tree:

    python tests/golden/make_golden.py

Outputs (committed): *.graph inputs and ref_outputs.json.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import fsig_gb300 as F  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle.build import build_reference  # noqa: E402


def digest(a) -> str:
    return hashlib.sha256(np.asarray(a, np.uint32).tobytes()).hexdigest()


def last_vertex_has_edge(g):
    """The reference reader and CSR transform index rows up to V-1 and read
    past their row vector when the last vertex has no edge (graph.cc:60-66,
    graph_format_transformer.cc:30-31); swap ids so that it has one."""
    V = g.num_vertices
    e = g.edges.copy()
    deg = np.bincount(e.reshape(-1), minlength=V)
    if deg[V - 1] > 0:
        return g
    w = int(np.nonzero(deg)[0].max())
    a, b = e == w, e == V - 1
    e[a], e[b] = V - 1, w
    lab = g.labels.copy()
    lab[[w, V - 1]] = lab[[V - 1, w]]
    return F.Graph(lab, e)


def main() -> None:
    if build_reference() is None:
        raise SystemExit("the reference tree is not available here")
    out = {"graphs": {}, "queries": {}}
    specs = {
        "small_l4": dict(kind="rmat", V=120, E=400, L=4, seed=11, labeled=1),
        "mid_l8": dict(kind="rmat", V=2000, E=9000, L=8, seed=12, labeled=1),
        "cl_zipf16": dict(kind="cl", V=3000, E=12000, L=16, seed=13, labeled=1),
        "unlabeled": dict(kind="rmat", V=800, E=3000, L=3, seed=14, labeled=0),
    }
    for name, s in specs.items():
        lab = F.gen_labels(s["V"], s["L"], "zipf" if s["kind"] == "cl" else "uniform", seed=s["seed"])
        if s["kind"] == "rmat":
            g = F.gen_rmat(s["V"], s["E"], seed=s["seed"], labels=lab)
        else:
            g = F.gen_chung_lu(s["V"], s["E"], 2.1, seed=s["seed"], labels=lab)
        g = last_vertex_has_edge(g)
        path = HERE / f"{name}.graph"
        g.write_tve(path)
        paths = [(name, path)]
        if name == "small_l4":  # the trailing-newline quirk
            qpath = HERE / f"{name}_trailing_newline.graph"
            qpath.write_text(path.read_text() + "\n")
            paths.append((name + "_trailing_newline", qpath))
        for gname, p in paths:
            rec = {"file": p.name, "labeled": s["labeled"]}
            csr = O.parse_dump(O.ref_dump("csr", p, s["labeled"]))
            rec["plain"] = csr["plain"][0]
            rec["labels_sha"] = digest(csr["labels"][0])
            rec["offsets_sha"] = digest(csr["offsets"][0])
            rec["edges_sha"] = digest(csr["edges"][0])
            if gname == "small_l4":
                rec["offsets"] = csr["offsets"][0]
                rec["edges"] = csr["edges"][0]
            for col in (0, 1):
                sig = O.parse_dump(O.ref_dump("sig", p, s["labeled"], col))["sig"][0]
                rec[f"sig{col}_sha"] = digest(sig)
                if gname == "small_l4" and col == 0:
                    rec["sig0"] = sig
            pc = O.parse_dump(O.ref_dump("pcsr", p, s["labeled"]))
            rec["pcsr_units"] = pc["units"][0][0]
            rec["pcsr"] = [[u[1], u[2], digest(o), digest(e)] for u, o, e in zip(pc["unit"], pc["offset"], pc["uedges"])]
            out["graphs"][gname] = rec
    # queries and the reference's join orders for seeded candidate counts
    g = F.read_graph(HERE / "cl_zipf16.graph")
    off, adj = g.csr()
    rng = np.random.default_rng(5)
    qi = 0
    for n in (3, 4, 5, 6, 8, 10, 12):
        for mode in (F.QUERY_INDUCED, F.QUERY_DENSE, F.QUERY_SPARSE):
            try:
                q = F.gen_query(g, n, mode, seed=100 + qi, csr=(off, adj))
            except F.FsigError:
                continue
            name = f"q{qi:02d}_n{n}_m{mode}"
            qpath = HERE / f"{name}.graph"
            q.write_tve(qpath)
            cases = []
            for trial in range(3):
                if trial == 0:
                    cnt = rng.integers(1, 50, n)
                elif trial == 1:
                    cnt = np.full(n, 7)  # all tied
                else:
                    cnt = rng.integers(1, 4, n)  # many ties
                gsi = O.parse_dump(O.ref_dump("gsiorder", qpath, 1, *cnt.tolist()))["order"][0]
                mm = O.parse_dump(O.ref_dump("mmorder", qpath, 1, *cnt.tolist()))
                cases.append({"counts": cnt.tolist(), "gsi_order": gsi, "mm_order": mm["order"][0],
                              "mm_types": mm["types"][0], "mm_classes": mm["classes"][0]})
            out["queries"][name] = {"file": qpath.name, "cases": cases}
            qi += 1
    # The oracle's count and set hash for every golden query on cl_zipf16
    # (the simple graph), so GPU tests need not re-run the slow ones.
    d = O.read_tve(HERE / "cl_zipf16.graph")
    soff, sadj = O.simplify(d["offsets"], d["edges"])
    out["oracle_cl_zipf16"] = {}
    for name, rec in sorted(out["queries"].items()):
        q = F.read_query(HERE / rec["file"])
        c, h, lv = O.match(d["labels"], soff, sadj, q.labels, q.edges)
        out["oracle_cl_zipf16"][name] = {"count": int(c), "hash": int(h), "levels": [int(x) for x in lv]}
    (HERE / "ref_outputs.json").write_text(json.dumps(out, indent=None, separators=(",", ":")))
    print("wrote", len(out["graphs"]), "graphs and", len(out["queries"]), "queries")


if __name__ == "__main__":
    main()
